// batch.cu -- nb_batch_*: many independent systems of uneven N advanced
// together.  Every stage of a step is one launch over all systems (the
// kernels of k_batch.cu walk a device table of SysDesc), and one whole step
// is captured into a CUDA graph that is replayed once per step.  The
// direct-sum kernel's shape (bodies per thread, threads per block, j-tile)
// is chosen by an autotuner that times the candidates on the batch and
// keeps the choice in a JSON cache keyed by the batch's size profile.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/nbgb.h"
#include "nbgb_internal.cuh"
#include "sysmem.cuh"

using namespace nbgb;

struct nb_batch {
    int dev = 0, sm = 0;
    cudaStream_t st = nullptr;
    int nsys = 0;
    std::vector<nb_config> cfg;
    std::vector<SysMem> mem;
    char *arena = nullptr;
    Ctrl *d_ctrl = nullptr;     // one Ctrl per system, contiguous
    Ctrl *h_ctrl = nullptr;     // pinned mirror
    std::vector<SysDesc> h_sys;
    SysDesc *d_sys = nullptr;
    int *d_pref = nullptr;      // prefix tables of nsys + 1 (batch_prefix_device_ints; the last written on the device)
    int *d_work = nullptr;
    float *d_stage = nullptr;   // 4 * max N floats of transfer staging
    BatchTables t{};
    int method = NB_EULER, comp = 0, quad = 0;
    int variant = 5;
    TreeShape shape{};  // launch shapes of the tree stages (autotuned)
    float dt = NAN;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    StepFork fork{};  // the captured step's second branch (direct sums)
    long long launches = 0;
    int launches_per_step = 0;
    nb_status last = NB_OK;
    std::string msg;
};

static nb_status bfail(nb_batch *b, nb_status s, const std::string &m) {
    if (b) {
        b->last = s;
        b->msg = m;
    }
    return s;
}

#define B_CUDA(b, call)                                                                             \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? NB_ERR_OUT_OF_MEMORY : NB_ERR_CUDA,   \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                        \
    } while (0)

static void drop_graph(nb_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

// Work offsets of every system in the batch-wide index spaces, with the
// tree shape's top-level cap and build chunk applied.
static nb_status rebuild_tables(nb_batch *b) {
    const int ns = b->nsys;
    for (int k = 0; k < ns; ++k)
        if (b->h_sys[k].kind == kSysBH)
            sysdesc_set_top(b->h_sys[k], b->mem[k], b->cfg[k].tree_semantics == NB_TREE_REFERENCE,
                            b->shape.top_levels);
    std::vector<int> pref(batch_prefix_ints(ns), 0);
    int totals[kBatchSpaces];
    batch_prefixes(b->h_sys.data(), ns, batch_direct_block_bodies(b->variant), pref.data(), totals,
                   b->shape.build_chunk);
    B_CUDA(b, cudaMemcpyAsync(b->d_sys, b->h_sys.data(), sizeof(SysDesc) * ns, cudaMemcpyHostToDevice, b->st));
    B_CUDA(b, cudaMemcpyAsync(b->d_pref, pref.data(), sizeof(int) * pref.size(), cudaMemcpyHostToDevice, b->st));
    B_CUDA(b, cudaStreamSynchronize(b->st));
    b->t = batch_tables(b->d_sys, ns, b->d_pref, totals, b->d_work);
    drop_graph(b);
    return NB_OK;
}

static std::string tune_key(const nb_batch *b) {
    std::map<int, int> hist;  // log2 size bucket of the direct systems
    for (int k = 0; k < b->nsys; ++k)
        if (b->h_sys[k].kind == kSysDirect) hist[(int)std::floor(std::log2((double)b->mem[k].n))] += 1;
    std::ostringstream os;
    os << "batch_direct/sm" << b->sm;
    for (auto &kv : hist) os << "/" << kv.first << "x" << kv.second;
    return os.str();
}

static std::map<std::string, int> read_cache(const char *path) {
    std::map<std::string, int> m;
    if (!path) return m;
    std::ifstream f(path);
    if (!f) return m;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string s = ss.str();
    size_t i = 0;
    while ((i = s.find('"', i)) != std::string::npos) {
        const size_t j = s.find('"', i + 1);
        if (j == std::string::npos) break;
        const std::string key = s.substr(i + 1, j - i - 1);
        const size_t c = s.find(':', j);
        if (c == std::string::npos) break;
        m[key] = std::atoi(s.c_str() + c + 1);
        i = s.find_first_of(",}", c);
        if (i == std::string::npos) break;
    }
    return m;
}

static void write_cache(const char *path, const std::map<std::string, int> &m) {
    if (!path) return;
    std::ofstream f(path);
    f << "{";
    bool first = true;
    for (auto &kv : m) {
        f << (first ? "" : ",") << "\n  \"" << kv.first << "\": " << kv.second;
        first = false;
    }
    f << "\n}\n";
}

extern "C" {

nb_status nb_batch_create(const nb_config *cfgs, int32_t nsys, nb_batch **out) {
    if (!cfgs || nsys < 1 || !out) return NB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NB_ERR_NO_DEVICE;
    const nb_config &c0 = cfgs[0];
    for (int k = 0; k < nsys; ++k) {
        const nb_config &c = cfgs[k];
        if (c.num_of_bodies < 1 || c.device != c0.device) return NB_ERR_INVALID_ARGUMENT;
        // one kernel instance serves the whole batch: these must agree
        if (c.numerical_method != c0.numerical_method || c.precision != c0.precision ||
            c.multipole != c0.multipole)
            return NB_ERR_UNSUPPORTED;
        if (c.algo_config < NB_BARNES_HUT || c.algo_config > NB_BRUTE_FORCE_LOCAL) return NB_ERR_INVALID_ARGUMENT;
        if (c.algo_config != NB_BARNES_HUT && c.force_law != NB_FORCE_PLUMMER) return NB_ERR_UNSUPPORTED;
        const float eps = c.algo_config == NB_BARNES_HUT ? c.epsilon
                                                         : (c.direct_epsilon >= 0.0f ? c.direct_epsilon : c.epsilon);
        if (!(eps > 0.0f)) return NB_ERR_UNSUPPORTED;
    }
    nb_batch *b = new nb_batch();
    b->nsys = nsys;
    b->dev = c0.device;
    b->cfg.assign(cfgs, cfgs + nsys);
    b->method = c0.numerical_method;
    b->comp = c0.precision == NB_PRECISION_COMPENSATED;
    b->quad = c0.multipole == NB_MULTIPOLE_QUADRUPOLE;
    auto fail_all = [&](nb_status s) {
        nb_batch_destroy(b);
        return s;
    };
    if (cudaSetDevice(b->dev) != cudaSuccess) return fail_all(NB_ERR_CUDA);
    cudaDeviceGetAttribute(&b->sm, cudaDevAttrMultiProcessorCount, b->dev);
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->fork.aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork.fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork.join, cudaEventDisableTiming) != cudaSuccess)
        return fail_all(NB_ERR_CUDA);
    b->mem.resize(nsys);
    size_t total = 0;
    int maxn = 0;
    long long bodies_total = 0, cells_total = 0;
    for (int k = 0; k < nsys; ++k) {
        const nb_config &c = cfgs[k];
        SysMem &m = b->mem[k];
        m.n = c.num_of_bodies;
        m.tree = c.algo_config == NB_BARNES_HUT;
        m.quad = m.tree && b->quad;
        m.cap = m.tree ? (c.cell_capacity > 0 ? c.cell_capacity : sysmem_default_capacity(m.n)) : 0;
        if (m.tree && (long long)m.n + m.cap + 1 >= (1LL << 26) - 1) return fail_all(NB_ERR_UNSUPPORTED);
        total = sysmem_align(total) + sysmem_layout(m, nullptr);
        maxn = std::max(maxn, m.n);
        // the batch-wide index spaces (bodies, cell slots) are 32-bit
        bodies_total += m.n;
        cells_total += m.tree ? (long long)m.cap + 1 : 0;
        if (bodies_total >= (1LL << 31) - 1 || cells_total >= (1LL << 31) - 1) return fail_all(NB_ERR_UNSUPPORTED);
    }
    if (cudaMalloc(&b->arena, total) != cudaSuccess) return fail_all(NB_ERR_OUT_OF_MEMORY);
    size_t off = 0;
    for (int k = 0; k < nsys; ++k) {
        off = sysmem_align(off);
        off += sysmem_layout(b->mem[k], b->arena + off);
    }
    if (cudaMalloc(&b->d_ctrl, sizeof(Ctrl) * nsys) != cudaSuccess ||
        cudaMallocHost(&b->h_ctrl, sizeof(Ctrl) * nsys) != cudaSuccess ||
        cudaMalloc(&b->d_sys, sizeof(SysDesc) * nsys) != cudaSuccess ||
        cudaMalloc(&b->d_pref, sizeof(int) * batch_prefix_device_ints(nsys)) != cudaSuccess ||
        cudaMalloc(&b->d_work, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&b->d_stage, sizeof(float) * 4 * (size_t)maxn) != cudaSuccess)
        return fail_all(NB_ERR_OUT_OF_MEMORY);
    memset(b->h_ctrl, 0, sizeof(Ctrl) * nsys);
    for (int k = 0; k < nsys; ++k) b->h_ctrl[k].budget = -1;  // no step limit
    if (cudaMemcpy(b->d_ctrl, b->h_ctrl, sizeof(Ctrl) * nsys, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail_all(NB_ERR_CUDA);
    b->h_sys.resize(nsys);
    for (int k = 0; k < nsys; ++k) {
        SysMem &m = b->mem[k];
        m.ctrl = b->d_ctrl + k;
        cudaMemset(m.vel, 0, sizeof(float4) * m.n);
        cudaMemset(m.acc, 0, sizeof(float4) * m.n);
        cudaMemset(m.body[0], 0, sizeof(float4) * m.n);
        int *top_counts = nullptr;
        size_t top_bytes = 0;
        sysmem_top_counts(m, &top_counts, &top_bytes);
        if (top_bytes) cudaMemset(top_counts, 0, top_bytes);
        b->h_sys[k] = sysmem_desc(m, cfgs[k], 0.0f);
    }
    if (cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess) return fail_all(NB_ERR_CUDA);
    if (rebuild_tables(b) != NB_OK) return fail_all(NB_ERR_CUDA);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail_all(NB_ERR_CUDA);
    *out = b;
    return NB_OK;
}

nb_status nb_batch_destroy(nb_batch *b) {
    if (!b) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->dev);
    if (b->st) cudaStreamSynchronize(b->st);
    drop_graph(b);
    cudaFree(b->arena);
    cudaFree(b->d_ctrl);
    if (b->h_ctrl) cudaFreeHost(b->h_ctrl);
    cudaFree(b->d_sys);
    cudaFree(b->d_pref);
    cudaFree(b->d_work);
    cudaFree(b->d_stage);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->fork.fork) cudaEventDestroy(b->fork.fork);
    if (b->fork.join) cudaEventDestroy(b->fork.join);
    if (b->fork.aux) cudaStreamDestroy(b->fork.aux);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return NB_OK;
}

static nb_status read_ctrls(nb_batch *b) {
    B_CUDA(b, cudaMemcpyAsync(b->h_ctrl, b->d_ctrl, sizeof(Ctrl) * b->nsys, cudaMemcpyDeviceToHost, b->st));
    B_CUDA(b, cudaStreamSynchronize(b->st));
    return NB_OK;
}

nb_status nb_batch_set_state(nb_batch *b, int32_t k, const float *pos3, const float *vel3, const float *mass) {
    if (!b || k < 0 || k >= b->nsys || !pos3 || !mass) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->dev);
    nb_status r = read_ctrls(b);
    if (r != NB_OK) return r;
    const SysMem &m = b->mem[k];
    const int par = b->h_ctrl[k].parity & 1;
    const size_t n = (size_t)m.n;
    float *sp = b->d_stage, *sm = b->d_stage + 3 * n;
    B_CUDA(b, cudaMemcpyAsync(sp, pos3, 12 * n, cudaMemcpyHostToDevice, b->st));
    B_CUDA(b, cudaMemcpyAsync(sm, mass, 4 * n, cudaMemcpyHostToDevice, b->st));
    B_CUDA(b, launch_pack(sp, sm, nullptr, m.body[par], nullptr, nullptr, m.n, b->st));
    if (vel3) {
        B_CUDA(b, cudaMemcpyAsync(sp, vel3, 12 * n, cudaMemcpyHostToDevice, b->st));
        B_CUDA(b, launch_pack(nullptr, nullptr, sp, nullptr, m.vel, m.acc, m.n, b->st));
    } else {
        B_CUDA(b, launch_pack(nullptr, nullptr, nullptr, nullptr, m.vel, m.acc, m.n, b->st));
    }
    B_CUDA(b, cudaMemsetAsync(&m.ctrl->kdk_primed, 0, sizeof(int), b->st));
    b->launches += 2;
    B_CUDA(b, cudaStreamSynchronize(b->st));
    return NB_OK;
}

nb_status nb_batch_get_state(nb_batch *b, int32_t k, float *pos3, float *vel3, float *acc3, float *mass) {
    if (!b || k < 0 || k >= b->nsys) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->dev);
    nb_status r = read_ctrls(b);
    if (r != NB_OK) return r;
    const SysMem &m = b->mem[k];
    const int par = b->h_ctrl[k].parity & 1;
    const size_t n = (size_t)m.n;
    float *s0 = b->d_stage;
    if (pos3) {
        B_CUDA(b, launch_unpack(m.body[par], nullptr, nullptr, s0, nullptr, nullptr, m.n, b->st));
        B_CUDA(b, cudaMemcpyAsync(pos3, s0, 12 * n, cudaMemcpyDeviceToHost, b->st));
        B_CUDA(b, cudaStreamSynchronize(b->st));
    }
    if (vel3) {
        B_CUDA(b, launch_unpack(nullptr, m.vel, nullptr, nullptr, s0, nullptr, m.n, b->st));
        B_CUDA(b, cudaMemcpyAsync(vel3, s0, 12 * n, cudaMemcpyDeviceToHost, b->st));
        B_CUDA(b, cudaStreamSynchronize(b->st));
    }
    if (acc3) {
        B_CUDA(b, launch_unpack(nullptr, nullptr, m.acc, nullptr, nullptr, s0, m.n, b->st));
        B_CUDA(b, cudaMemcpyAsync(acc3, s0, 12 * n, cudaMemcpyDeviceToHost, b->st));
        B_CUDA(b, cudaStreamSynchronize(b->st));
    }
    if (mass) {
        std::vector<float4> tmp(n);
        B_CUDA(b, cudaMemcpyAsync(tmp.data(), m.body[par], 16 * n, cudaMemcpyDeviceToHost, b->st));
        B_CUDA(b, cudaStreamSynchronize(b->st));
        for (size_t i = 0; i < n; ++i) mass[i] = tmp[i].w;
    }
    b->launches += (pos3 ? 1 : 0) + (vel3 ? 1 : 0) + (acc3 ? 1 : 0);
    return NB_OK;
}

// The kernels read dt from the device table, so a new dt needs no new graph.
static nb_status set_dt(nb_batch *b, float dt) {
    if (dt == b->dt) return NB_OK;
    for (auto &d : b->h_sys) d.p.dt = dt;
    b->dt = dt;
    B_CUDA(b, cudaMemcpyAsync(b->d_sys, b->h_sys.data(), sizeof(SysDesc) * b->nsys, cudaMemcpyHostToDevice, b->st));
    B_CUDA(b, cudaStreamSynchronize(b->st));
    return NB_OK;
}

static nb_status enqueue_steps(nb_batch *b, float dt, int nsteps) {
    nb_status r = set_dt(b, dt);
    if (r != NB_OK) return r;
    B_CUDA(b, launch_batch_clear(b->t, b->st));
    b->launches += 1;
    if (!b->exec) {
        // capture one step; the step flips each system's buffer parity on
        // the device, so the same graph serves every step
        B_CUDA(b, cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
        int nl = 0;
        cudaError_t e = launch_batch_step(b->t, b->method, b->comp, b->quad, b->variant, b->shape, b->sm, b->st,
                                          &b->fork, &nl);
        cudaGraph_t g = nullptr;
        cudaError_t e2 = cudaStreamEndCapture(b->st, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return bfail(b, NB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        b->graph = g;
        B_CUDA(b, cudaGraphInstantiate(&b->exec, b->graph, 0));
        b->launches_per_step = nl;
    }
    for (int i = 0; i < nsteps; ++i) B_CUDA(b, cudaGraphLaunch(b->exec, b->st));
    b->launches += (long long)nsteps * b->launches_per_step;
    return NB_OK;
}

static nb_status check_status(nb_batch *b) {
    nb_status r = read_ctrls(b);
    if (r != NB_OK) return r;
    for (int k = 0; k < b->nsys; ++k) {
        if (b->h_ctrl[k].status) {
            char buf[128];
            snprintf(buf, sizeof(buf), "system %d: device status %d (%s)", k, b->h_ctrl[k].status,
                     nb_status_string((nb_status)b->h_ctrl[k].status));
            return bfail(b, (nb_status)b->h_ctrl[k].status, buf);
        }
    }
    b->last = NB_OK;
    return NB_OK;
}

nb_status nb_batch_step(nb_batch *b, float dt, int32_t nsteps) {
    if (!b || nsteps < 0 || !std::isfinite(dt)) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->dev);
    nb_status r = enqueue_steps(b, dt, nsteps);
    if (r != NB_OK) return r;
    return check_status(b);
}

nb_status nb_batch_time_steps(nb_batch *b, float dt, int32_t nsteps, float *total_ms) {
    if (!b || !total_ms || nsteps < 0) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->dev);
    nb_status r = set_dt(b, dt);
    if (r != NB_OK) return r;
    if (!b->exec) {  // capture outside the timed region
        r = enqueue_steps(b, dt, 0);
        if (r != NB_OK) return r;
    }
    B_CUDA(b, cudaStreamSynchronize(b->st));
    B_CUDA(b, cudaEventRecord(b->e0, b->st));
    r = enqueue_steps(b, dt, nsteps);
    if (r != NB_OK) return r;
    B_CUDA(b, cudaEventRecord(b->e1, b->st));
    r = check_status(b);
    float ms = 0.0f;
    B_CUDA(b, cudaEventElapsedTime(&ms, b->e0, b->e1));
    *total_ms = ms;
    return r;
}

nb_status nb_batch_system_status(nb_batch *b, int32_t k) {
    if (!b || k < 0 || k >= b->nsys) return NB_ERR_INVALID_ARGUMENT;
    return (nb_status)b->h_ctrl[k].status;
}

// Velocities and accelerations of the systems of one kind, saved before
// the autotuner's dt = 0 runs and put back after them (those runs rewrite the
// accelerations, and v + a * 0 can turn a -0 velocity into +0).
struct SavedState {
    float4 *buf = nullptr;
    size_t bodies = 0;
};

static cudaError_t move_state(nb_batch *b, int kind, SavedState &sv, bool save) {
    size_t o = 0;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < b->nsys && e == cudaSuccess; ++k) {
        if (b->h_sys[k].kind != kind) continue;
        const size_t n = (size_t)b->mem[k].n, bytes = sizeof(float4) * n;
        float4 *v = sv.buf + o, *a = sv.buf + sv.bodies + o;
        if (save) {
            e = cudaMemcpyAsync(v, b->mem[k].vel, bytes, cudaMemcpyDeviceToDevice, b->st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(a, b->mem[k].acc, bytes, cudaMemcpyDeviceToDevice, b->st);
        } else {
            e = cudaMemcpyAsync(b->mem[k].vel, v, bytes, cudaMemcpyDeviceToDevice, b->st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(b->mem[k].acc, a, bytes, cudaMemcpyDeviceToDevice, b->st);
        }
        o += n;
    }
    return e;
}

static cudaError_t save_state(nb_batch *b, int kind, SavedState &sv) {
    sv.bodies = 0;
    for (int k = 0; k < b->nsys; ++k)
        if (b->h_sys[k].kind == kind) sv.bodies += (size_t)b->mem[k].n;
    cudaError_t e = cudaMalloc(&sv.buf, sizeof(float4) * 2 * (sv.bodies > 0 ? sv.bodies : 1));
    return e == cudaSuccess ? move_state(b, kind, sv, true) : e;
}

static cudaError_t restore_state(nb_batch *b, int kind, SavedState &sv) {
    cudaError_t e = move_state(b, kind, sv, false);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(sv.buf);
    sv.buf = nullptr;
    return e;
}

// The candidates of the tree stages' launch shapes; the cache keeps the
// chosen shape as one integer of their indices.
static const int kTuneWarps[] = {2, 4, 8};
static const int kTunePct[] = {100, 75, 50};
static const int kTuneChunk[] = {0, 1024, 2048, 4096};  // 0: batch_chunk's rule
static const int kTuneLevels[] = {4, 3, 2, 0};
static_assert(kBatchTopMaxLevels == 4, "kTuneLevels starts at the largest level count");

static int shape_code(const TreeShape &t) {
    auto idx = [](const int *a, int n, int v) {
        for (int i = 0; i < n; ++i)
            if (a[i] == v) return i;
        return 0;
    };
    return idx(kTuneWarps, 3, t.force_warps) + 3 * idx(kTunePct, 3, t.force_grid_pct) +
           9 * idx(kTuneChunk, 4, t.build_chunk) + 36 * idx(kTuneLevels, 4, t.top_levels);
}

static bool shape_from_code(int c, TreeShape &t) {
    if (c < 0 || c >= 3 * 3 * 4 * 4) return false;
    t.force_warps = kTuneWarps[c % 3];
    t.force_grid_pct = kTunePct[(c / 3) % 3];
    t.build_chunk = kTuneChunk[(c / 9) % 4];
    t.top_levels = kTuneLevels[c / 36];
    return true;
}

static std::string tree_tune_key(const nb_batch *b) {
    std::map<int, int> hist;  // log2 size bucket of the tree systems
    for (int k = 0; k < b->nsys; ++k)
        if (b->h_sys[k].kind == kSysBH) hist[(int)std::floor(std::log2((double)b->mem[k].n))] += 1;
    std::ostringstream os;
    os << "batch_tree/sm" << b->sm << "/quad" << b->quad << "/comp" << b->comp;
    for (auto &kv : hist) os << "/" << kv.first << "x" << kv.second;
    return os.str();
}

// Device time of 3 steps (after one warm-up) with the batch's current
// direct variant and tree shape, without the collision update and the flip:
// the tree stages and the direct sums beside them, captured into a CUDA graph
// and replayed as a step is (measured: the same kernels issued one by one on
// the streams schedule differently, and ranked the build chunks the other
// way round).  dt is 0 in every system's parameters.
static cudaError_t time_shapes(nb_batch *b, float *ms) {
    cudaError_t e = launch_batch_clear(b->t, b->st);
    if (e != cudaSuccess) return e;
    if ((e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    int nl = 0;
    const cudaError_t le = launch_batch_step(b->t, b->method, b->comp, b->quad, b->variant, b->shape, b->sm, b->st,
                                             &b->fork, &nl, false);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->st, &g);
    if (le != cudaSuccess) e = le;
    cudaGraphExec_t x = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e == cudaSuccess) e = cudaGraphLaunch(x, b->st);
    if (e == cudaSuccess) e = cudaEventRecord(b->e0, b->st);
    for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) e = cudaGraphLaunch(x, b->st);
    if (e == cudaSuccess) e = cudaEventRecord(b->e1, b->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b->e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, b->e0, b->e1);
    if (x) cudaGraphExecDestroy(x);
    b->launches += 4 * (long long)nl;
    // a trial in which a system failed skipped work: its time means nothing
    if (e == cudaSuccess) e = cudaMemcpy(b->h_ctrl, b->d_ctrl, sizeof(Ctrl) * b->nsys, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        for (int k = 0; k < b->nsys; ++k)
            if (b->h_ctrl[k].status != 0) *ms = INFINITY;
    return e;
}

// One pass of coordinate descent over the four shape parameters (top-level
// cap, build chunk, warps per block, grid fraction), each timed in whole
// steps of this batch; every shape gives the same results, only the time
// differs.
static nb_status tune_tree_shape(nb_batch *b, TreeShape &best) {
    SavedState sv, sv_d;
    cudaError_t e = save_state(b, kSysBH, sv);
    if (e == cudaSuccess) e = save_state(b, kSysDirect, sv_d);
    if (e != cudaSuccess) {
        cudaFree(sv.buf);
        cudaFree(sv_d.buf);
        return bfail(b, NB_ERR_CUDA, std::string("autotune save: ") + cudaGetErrorString(e));
    }
    const float keep_dt = b->dt;
    for (auto &d : b->h_sys) d.p.dt = 0.0f;
    best = b->shape;
    float best_ms = INFINITY;
    nb_status r = NB_OK;
    auto trial = [&](const TreeShape &t) {
        if (r != NB_OK || e != cudaSuccess) return;
        b->shape = t;
        if ((r = rebuild_tables(b)) != NB_OK) return;
        float ms = 0.0f;
        e = time_shapes(b, &ms);
        if (e == cudaSuccess && ms < best_ms) {
            best_ms = ms;
            best = t;
        }
    };
    trial(best);
    for (int v : kTuneLevels) { TreeShape t = best; t.top_levels = v; if (v != best.top_levels) trial(t); }
    for (int v : kTuneChunk) { TreeShape t = best; t.build_chunk = v; if (v != best.build_chunk) trial(t); }
    for (int v : kTuneWarps) { TreeShape t = best; t.force_warps = v; if (v != best.force_warps) trial(t); }
    for (int v : kTunePct) { TreeShape t = best; t.force_grid_pct = v; if (v != best.force_grid_pct) trial(t); }
    for (auto &d : b->h_sys) d.p.dt = keep_dt;
    b->dt = keep_dt;
    b->shape = best;
    cudaError_t er = restore_state(b, kSysBH, sv);
    const cudaError_t er2 = restore_state(b, kSysDirect, sv_d);
    if (er == cudaSuccess) er = er2;
    if (r != NB_OK) return r;
    if (e != cudaSuccess || er != cudaSuccess)
        return bfail(b, NB_ERR_CUDA,
                     std::string("autotune (tree shapes): ") + cudaGetErrorString(e != cudaSuccess ? e : er));
    return rebuild_tables(b);
}

nb_status nb_batch_autotune(nb_batch *b, const char *cache_path, int32_t *chosen) {
    if (!b) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->dev);
    std::map<std::string, int> cache = read_cache(cache_path);
    bool dirty = false;
    // --- the direct-sum kernel shape ---
    const std::string key = tune_key(b);
    int best = b->variant;
    bool have_direct = false, have_tree = false;
    for (auto &d : b->h_sys) {
        have_direct |= d.kind == kSysDirect && d.active;
        have_tree |= d.kind == kSysBH && d.active;
    }
    auto it = cache.find(key);
    if (!have_direct) {
        best = b->variant;
    } else if (it != cache.end() && it->second >= 0 && it->second < batch_direct_variants()) {
        best = it->second;
    } else {
        // time every variant on this batch with dt = 0 in whole steps (the
        // direct sums run beside the tree stages): positions stay as they
        // are, and the velocities and accelerations the runs rewrite are
        // saved before and put back after
        SavedState sv_d, sv_t;
        cudaError_t e = save_state(b, kSysDirect, sv_d);
        if (e == cudaSuccess) e = save_state(b, kSysBH, sv_t);
        if (e != cudaSuccess) {
            cudaFree(sv_d.buf);
            cudaFree(sv_t.buf);
            return bfail(b, NB_ERR_CUDA, std::string("autotune save: ") + cudaGetErrorString(e));
        }
        const float keep = b->dt;
        float best_ms = INFINITY;
        nb_status r = NB_OK;
        for (int v = 0; v < batch_direct_variants() && r == NB_OK && e == cudaSuccess; ++v) {
            b->variant = v;
            for (auto &d : b->h_sys) d.p.dt = 0.0f;
            if ((r = rebuild_tables(b)) != NB_OK) break;
            float ms = 0.0f;
            e = time_shapes(b, &ms);
            if (e == cudaSuccess && ms < best_ms) {
                best_ms = ms;
                best = v;
            }
        }
        for (auto &d : b->h_sys) d.p.dt = keep;
        const cudaError_t er = restore_state(b, kSysDirect, sv_d);
        const cudaError_t er2 = restore_state(b, kSysBH, sv_t);
        if (r != NB_OK) return r;
        if (e != cudaSuccess || er != cudaSuccess || er2 != cudaSuccess)
            return bfail(b, NB_ERR_CUDA,
                         std::string("autotune: ") +
                             cudaGetErrorString(e != cudaSuccess ? e : (er != cudaSuccess ? er : er2)));
        cache[key] = best;
        dirty = true;
    }
    b->variant = best;
    nb_status r = rebuild_tables(b);
    if (r != NB_OK) return r;
    // --- the tree stages' launch shapes ---
    if (have_tree) {
        const std::string tkey = tree_tune_key(b);
        auto ti = cache.find(tkey);
        TreeShape shape;
        if (ti != cache.end() && shape_from_code(ti->second, shape)) {
            b->shape = shape;
            if ((r = rebuild_tables(b)) != NB_OK) return r;
        } else {
            if ((r = tune_tree_shape(b, shape)) != NB_OK) return r;
            cache[tkey] = shape_code(shape);
            dirty = true;
        }
    }
    if (dirty) write_cache(cache_path, cache);
    if (chosen) *chosen = best;
    return NB_OK;
}

nb_status nb_batch_tree_shape(nb_batch *b, int32_t out[4]) {
    if (!b || !out) return NB_ERR_INVALID_ARGUMENT;
    out[0] = b->shape.force_warps;
    out[1] = b->shape.force_grid_pct;
    out[2] = b->shape.build_chunk;
    out[3] = b->shape.top_levels;
    return NB_OK;
}

nb_status nb_batch_info(nb_batch *b, int64_t out[8]) {
    if (!b || !out) return NB_ERR_INVALID_ARGUMENT;
    int64_t bodies = 0, bh = 0, direct = 0;
    for (int k = 0; k < b->nsys; ++k) {
        bodies += b->mem[k].n;
        (b->h_sys[k].kind == kSysBH ? bh : direct) += 1;
    }
    out[0] = b->nsys;
    out[1] = bodies;
    out[2] = bh;
    out[3] = direct;
    out[4] = b->launches_per_step;
    out[5] = b->variant;
    out[6] = b->launches;
    int64_t inter = 0;
    for (int k = 0; k < b->nsys; ++k) inter += (int64_t)b->h_ctrl[k].interactions;
    out[7] = inter;
    return NB_OK;
}

const char *nb_batch_last_error_message(const nb_batch *b) { return b ? b->msg.c_str() : "null handle"; }

}  // extern "C"
