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

// Work offsets of every system in the batch-wide index spaces.
static nb_status rebuild_tables(nb_batch *b) {
    const int ns = b->nsys;
    std::vector<int> pref(batch_prefix_ints(ns), 0);
    int totals[kBatchSpaces];
    batch_prefixes(b->h_sys.data(), ns, batch_direct_block_bodies(b->variant), pref.data(), totals);
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
        cudaError_t e = launch_batch_step(b->t, b->method, b->comp, b->quad, b->variant, b->sm, b->st, &b->fork, &nl);
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

nb_status nb_batch_autotune(nb_batch *b, const char *cache_path, int32_t *chosen) {
    if (!b) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(b->dev);
    const std::string key = tune_key(b);
    std::map<std::string, int> cache = read_cache(cache_path);
    int best = b->variant;
    bool have_direct = false;
    for (auto &d : b->h_sys) have_direct |= d.kind == kSysDirect && d.active;
    auto it = cache.find(key);
    if (!have_direct) {
        best = b->variant;
    } else if (it != cache.end() && it->second >= 0 && it->second < batch_direct_variants()) {
        best = it->second;
    } else {
        // time every variant on this batch with dt = 0: positions and
        // velocities stay as they are, and the accelerations the runs
        // overwrite (the first half-kick of the next leapfrog step reads
        // them) are saved before and put back after
        size_t acc_n = 0;
        for (int k = 0; k < b->nsys; ++k)
            if (b->h_sys[k].kind == kSysDirect) acc_n += (size_t)b->mem[k].n;
        float4 *saved = nullptr;
        B_CUDA(b, cudaMalloc(&saved, sizeof(float4) * acc_n));
        auto move_acc = [&](bool save) {
            size_t o = 0;
            cudaError_t e = cudaSuccess;
            for (int k = 0; k < b->nsys && e == cudaSuccess; ++k) {
                if (b->h_sys[k].kind != kSysDirect) continue;
                const size_t bytes = sizeof(float4) * (size_t)b->mem[k].n;
                e = save ? cudaMemcpyAsync(saved + o, b->mem[k].acc, bytes, cudaMemcpyDeviceToDevice, b->st)
                         : cudaMemcpyAsync(b->mem[k].acc, saved + o, bytes, cudaMemcpyDeviceToDevice, b->st);
                o += (size_t)b->mem[k].n;
            }
            return e;
        };
        cudaError_t e = move_acc(true);
        if (e != cudaSuccess) {
            cudaFree(saved);
            return bfail(b, NB_ERR_CUDA, std::string("autotune save: ") + cudaGetErrorString(e));
        }
        const float keep = b->dt;
        for (auto &d : b->h_sys) d.p.dt = 0.0f;
        float best_ms = INFINITY;
        nb_status r = NB_OK;
        for (int v = 0; v < batch_direct_variants() && r == NB_OK && e == cudaSuccess; ++v) {
            b->variant = v;
            for (auto &d : b->h_sys) d.p.dt = 0.0f;
            if ((r = rebuild_tables(b)) != NB_OK) break;
            e = launch_batch_direct_only(b->t, v, b->st);  // warm-up
            if (e == cudaSuccess) e = cudaEventRecord(b->e0, b->st);
            for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep) e = launch_batch_direct_only(b->t, v, b->st);
            if (e == cudaSuccess) e = cudaEventRecord(b->e1, b->st);
            if (e == cudaSuccess) e = cudaEventSynchronize(b->e1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, b->e0, b->e1);
            b->launches += 4;
            if (e == cudaSuccess && ms < best_ms) {
                best_ms = ms;
                best = v;
            }
        }
        if (r != NB_OK || e != cudaSuccess) {
            for (auto &d : b->h_sys) d.p.dt = keep;
            move_acc(false);
            cudaStreamSynchronize(b->st);
            cudaFree(saved);
            if (r != NB_OK) return r;
            return bfail(b, NB_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
        }
        for (auto &d : b->h_sys) d.p.dt = keep;
        e = move_acc(false);
        if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
        cudaFree(saved);
        if (e != cudaSuccess) return bfail(b, NB_ERR_CUDA, std::string("autotune restore: ") + cudaGetErrorString(e));
        cache[key] = best;
        write_cache(cache_path, cache);
    }
    b->variant = best;
    nb_status r = rebuild_tables(b);
    if (r != NB_OK) return r;
    if (chosen) *chosen = best;
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
