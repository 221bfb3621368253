// api.cu -- the C ABI of include/nbgb.h: handle lifetime, state transfer and
// the per-step pipeline (the GB300 counterpart of CMyApp::InitCL /
// InitParticles / Update, src/MyApp.cpp:110-656).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/nbgb.h"
#include "nbgb_internal.cuh"

using namespace nbgb;

namespace {

enum Stage { kStBboxReset = 0, kStBuild, kStSummarize, kStSort, kStForce, kStCollision, kStDirect, kNumStages };

template <class T>
cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void **)p, sizeof(T) * count);
}

}  // namespace

struct nb_sim {
    nb_config cfg{};
    int dev = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    int n = 0;
    int cap = 0;
    bool tree = false;
    float4 *body[2] = {nullptr, nullptr};
    int cur = 0;
    int last_force_buf = -1;  // body buffer the last force pass read
    float4 *vel = nullptr, *acc = nullptr, *part = nullptr;
    int *parent = nullptr, *child = nullptr, *wchild = nullptr, *count = nullptr, *start = nullptr,
        *arrive = nullptr, *sorted = nullptr;
    float4 *wpm = nullptr, *cell_pm = nullptr;
    float4 *cell_q = nullptr, *wqa = nullptr;
    float2 *wqb = nullptr;
    int *top = nullptr;  // top-level tables: counts, start entries (kTopRegions each), level L-1 entries
    int top_levels = 0;
    bool quad = false;
    Ctrl *ctrl = nullptr;
    Ctrl *h_ctrl = nullptr;       // pinned mirror for status read-back
    float *stage3 = nullptr;      // device staging, 3N floats
    float *stage1 = nullptr;      // device staging, N floats
    bool have_state = false;
    bool kdk_primed = false;
    bool profiling = false;
    std::vector<cudaEvent_t> ev;  // (kNumStages + 1) per timed step
    int timed_steps = 0;
    cudaEvent_t t_begin = nullptr, t_end = nullptr;
    float stage_ms[kNumStages] = {};
    bool stage_ran[kNumStages] = {};
    long long launches = 0;
    nb_status last = NB_OK;
    std::string msg;
};

static nb_status fail(nb_sim *s, nb_status st, const std::string &m) {
    if (s) {
        s->last = st;
        s->msg = m;
    }
    return st;
}

static nb_status cuda_fail(nb_sim *s, cudaError_t e, const char *where) {
    std::string m = std::string(where) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(s, NB_ERR_OUT_OF_MEMORY, m);
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return fail(s, NB_ERR_NO_DEVICE, m);
    return fail(s, NB_ERR_CUDA, m);
}

#define NB_CUDA(s, call)                                   \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_fail(s, e_, #call); \
    } while (0)

static DevSim dev_view(const nb_sim *s) {
    DevSim d{};
    d.n = s->n;
    d.cap = s->cap;
    d.body_cur = s->body[s->cur];
    d.body_next = s->body[s->cur ^ 1];
    d.vel = s->vel;
    d.acc = s->acc;
    d.parent = s->parent;
    d.child = s->child;
    d.wchild = s->wchild;
    d.wpm = s->wpm;
    d.cell_pm = s->cell_pm;
    d.count = s->count;
    d.start = s->start;
    d.arrive = s->arrive;
    d.sorted = s->sorted;
    d.part = s->part;
    d.cell_q = s->cell_q;
    d.wqa = s->wqa;
    d.wqb = s->wqb;
    d.ctrl = s->ctrl;
    return d;
}

static void free_tree(nb_sim *s) {
    cudaFree(s->parent); cudaFree(s->child); cudaFree(s->wchild); cudaFree(s->wpm); cudaFree(s->cell_pm);
    cudaFree(s->count); cudaFree(s->start); cudaFree(s->arrive);
    cudaFree(s->cell_q); cudaFree(s->wqa); cudaFree(s->wqb); cudaFree(s->top);
    s->parent = s->child = s->wchild = s->count = s->start = s->arrive = s->top = nullptr;
    s->wpm = s->cell_pm = s->cell_q = s->wqa = nullptr;
    s->wqb = nullptr;
}

static nb_status alloc_tree(nb_sim *s, int cap) {
    free_tree(s);
    s->cap = cap;
    const size_t cells = (size_t)cap + 1;
    NB_CUDA(s, dalloc(&s->parent, cells));
    NB_CUDA(s, dalloc(&s->child, cells * 8));
    NB_CUDA(s, dalloc(&s->wchild, cells * 8));
    NB_CUDA(s, dalloc(&s->wpm, cells * 8));
    NB_CUDA(s, dalloc(&s->cell_pm, cells));
    NB_CUDA(s, dalloc(&s->count, cells));
    NB_CUDA(s, dalloc(&s->start, cells));
    NB_CUDA(s, dalloc(&s->arrive, cells));
    if (s->quad) {
        NB_CUDA(s, dalloc(&s->cell_q, cells * 2));
        NB_CUDA(s, dalloc(&s->wqa, cells * 8));
        NB_CUDA(s, dalloc(&s->wqb, cells * 8));
    }
    s->top_levels = top_levels_for(s->n);
    if (s->top_levels) {  // the counts start at zero; the build leaves them at zero
        NB_CUDA(s, dalloc(&s->top, (size_t)2 * kTopRegions + kTopRegions / 8));
        NB_CUDA(s, cudaMemset(s->top, 0, sizeof(int) * kTopRegions));
    }
    return NB_OK;
}

static int default_capacity(int n, int sm_count) {
    // SetKernelConfig (src/MyApp.cpp:75-79): max(2N, 1024*CUs) rounded up to 16
    long long c = 2LL * n;
    if (c < 1024LL * sm_count) c = 1024LL * sm_count;
    c = (c + 15) / 16 * 16;
    if (c > (1LL << 30)) c = 1LL << 30;
    return (int)c;
}

extern "C" {

int32_t nb_abi_version(void) { return NBGB_ABI_VERSION; }

const char *nb_status_string(nb_status s) {
    switch (s) {
    case NB_OK: return "ok";
    case NB_ERR_INVALID_ARGUMENT: return "invalid argument";
    case NB_ERR_CUDA: return "CUDA error";
    case NB_ERR_OUT_OF_MEMORY: return "out of device memory";
    case NB_ERR_CELL_OVERFLOW: return "tree cell capacity exceeded";
    case NB_ERR_DEPTH: return "tree deeper than NB_MAX_DEPTH";
    case NB_ERR_SPIN_TIMEOUT: return "bounded device wait gave up";
    case NB_ERR_NONFINITE: return "non-finite body position";
    case NB_ERR_NO_DEVICE: return "no CUDA device";
    case NB_ERR_STATE: return "call out of order";
    case NB_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

void nb_config_default(nb_config *c) {
    if (!c) return;
    memset(c, 0, sizeof(*c));
    c->num_of_bodies = 20000;
    c->gravitational_constant = 6.67e-11f;
    c->starting_speed_mul = 1.0f;
    c->starting_volume_radius = 1.5f;
    c->number_of_massive_objects = 0;
    c->massive_object_mass = 1.0f;
    c->collision = 0;
    c->pos_config = NB_UNIFORM_POS;
    c->vel_config = NB_FUNC_ZERO_VEL;
    c->algo_config = NB_BRUTE_FORCE_GLOBAL;
    c->mass_mean = 0.5f;
    c->mass_deviation = 0.25f;
    c->numerical_method = NB_EULER;
    c->max_octree_depth = 32;
    c->theta = 1.5f;
    c->epsilon = 0.01f;
    c->simulation_speed_mul = 1.0f;
    c->particle_size = 0.05f;
    c->tree_semantics = NB_TREE_GEOMETRIC;
    c->theta_semantics = NB_THETA_STANDARD;
    c->precision = NB_PRECISION_FP32;
    c->force_law = NB_FORCE_PLUMMER;
    c->direct_epsilon = -1.0f;
    c->cell_capacity = 0;
    c->mass_config = NB_MASS_NORMAL_ABS;
    c->pos_sigma[0] = c->pos_sigma[1] = c->pos_sigma[2] = 1.0f;
    c->mass_lognormal_sigma = 0.5f;
    c->seed = 0;
    c->device = 0;
}

nb_status nb_create(const nb_config *cfg, nb_sim **out) {
    if (!cfg || !out) return NB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (cfg->num_of_bodies < 1 || cfg->num_of_bodies > (1 << 28)) return NB_ERR_INVALID_ARGUMENT;
    if (cfg->algo_config < NB_BARNES_HUT || cfg->algo_config > NB_BRUTE_FORCE_LOCAL) return NB_ERR_INVALID_ARGUMENT;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return NB_ERR_NO_DEVICE;
    if (cfg->device < 0 || cfg->device >= ndev) return NB_ERR_INVALID_ARGUMENT;
    nb_sim *s = new nb_sim();
    s->cfg = *cfg;
    s->dev = cfg->device;
    s->n = cfg->num_of_bodies;
    auto cleanup = [&](nb_status st) {
        nb_destroy(s);
        return st;
    };
    if (cudaSetDevice(s->dev) != cudaSuccess) return cleanup(NB_ERR_CUDA);
    cudaDeviceGetAttribute(&s->sm_count, cudaDevAttrMultiProcessorCount, s->dev);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) return cleanup(NB_ERR_CUDA);
    const size_t n = (size_t)s->n;
    bool ok = dalloc(&s->body[0], n) == cudaSuccess && dalloc(&s->body[1], n) == cudaSuccess &&
              dalloc(&s->vel, n) == cudaSuccess && dalloc(&s->acc, n) == cudaSuccess &&
              dalloc(&s->part, n) == cudaSuccess && dalloc(&s->stage3, 3 * n) == cudaSuccess &&
              dalloc(&s->stage1, n) == cudaSuccess && dalloc(&s->ctrl, 1) == cudaSuccess;
    if (!ok) return cleanup(NB_ERR_OUT_OF_MEMORY);
    if (cudaMallocHost((void **)&s->h_ctrl, sizeof(Ctrl)) != cudaSuccess) return cleanup(NB_ERR_OUT_OF_MEMORY);
    cudaMemset(s->ctrl, 0, sizeof(Ctrl));
    cudaMemset(s->vel, 0, sizeof(float4) * n);
    cudaMemset(s->acc, 0, sizeof(float4) * n);
    s->tree = cfg->algo_config == NB_BARNES_HUT;
    s->quad = cfg->multipole == NB_MULTIPOLE_QUADRUPOLE;
    if (s->tree) {
        int cap = cfg->cell_capacity > 0 ? cfg->cell_capacity : default_capacity(s->n, s->sm_count);
        // the force walk packs (level << 26) | node into one word
        if ((long long)s->n + cap + 1 >= (1LL << 26) - 1) return cleanup(NB_ERR_UNSUPPORTED);
        if (alloc_tree(s, cap) != NB_OK) return cleanup(NB_ERR_OUT_OF_MEMORY);
        if (dalloc(&s->sorted, n) != cudaSuccess) return cleanup(NB_ERR_OUT_OF_MEMORY);
    }
    if (cudaEventCreate(&s->t_begin) != cudaSuccess || cudaEventCreate(&s->t_end) != cudaSuccess)
        return cleanup(NB_ERR_CUDA);
    if (cudaDeviceSynchronize() != cudaSuccess) return cleanup(NB_ERR_CUDA);
    *out = s;
    return NB_OK;
}

nb_status nb_destroy(nb_sim *s) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->dev);
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->body[0]); cudaFree(s->body[1]); cudaFree(s->vel); cudaFree(s->acc); cudaFree(s->part);
    cudaFree(s->stage3); cudaFree(s->stage1); cudaFree(s->ctrl); cudaFree(s->sorted);
    free_tree(s);
    if (s->h_ctrl) cudaFreeHost(s->h_ctrl);
    for (auto &e : s->ev)
        if (e) cudaEventDestroy(e);
    if (s->t_begin) cudaEventDestroy(s->t_begin);
    if (s->t_end) cudaEventDestroy(s->t_end);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return NB_OK;
}

nb_status nb_get_config(const nb_sim *s, nb_config *out) {
    if (!s || !out) return NB_ERR_INVALID_ARGUMENT;
    *out = s->cfg;
    return NB_OK;
}

// The device address of a host array the device can read and write
// directly (page-locked: nb_host_alloc, cudaMallocHost, cudaHostRegister),
// else null.  Such arrays are packed and unpacked by the kernels in place,
// without a staging copy: one pass over the host link at full width.
static void *host_device_view(const void *p, int dev) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    // page-locked for this handle's device (allocated or registered while it
    // was current); other arrays take the staging copy
    return a.type == cudaMemoryTypeHost && a.device == dev ? a.devicePointer : nullptr;
}

nb_status nb_set_state(nb_sim *s, const float *pos3, const float *vel3, const float *mass, int32_t n) {
    if (!s || !pos3 || !mass) return fail(s, NB_ERR_INVALID_ARGUMENT, "nb_set_state: pos3 and mass are required");
    if (n != s->n) return fail(s, NB_ERR_INVALID_ARGUMENT, "nb_set_state: n differs from num_of_bodies");
    cudaSetDevice(s->dev);
    const size_t nn = (size_t)n;
    {
        const float *dp = static_cast<const float *>(host_device_view(pos3, s->dev));
        const float *dm = static_cast<const float *>(host_device_view(mass, s->dev));
        const float *dv = static_cast<const float *>(host_device_view(vel3, s->dev));
        if (dp && dm && (!vel3 || dv)) {  // page-locked: the kernel reads the host arrays
            NB_CUDA(s, launch_pack(dp, dm, dv, s->body[s->cur], s->vel, s->acc, n, s->stream));
            s->launches += 1;
            NB_CUDA(s, cudaStreamSynchronize(s->stream));
            s->have_state = true;
            s->kdk_primed = false;
            s->last_force_buf = -1;
            return NB_OK;
        }
    }
    NB_CUDA(s, cudaMemcpyAsync(s->stage3, pos3, 12 * nn, cudaMemcpyHostToDevice, s->stream));
    NB_CUDA(s, cudaMemcpyAsync(s->stage1, mass, 4 * nn, cudaMemcpyHostToDevice, s->stream));
    float *dvel = nullptr;
    if (vel3) {
        // velocities go through the partial-sum buffer as 3N floats
        dvel = reinterpret_cast<float *>(s->part);
        NB_CUDA(s, cudaMemcpyAsync(dvel, vel3, 12 * nn, cudaMemcpyHostToDevice, s->stream));
    }
    NB_CUDA(s, launch_pack(s->stage3, s->stage1, dvel, s->body[s->cur], s->vel, s->acc, n, s->stream));
    s->launches += 1;
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    s->have_state = true;
    s->kdk_primed = false;
    s->last_force_buf = -1;
    return NB_OK;
}

nb_status nb_set_state_device(nb_sim *s, const float *d_pos3, const float *d_vel3, const float *d_mass) {
    if (!s || !d_pos3 || !d_mass) return fail(s, NB_ERR_INVALID_ARGUMENT, "nb_set_state_device: null array");
    cudaSetDevice(s->dev);
    NB_CUDA(s, launch_pack(d_pos3, d_mass, d_vel3, s->body[s->cur], s->vel, s->acc, s->n, s->stream));
    s->launches += 1;
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    s->have_state = true;
    s->kdk_primed = false;
    s->last_force_buf = -1;
    return NB_OK;
}

nb_status nb_get_state(nb_sim *s, float *pos3, float *vel3, float *acc3, float *mass) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    if (!s->have_state) return fail(s, NB_ERR_STATE, "nb_get_state before nb_set_state");
    cudaSetDevice(s->dev);
    const size_t nn = (size_t)s->n;
    float *dv = reinterpret_cast<float *>(s->part);
    float *da = nullptr;  // acceleration staged behind the positions when asked
    std::vector<float> tmp;
    if ((pos3 || vel3) && !acc3 && !mass) {
        float *hp = static_cast<float *>(host_device_view(pos3, s->dev));
        float *hv = static_cast<float *>(host_device_view(vel3, s->dev));
        if ((!pos3 || hp) && (!vel3 || hv)) {  // page-locked: the kernel writes the host arrays
            NB_CUDA(s, launch_unpack(s->body[s->cur], s->vel, s->acc, hp, hv, nullptr, s->n, s->stream));
            s->launches += 1;
            NB_CUDA(s, cudaStreamSynchronize(s->stream));
            return NB_OK;
        }
    }
    if (pos3 || vel3) {
        NB_CUDA(s, launch_unpack(s->body[s->cur], s->vel, s->acc, pos3 ? s->stage3 : nullptr, vel3 ? dv : nullptr,
                                 nullptr, s->n, s->stream));
        s->launches += 1;
        if (pos3) NB_CUDA(s, cudaMemcpyAsync(pos3, s->stage3, 12 * nn, cudaMemcpyDeviceToHost, s->stream));
        if (vel3) NB_CUDA(s, cudaMemcpyAsync(vel3, dv, 12 * nn, cudaMemcpyDeviceToHost, s->stream));
    }
    if (acc3 || mass) {
        NB_CUDA(s, cudaStreamSynchronize(s->stream));
        if (acc3) {
            da = s->stage3;
            NB_CUDA(s, launch_unpack(nullptr, nullptr, s->acc, nullptr, nullptr, da, s->n, s->stream));
            s->launches += 1;
            NB_CUDA(s, cudaMemcpyAsync(acc3, da, 12 * nn, cudaMemcpyDeviceToHost, s->stream));
        }
        if (mass) {
            tmp.resize(4 * nn);
            NB_CUDA(s, cudaMemcpyAsync(tmp.data(), s->body[s->cur], 16 * nn, cudaMemcpyDeviceToHost, s->stream));
        }
    }
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    if (mass)
        for (size_t i = 0; i < nn; ++i) mass[i] = tmp[4 * i + 3];
    return NB_OK;
}

nb_status nb_get_state_device(nb_sim *s, float *d_pos3, float *d_vel3) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->dev);
    NB_CUDA(s, launch_unpack(s->body[s->cur], s->vel, s->acc, d_pos3, d_vel3, nullptr, s->n, s->stream));
    s->launches += 1;
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    return NB_OK;
}

nb_status nb_init_bodies(nb_sim *s) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    std::vector<float> pos(3 * (size_t)s->n), vel(3 * (size_t)s->n), mass(s->n);
    nb_status st = nb_generate_ic(&s->cfg, pos.data(), vel.data(), mass.data());
    if (st != NB_OK) return fail(s, st, "nb_generate_ic failed");
    return nb_set_state(s, pos.data(), vel.data(), mass.data(), s->n);
}

nb_status nb_set_profiling(nb_sim *s, int32_t on) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    s->profiling = on != 0;
    return NB_OK;
}

nb_status nb_get_timings(nb_sim *s, float *ms, int32_t nms) {
    if (!s || !ms) return NB_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < nms && i < kNumStages; ++i) ms[i] = s->stage_ran[i] ? s->stage_ms[i] : 0.0f;
    return NB_OK;
}

int64_t nb_kernel_launches(const nb_sim *s) { return s ? s->launches : -1; }

}  // extern "C"

constexpr int kMaxTimedSteps = 256;

// One step of the configured algorithm on the handle's stream.  Records the
// stage events of timed step `timed` (< 0: untimed).  Returns NB_OK or a
// CUDA launch error.
static nb_status enqueue_step(nb_sim *s, float dt, int timed) {
    const nb_config &c = s->cfg;
    StepParams p{};
    p.dt = dt;
    p.G = c.gravitational_constant;
    p.theta = c.theta;
    p.method = c.numerical_method;
    p.kdk_primed = s->kdk_primed ? 1 : 0;
    p.tree_ref = c.tree_semantics == NB_TREE_REFERENCE;
    p.crit_ref = c.theta_semantics == NB_THETA_REFERENCE;
    p.quadrupole = s->quad ? 1 : 0;
    DevSim d = dev_view(s);
    cudaStream_t st = s->stream;
    // profiling: CUDA events between the stages of the timed steps, and an
    // NVTX range per stage for a timeline tool (free when none is attached)
    static const char *const kStageName[] = {"nbgb bbox", "nbgb build", "nbgb summarize", "nbgb sort",
                                             "nbgb force", "nbgb collision", "nbgb end"};
    bool open_range = false;
    auto mark = [&](int k) {
        if (timed >= 0) cudaEventRecord(s->ev[(size_t)timed * (kNumStages + 1) + k], st);
        if (s->profiling) {
            if (open_range) nvtxRangePop();
            open_range = k < 6;
            if (open_range) nvtxRangePushA(s->tree ? kStageName[k] : "nbgb direct");
        }
    };
    for (int k = 0; k < kNumStages; ++k) s->stage_ran[k] = false;
    if (s->tree) {
        p.eps = c.epsilon;
        mark(0);
        NB_CUDA(s, launch_reset(d, st));
        NB_CUDA(s, launch_bbox(d, s->sm_count, st));
        mark(1);
        const TopTables top{s->top, s->top ? s->top + kTopRegions : nullptr, s->top ? s->top_levels : 0,
                            s->top ? s->top + 2 * kTopRegions : nullptr};
        int build_launches = 1;
        NB_CUDA(s, launch_build(d, top, p.tree_ref, s->sm_count, st, &build_launches));
        mark(2);
        NB_CUDA(s, launch_summarize(d, p.quadrupole, s->sm_count, st));
        mark(3);
        NB_CUDA(s, launch_sort(d, s->sm_count, st));
        mark(4);
        NB_CUDA(s, launch_force(d, p, c.precision == NB_PRECISION_COMPENSATED, s->sm_count, st));
        mark(5);
        s->launches += 5 + build_launches;
        for (int k = kStBboxReset; k <= kStForce; ++k) s->stage_ran[k] = true;
    } else {
        const bool quirk = c.force_law == NB_FORCE_REFERENCE_QUIRK;
        const bool tiled = c.algo_config == NB_BRUTE_FORCE_LOCAL;
        if (quirk) p.eps = tiled ? 0.1f : 0.01f;  // brute_force_update.cl:56,116
        else p.eps = c.direct_epsilon >= 0.0f ? c.direct_epsilon : c.epsilon;
        mark(0);
        for (int k = 1; k <= 5; ++k) mark(k);
        NB_CUDA(s, launch_direct(d, p, tiled ? 1 : 0, quirk ? 1 : 0, s->sm_count, st));
        s->launches += 2;
        s->stage_ran[kStDirect] = true;
    }
    if (c.collision) {
        NB_CUDA(s, launch_collision(d, s->tree ? 1 : 0, s->sm_count, st));
        s->launches += 1;
        s->stage_ran[kStCollision] = true;
    }
    mark(6);
    if (!s->tree) {
        // direct path: stage 6 spans the direct kernel (events 5 -> 6 minus collision)
    }
    s->last_force_buf = s->cur;
    s->cur ^= 1;
    if (c.numerical_method == NB_KDK_LEAPFROG) s->kdk_primed = true;
    return NB_OK;
}

static nb_status finish_steps(nb_sim *s) {
    NB_CUDA(s, cudaMemcpyAsync(s->h_ctrl, s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s->stream));
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    if (s->timed_steps > 0) {
        // average per step over the timed steps of the call
        for (int k = 0; k < kNumStages; ++k) s->stage_ms[k] = 0.0f;
        for (int t = 0; t < s->timed_steps; ++t) {
            cudaEvent_t *e = &s->ev[(size_t)t * (kNumStages + 1)];
            float ms = 0.0f;
            if (s->tree) {
                for (int k = 0; k < 5; ++k) {
                    cudaEventElapsedTime(&ms, e[k], e[k + 1]);
                    s->stage_ms[k] += ms;
                }
                if (s->cfg.collision) {
                    cudaEventElapsedTime(&ms, e[5], e[6]);
                    s->stage_ms[kStCollision] += ms;
                }
            } else {
                cudaEventElapsedTime(&ms, e[0], e[6]);
                s->stage_ms[kStDirect] += ms;
            }
        }
        for (int k = 0; k < kNumStages; ++k) s->stage_ms[k] /= (float)s->timed_steps;
    }
    const int st = s->h_ctrl->status;
    if (st != 0) {
        char buf[160];
        snprintf(buf, sizeof(buf), "device status %d (%s), info %d", st, nb_status_string((nb_status)st),
                 s->h_ctrl->status_info);
        return fail(s, (nb_status)st, buf);
    }
    s->last = NB_OK;
    return NB_OK;
}

extern "C" {

nb_status nb_step_async(nb_sim *s, float dt, int32_t nsteps) {
    if (!s || nsteps < 0 || !std::isfinite(dt)) return fail(s, NB_ERR_INVALID_ARGUMENT, "nb_step: bad argument");
    if (!s->have_state) return fail(s, NB_ERR_STATE, "nb_step before nb_set_state");
    cudaSetDevice(s->dev);
    // the status word and the work counters are cleared once per call, so a
    // failed step stays visible to the later ones
    NB_CUDA(s, cudaMemsetAsync(&s->ctrl->status, 0, sizeof(Ctrl) - offsetof(Ctrl, status), s->stream));
    s->timed_steps = 0;
    if (s->profiling) {
        const int want = std::min(nsteps, kMaxTimedSteps);
        while ((int)s->ev.size() < want * (kNumStages + 1)) {
            cudaEvent_t e;
            NB_CUDA(s, cudaEventCreate(&e));
            s->ev.push_back(e);
        }
        s->timed_steps = want;
    }
    for (int i = 0; i < nsteps; ++i) {
        nb_status r = enqueue_step(s, dt, i < s->timed_steps ? i : -1);
        if (r != NB_OK) return r;
    }
    return NB_OK;
}

nb_status nb_synchronize(nb_sim *s) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->dev);
    return finish_steps(s);
}

nb_status nb_step(nb_sim *s, float dt, int32_t nsteps) {
    nb_status r = nb_step_async(s, dt, nsteps);
    if (r != NB_OK) return r;
    return finish_steps(s);
}

nb_status nb_time_steps(nb_sim *s, float dt, int32_t nsteps, float *total_ms) {
    if (!s || !total_ms) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->dev);
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    NB_CUDA(s, cudaEventRecord(s->t_begin, s->stream));
    nb_status r = nb_step_async(s, dt, nsteps);
    if (r != NB_OK) return r;
    NB_CUDA(s, cudaEventRecord(s->t_end, s->stream));
    r = finish_steps(s);
    float ms = 0.0f;
    NB_CUDA(s, cudaEventElapsedTime(&ms, s->t_begin, s->t_end));
    *total_ms = ms;
    return r;
}

nb_status nb_debug_set_spin_cap(nb_sim *s, int32_t cap) {
    if (!s || cap < 0) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->dev);
    NB_CUDA(s, cudaMemcpyAsync(&s->ctrl->spin_cap, &cap, sizeof(int), cudaMemcpyHostToDevice, s->stream));
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    return NB_OK;
}

nb_status nb_get_work_counters(nb_sim *s, uint64_t out[3]) {
    if (!s || !out) return NB_ERR_INVALID_ARGUMENT;
    out[0] = s->h_ctrl->interactions;
    out[1] = s->h_ctrl->opened;
    out[2] = s->h_ctrl->cell_interactions;
    return NB_OK;
}

nb_status nb_update(nb_sim *s, float frame_dt) {
    if (!s) return NB_ERR_INVALID_ARGUMENT;
    float dt = frame_dt;
    if (dt > 0.005f) dt = 0.005f;
    if (dt < 0.0001f) dt = 0.0001f;
    dt *= s->cfg.simulation_speed_mul;
    return nb_step(s, dt, 1);
}

nb_status nb_copy_vertices(nb_sim *s, float *dst4, int32_t dst_is_device) {
    if (!s || !dst4) return NB_ERR_INVALID_ARGUMENT;
    if (!s->have_state) return fail(s, NB_ERR_STATE, "nb_copy_vertices before nb_set_state");
    cudaSetDevice(s->dev);
    const size_t nn = (size_t)s->n;
    const bool aligned = ((uintptr_t)dst4 & 15) == 0;  // float4 stores
    if (dst_is_device) {
        if (!aligned) return fail(s, NB_ERR_INVALID_ARGUMENT, "nb_copy_vertices: a device dst must be 16-byte aligned");
        NB_CUDA(s, launch_copy_vertices(s->body[s->cur], s->n, reinterpret_cast<float4 *>(dst4), s->stream));
        s->launches += 1;
    } else if (float *hd = aligned ? static_cast<float *>(host_device_view(dst4, s->dev)) : nullptr) {  // page-locked host
        NB_CUDA(s, launch_copy_vertices(s->body[s->cur], s->n, reinterpret_cast<float4 *>(hd), s->stream));
        s->launches += 1;
    } else {
        NB_CUDA(s, launch_copy_vertices(s->body[s->cur], s->n, s->part, s->stream));
        s->launches += 1;
        NB_CUDA(s, cudaMemcpyAsync(dst4, s->part, 16 * nn, cudaMemcpyDeviceToHost, s->stream));
    }
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    return NB_OK;
}

nb_status nb_get_device_view(nb_sim *s, nb_device_view *out) {
    if (!s || !out) return NB_ERR_INVALID_ARGUMENT;
    out->body_pm = s->body[s->cur];
    out->vel = s->vel;
    out->acc = s->acc;
    out->stream = (void *)s->stream;
    out->n = s->n;
    return NB_OK;
}

nb_status nb_get_stage_debug(nb_sim *s, int32_t which, void *dst, size_t bytes, size_t *written) {
    if (!s || !dst) return NB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->dev);
    const size_t n = (size_t)s->n, total = n + (size_t)s->cap + 1;
    size_t need = 0;
    switch (which) {
    case NB_DEBUG_BBOX: need = 6 * 4; break;
    case NB_DEBUG_CHILDREN: need = total * 8 * 4; break;
    case NB_DEBUG_NODE_POS: need = total * 3 * 4; break;
    case NB_DEBUG_NODE_MASS: need = total * 4; break;
    case NB_DEBUG_BODY_COUNT: need = total * 4; break;
    case NB_DEBUG_SORTED: need = n * 4; break;
    case NB_DEBUG_TREE_INFO: need = 4 * 4; break;
    case NB_DEBUG_DQ: need = 64 * 4; break;
    case NB_DEBUG_NODE_QUAD: need = total * 6 * 4; break;
    default: return fail(s, NB_ERR_INVALID_ARGUMENT, "nb_get_stage_debug: unknown item");
    }
    if (written) *written = need;
    if (bytes < need) return fail(s, NB_ERR_INVALID_ARGUMENT, "nb_get_stage_debug: buffer too small");
    if (!s->tree && which != NB_DEBUG_BBOX)
        return fail(s, NB_ERR_STATE, "nb_get_stage_debug: no tree for a direct-sum configuration");
    NB_CUDA(s, cudaMemcpyAsync(s->h_ctrl, s->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, s->stream));
    NB_CUDA(s, cudaStreamSynchronize(s->stream));
    float box[6];
    for (int k = 0; k < 6; ++k) {
        unsigned key = s->h_ctrl->bbox_key[k];
        unsigned b = (key & 0x80000000u) ? (key & 0x7fffffffu) : ~key;
        memcpy(&box[k], &b, 4);
    }
    if (which == NB_DEBUG_BBOX) {
        memcpy(dst, box, sizeof(box));
        return NB_OK;
    }
    if (which == NB_DEBUG_TREE_INFO) {
        int info[4] = {s->n, s->cap, s->h_ctrl->bottom, s->h_ctrl->max_depth};
        memcpy(dst, info, sizeof(info));
        return NB_OK;
    }
    if (which == NB_DEBUG_DQ) {
        // the same recurrence as the force kernel's thresholds, on the host
        float *dq = (float *)dst;
        const nb_config &c = s->cfg;
        const float radius = 0.5f * std::fmax(std::fmax(box[3] - box[0], box[4] - box[1]), box[5] - box[2]);
        volatile float rr = radius * radius;
        float d0;
        if (c.theta_semantics == NB_THETA_REFERENCE) d0 = c.theta > 0 ? rr / c.theta : (float)rr;
        else {
            volatile float t2 = c.theta * c.theta;
            volatile float itol = 1.0f / t2;
            d0 = rr * itol;
        }
        volatile float add = c.theta_semantics == NB_THETA_REFERENCE ? c.epsilon : c.epsilon * c.epsilon;
        volatile float base = d0;
        for (int i = 0; i < 64; ++i) {
            dq[i] = base + add;
            base = 0.25f * base;
        }
        return NB_OK;
    }
    if (which == NB_DEBUG_SORTED) {
        NB_CUDA(s, cudaMemcpy(dst, s->sorted, need, cudaMemcpyDeviceToHost));
        return NB_OK;
    }
    // tree arrays: export at the positions of the last force pass
    DevSim d = dev_view(s);
    if (s->last_force_buf >= 0) d.body_cur = s->body[s->last_force_buf];
    void *tmp = nullptr;
    NB_CUDA(s, cudaMalloc(&tmp, need));
    cudaError_t e = launch_export_tree(d, which == NB_DEBUG_CHILDREN ? (int *)tmp : nullptr,
                                       which == NB_DEBUG_NODE_POS ? (float *)tmp : nullptr,
                                       which == NB_DEBUG_NODE_MASS ? (float *)tmp : nullptr,
                                       which == NB_DEBUG_BODY_COUNT ? (int *)tmp : nullptr,
                                       which == NB_DEBUG_NODE_QUAD ? (float *)tmp : nullptr, s->stream);
    s->launches += 1;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(dst, tmp, need, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(s, e, "nb_get_stage_debug");
    return NB_OK;
}

nb_status nb_force_error_probe(nb_sim *s, const int32_t *sample, int32_t ns, double *max_rel, double *rms_rel,
                               double *rel_err) {
    if (!s || !sample || ns <= 0) return NB_ERR_INVALID_ARGUMENT;
    if (s->last_force_buf < 0) return fail(s, NB_ERR_STATE, "nb_force_error_probe: no force pass yet");
    cudaSetDevice(s->dev);
    for (int i = 0; i < ns; ++i)
        if (sample[i] < 0 || sample[i] >= s->n) return fail(s, NB_ERR_INVALID_ARGUMENT, "sample index out of range");
    int *d_sample = nullptr;
    double *d_out = nullptr;
    NB_CUDA(s, cudaMalloc(&d_sample, sizeof(int) * ns));
    cudaError_t e = cudaMalloc(&d_out, sizeof(double) * 3 * ns);
    if (e != cudaSuccess) {
        cudaFree(d_sample);
        return cuda_fail(s, e, "nb_force_error_probe");
    }
    std::vector<double> a64(3 * (size_t)ns);
    std::vector<float4> a32(s->n);
    const nb_config &c = s->cfg;
    double eps = c.epsilon;
    if (!s->tree) eps = c.direct_epsilon >= 0.0f ? c.direct_epsilon : c.epsilon;
    e = cudaMemcpyAsync(d_sample, sample, sizeof(int) * ns, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess)
        e = launch_force_probe(s->body[s->last_force_buf], s->n, d_sample, ns, eps, c.gravitational_constant, d_out,
                               s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(a64.data(), d_out, sizeof(double) * 3 * ns, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(a32.data(), s->acc, sizeof(float4) * s->n, cudaMemcpyDeviceToHost);
    cudaFree(d_sample);
    cudaFree(d_out);
    s->launches += 1;
    if (e != cudaSuccess) return cuda_fail(s, e, "nb_force_error_probe");
    double mx = 0.0, sq = 0.0;
    for (int k = 0; k < ns; ++k) {
        const float4 a = a32[sample[k]];
        const double ex = a.x - a64[3 * k], ey = a.y - a64[3 * k + 1], ez = a.z - a64[3 * k + 2];
        const double nrm = std::sqrt(a64[3 * k] * a64[3 * k] + a64[3 * k + 1] * a64[3 * k + 1] +
                                     a64[3 * k + 2] * a64[3 * k + 2]);
        const double r = nrm > 0 ? std::sqrt(ex * ex + ey * ey + ez * ez) / nrm : 0.0;
        if (rel_err) rel_err[k] = r;
        mx = std::max(mx, r);
        sq += r * r;
    }
    if (max_rel) *max_rel = mx;
    if (rms_rel) *rms_rel = std::sqrt(sq / ns);
    return NB_OK;
}

nb_status nb_diagnostics(nb_sim *s, int32_t with_potential, double out[9]) {
    if (!s || !out) return NB_ERR_INVALID_ARGUMENT;
    if (!s->have_state) return fail(s, NB_ERR_STATE, "nb_diagnostics before nb_set_state");
    cudaSetDevice(s->dev);
    double *d_out = nullptr;
    NB_CUDA(s, cudaMalloc(&d_out, 9 * sizeof(double)));
    const double eps = s->tree ? s->cfg.epsilon
                               : (s->cfg.direct_epsilon >= 0.0f ? s->cfg.direct_epsilon : s->cfg.epsilon);
    cudaError_t e = launch_diagnostics(s->body[s->cur], s->vel, s->n, with_potential, eps,
                                       s->cfg.gravitational_constant, d_out, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(out, d_out, 9 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    s->launches += with_potential ? 2 : 1;
    if (e != cudaSuccess) return cuda_fail(s, e, "nb_diagnostics");
    return NB_OK;
}

nb_status nb_last_error(const nb_sim *s) { return s ? s->last : NB_ERR_INVALID_ARGUMENT; }
const char *nb_last_error_message(const nb_sim *s) { return s ? s->msg.c_str() : "null handle"; }

void *nb_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
    return p;
}
void nb_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
