// k_force.cu -- the single-system Barnes-Hut force kernel: warps take
// groups of 32 sorted bodies from a global counter and walk the tree
// (force_group, force_device.cuh), then integrate.
#include "force_device.cuh"

namespace nbgb {

template <int kMethod, bool kComp, bool kEpsZero, bool kQuad>
__global__ void __launch_bounds__(kForceThreads) k_force(DevSim s, StepParams p) {
    __shared__ float s_dq[kMaxDepth];
    __shared__ int s_stack[kForceWarps][kStack];
    __shared__ float4 s_bpm[kForceWarps][8 * kBatch];
    __shared__ float4 s_cpm[kForceWarps][8 * kBatch];
    __shared__ float4 s_cmeta[kForceWarps][8 * kBatch];
    __shared__ float4 s_cqa[kForceWarps][kQuad ? 8 * kBatch : 1];
    __shared__ int s_skip;
    Ctrl *ctrl = s.ctrl;
    const int n = s.n;
    if (threadIdx.x == 0) {
        int skip = read_status(ctrl);
        if (!skip && ctrl->max_depth >= kMaxDepth) {
            set_status(ctrl, kStDepth, ctrl->max_depth);
            skip = 1;
        }
        s_skip = skip;
        float box[6];
        load_box(ctrl, box);
        make_thresholds(box, p.theta, p.eps, p.crit_ref, s_dq);
    }
    __syncthreads();
    if (s_skip) {  // a failed step keeps the step-start state
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            s.body_next[i] = s.body_cur[i];
        return;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const WarpStage ws{s_stack[w], s_bpm[w], s_cpm[w], s_cmeta[w], s_cqa[w]};
    const int ngroups = (n + 31) >> 5;
    while (true) {
        int g = 0;
        if (lane == 0) g = atomicAdd(&ctrl->work, 1);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= ngroups) break;
        force_group<kMethod, kComp, kEpsZero, kQuad>(s, p, s_dq, g, lane, ws);
    }
}

template <int kMethod, bool kComp, bool kQuad>
static cudaError_t launch_force_t(const DevSim &s, const StepParams &p, int sm_count, cudaStream_t st) {
    const bool ez = !(p.eps > 0.0f);
    const void *fn = ez ? (const void *)k_force<kMethod, kComp, true, kQuad>
                        : (const void *)k_force<kMethod, kComp, false, kQuad>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kForceThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int blocks = per_sm * sm_count;
    const int need = ((s.n + 31) / 32 + kForceWarps - 1) / kForceWarps;
    if (blocks > need) blocks = need > 0 ? need : 1;
    if (ez) k_force<kMethod, kComp, true, kQuad><<<blocks, kForceThreads, 0, st>>>(s, p);
    else k_force<kMethod, kComp, false, kQuad><<<blocks, kForceThreads, 0, st>>>(s, p);
    return cudaGetLastError();
}

template <int kMethod>
static cudaError_t launch_force_m(const DevSim &s, const StepParams &p, int compensated, int sm_count,
                                  cudaStream_t st) {
    if (p.quadrupole) {
        return compensated ? launch_force_t<kMethod, true, true>(s, p, sm_count, st)
                           : launch_force_t<kMethod, false, true>(s, p, sm_count, st);
    }
    return compensated ? launch_force_t<kMethod, true, false>(s, p, sm_count, st)
                       : launch_force_t<kMethod, false, false>(s, p, sm_count, st);
}

cudaError_t launch_force(const DevSim &s, const StepParams &p, int compensated, int sm_count, cudaStream_t st) {
    switch (p.method) {
    case 1: return launch_force_m<1>(s, p, compensated, sm_count, st);
    case 2: return launch_force_m<2>(s, p, compensated, sm_count, st);
    case 3: return launch_force_m<3>(s, p, compensated, sm_count, st);
    default: return launch_force_m<0>(s, p, compensated, sm_count, st);
    }
}

}  // namespace nbgb
