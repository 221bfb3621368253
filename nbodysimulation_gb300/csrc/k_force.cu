// k_force.cu -- Barnes-Hut force walk with the fused integrator
// (calculate_force_local, kernels/calculate_forces.cl:4-185).
//
// One warp owns 32 consecutive bodies of the in-order sort, so its bodies
// are spatial neighbours.  The warp walks the tree with one shared stack of
// cells to open (shared memory, 512 entries per warp).  Opening a cell reads
// its compacted child list (32 B) and the packed {x,y,z,m} of its children
// (one 128 B line) -- all loads issued at once, one memory round trip per
// opened cell.  A child body is always accumulated; a child cell is
// accumulated when EVERY lane of the warp accepts it (__all_sync of
// d^2 >= dq[level], the reference's work_group_all at :121, here over a real
// 32-lane warp), otherwise it is pushed.  Softened gravity
// F = m * rsqrt(d^2)^3 (MUFU rsqrt), d^2 = |d|^2 + eps^2 as FMAs.
//
// The integrator writes the next position buffer, so every force of the step
// sees step-start positions (the reference integrates in place while other
// work-items still read positions, :159-180).
#include "nbgb_internal.cuh"

namespace nbgb {

constexpr int kForceWarps = 8;
constexpr int kForceThreads = kForceWarps * 32;
constexpr int kStack = 512;  // >= 7 * kMaxDepth + 1 cells pending per warp

template <int kMethod>
__device__ __forceinline__ void integrate_body(const DevSim &s, const StepParams &p, int b, const float4 P, float ax,
                                               float ay, float az) {
    const float dt = p.dt;
    const float4 v = s.vel[b];
    float4 x = P, vo = v;
    if constexpr (kMethod == 2) {  // Euler (calculate_forces.cl:168-181)
        vo.x = __fadd_rn(v.x, __fmul_rn(ax, dt));
        vo.y = __fadd_rn(v.y, __fmul_rn(ay, dt));
        vo.z = __fadd_rn(v.z, __fmul_rn(az, dt));
        x.x = __fadd_rn(P.x, __fmul_rn(vo.x, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(vo.y, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(vo.z, dt));
        s.acc[b] = make_float4(ax, ay, az, 0.0f);
    } else if constexpr (kMethod == 1) {  // "Leapfrog" as written (:152-167): acc read, not written
        const float4 ap = s.acc[b];
        const float hx = __fadd_rn(v.x, __fmul_rn(__fmul_rn(ap.x, dt), 0.5f));
        const float hy = __fadd_rn(v.y, __fmul_rn(__fmul_rn(ap.y, dt), 0.5f));
        const float hz = __fadd_rn(v.z, __fmul_rn(__fmul_rn(ap.z, dt), 0.5f));
        x.x = __fadd_rn(P.x, __fmul_rn(hx, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(hy, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(hz, dt));
        vo.x = __fadd_rn(hx, __fmul_rn(__fmul_rn(ax, dt), 0.5f));
        vo.y = __fadd_rn(hy, __fmul_rn(__fmul_rn(ay, dt), 0.5f));
        vo.z = __fadd_rn(hz, __fmul_rn(__fmul_rn(az, dt), 0.5f));
    } else if constexpr (kMethod == 3) {  // kick-drift-kick, velocities at half steps
        const float h = p.kdk_primed ? dt : __fmul_rn(dt, 0.5f);
        vo.x = __fadd_rn(v.x, __fmul_rn(ax, h));
        vo.y = __fadd_rn(v.y, __fmul_rn(ay, h));
        vo.z = __fadd_rn(v.z, __fmul_rn(az, h));
        x.x = __fadd_rn(P.x, __fmul_rn(vo.x, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(vo.y, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(vo.z, dt));
        s.acc[b] = make_float4(ax, ay, az, 0.0f);
    } else {  // any other method value moves nothing (the as-wired reference)
    }
    s.vel[b] = vo;
    s.body_next[b] = x;
}

__device__ __forceinline__ void two_sum_add(float &hi, float &lo, float t) {
    const float s = __fadd_rn(hi, t);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(t, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}

template <int kMethod, bool kComp, bool kEpsZero>
__global__ void __launch_bounds__(kForceThreads, 2) k_force(DevSim s, StepParams p) {
    __shared__ float s_dq[kMaxDepth];
    __shared__ int2 s_stack[kForceWarps][kStack];
    __shared__ int s_skip;
    Ctrl *ctrl = s.ctrl;
    const int n = s.n, root = n + s.cap;
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
    int2 *stack = s_stack[w];
    const float eps2 = __fmul_rn(p.eps, p.eps);
    const int ngroups = (n + 31) >> 5;
    const int4 *wchild4 = reinterpret_cast<const int4 *>(s.wchild);
    for (int g = blockIdx.x * kForceWarps + w; g < ngroups; g += gridDim.x * kForceWarps) {
        const int sidx = g * 32 + lane;
        const bool valid = sidx < n;
        const int b = s.sorted[valid ? sidx : g * 32];
        const float4 P = s.body_cur[b];
        float ax = 0.0f, ay = 0.0f, az = 0.0f, lx = 0.0f, ly = 0.0f, lz = 0.0f;
        int sp = 1;
        unsigned n_acc = 0, n_open = 0;
        if (lane == 0) stack[0] = make_int2(root, 0);
        __syncwarp();
        while (sp > 0) {
            --sp;
            const int2 e = stack[sp];
            __syncwarp();
            const int c = e.x - n;
            const float thr = s_dq[e.y];
            ++n_open;
            const int4 i0 = __ldg(&wchild4[c * 2]);
            const int4 i1 = __ldg(&wchild4[c * 2 + 1]);
            float4 q[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) q[j] = __ldg(&s.wpm[c * 8 + j]);
            const int chs[8] = {i0.x, i0.y, i0.z, i0.w, i1.x, i1.y, i1.z, i1.w};
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int ch = chs[j];
                if (ch < 0) break;
                const float dx = q[j].x - P.x, dy = q[j].y - P.y, dz = q[j].z - P.z;
                const float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                if (ch < n || __all_sync(0xffffffffu, !valid || d2 >= thr)) {
                    ++n_acc;
                    const float r = rsqrtf(d2);
                    float F = (q[j].w * r) * (r * r);
                    if constexpr (kEpsZero) F = d2 > 0.0f ? F : 0.0f;
                    if constexpr (kComp) {
                        two_sum_add(ax, lx, dx * F);
                        two_sum_add(ay, ly, dy * F);
                        two_sum_add(az, lz, dz * F);
                    } else {
                        ax = fmaf(dx, F, ax);
                        ay = fmaf(dy, F, ay);
                        az = fmaf(dz, F, az);
                    }
                } else if (sp < kStack && e.y + 1 < kMaxDepth) {
                    if (lane == 0) stack[sp] = make_int2(ch, e.y + 1);
                    ++sp;
                } else if (lane == 0) {  // cannot happen below kMaxDepth levels; never overrun
                    set_status(ctrl, kStDepth, e.y + 1);
                }
            }
            __syncwarp();
        }
        if (lane == 0) {
            const unsigned lanes = (unsigned)min(32, n - g * 32);
            atomicAdd(&ctrl->interactions, (unsigned long long)n_acc * lanes);
            atomicAdd(&ctrl->opened, (unsigned long long)n_open);
        }
        if constexpr (kComp) {
            ax = ax + lx;
            ay = ay + ly;
            az = az + lz;
        }
        ax *= p.G;
        ay *= p.G;
        az *= p.G;
        if (valid) integrate_body<kMethod>(s, p, b, P, ax, ay, az);
    }
}

template <int kMethod, bool kComp>
static cudaError_t launch_force_t(const DevSim &s, const StepParams &p, int sm_count, cudaStream_t st) {
    const bool ez = !(p.eps > 0.0f);
    const void *fn = ez ? (const void *)k_force<kMethod, kComp, true> : (const void *)k_force<kMethod, kComp, false>;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kForceThreads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    int blocks = per_sm * sm_count;
    const int need = ((s.n + 31) / 32 + kForceWarps - 1) / kForceWarps;
    if (blocks > need) blocks = need > 0 ? need : 1;
    if (ez) k_force<kMethod, kComp, true><<<blocks, kForceThreads, 0, st>>>(s, p);
    else k_force<kMethod, kComp, false><<<blocks, kForceThreads, 0, st>>>(s, p);
    return cudaGetLastError();
}

cudaError_t launch_force(const DevSim &s, const StepParams &p, int compensated, int sm_count, cudaStream_t st) {
    switch (p.method) {
    case 1: return compensated ? launch_force_t<1, true>(s, p, sm_count, st) : launch_force_t<1, false>(s, p, sm_count, st);
    case 2: return compensated ? launch_force_t<2, true>(s, p, sm_count, st) : launch_force_t<2, false>(s, p, sm_count, st);
    case 3: return compensated ? launch_force_t<3, true>(s, p, sm_count, st) : launch_force_t<3, false>(s, p, sm_count, st);
    default: return compensated ? launch_force_t<0, true>(s, p, sm_count, st) : launch_force_t<0, false>(s, p, sm_count, st);
    }
}

}  // namespace nbgb
