// collide_device.cuh -- the collision update (update_collision_local,
// kernels/collision_update.cl:17-83), shared by the single-system kernels
// (k_direct.cu) and the batched one (k_batch.cu), so a batched system's
// velocities equal a standalone handle's bit for bit.
//
// For target i, every other body j in ascending order: if |p_i - p_j| <=
// r_i + r_j (both radii 0.015, :59,65) the running velocity is reflected,
// v <- v - 2 (n.v) n with n = normalize(p_j - p_i) (calc_collision_traj,
// :3-15).  Positions are the ones the integrator of the same step wrote
// (the reference runs the update after the force kernel,
// src/MyApp.cpp:593-596).  Distance and reflection use separately rounded
// operations and a correctly rounded square root and division, so every
// decision and result matches the oracle bit for bit.
//
// Most pairs are far apart.  A pair whose separation along one axis is
// already larger than the contact distance is skipped before the distance
// is formed: in binary floating point sqrt_rn(fl(x*x)) = |x|, and adding the
// other squares (non-negative, rounded to nearest) cannot lower the sum, so
// |dx| > r implies sqrt_rn(dx^2 + dy^2 + dz^2) > r -- the skip takes exactly
// the pairs the full test rejects through that axis, nothing else.  It is
// used only where both positions are finite: with a NaN component the
// reference's distance is NaN, which it counts as a contact.  The skips are
// branches; they stay uniform across a warp when its targets are spatial
// neighbours, so a tree system hands out its targets in the in-order sort
// (each target's result does not depend on which thread computes it).
#pragma once
#include "nbgb_internal.cuh"
#include "tma.cuh"

namespace nbgb {

constexpr int kCollideThreads = kCollideBlockBodies;  // targets per block of the block form
constexpr int kCollideTile = 256;                     // bodies per staged tile (4 KiB)
constexpr int kCollideWarps = 8;                      // targets per block of the warp form

// The warp form serves systems with fewer blocks of targets than SMs (N <
// 38,912 bodies on 152 SMs), the block form the rest.  Measured on a GB300,
// unit ball, tree systems (targets in sort order), warp against block form:
// N = 8,192 0.078 / 0.467 ms, 32,768 1.12 / 1.79 ms, 65,536 4.09 / 3.67 ms,
// 262,144 62.0 / 25.6 ms.
inline int collide_warp_form_below(int sm_count) { return sm_count; }

__device__ __forceinline__ float contact_distance() { return __fadd_rn(0.015f, 0.015f); }

__device__ __forceinline__ bool finite3(const float4 p) {
    return fabsf(p.x) <= 3.402823466e38f && fabsf(p.y) <= 3.402823466e38f && fabsf(p.z) <= 3.402823466e38f;
}

// Is body q within the contact distance rr of me?  (:59-65: the reference
// rejects when dist > rr, so a NaN distance counts as a contact.)  `fast`:
// both positions are finite, so the one-axis rejections apply.
__device__ __forceinline__ bool in_contact(const float4 me, const float4 q, float rr, bool fast) {
    const float ex = __fsub_rn(me.x, q.x);
    if (fast && fabsf(ex) > rr) return false;
    const float ey = __fsub_rn(me.y, q.y);
    if (fast && fabsf(ey) > rr) return false;
    const float ez = __fsub_rn(me.z, q.z);
    if (fast && fabsf(ez) > rr) return false;
    const float dist = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez)));
    return !(dist > rr);
}

// v <- v - 2 (n.v) n, n = normalize(q - me) (normalize leaves a zero
// vector unchanged).
__device__ __forceinline__ void reflect(const float4 me, const float4 q, float4 &v) {
    float nx = __fsub_rn(q.x, me.x), ny = __fsub_rn(q.y, me.y), nz = __fsub_rn(q.z, me.z);
    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
    if (l2 != 0.0f) {
        const float inv = __fdiv_rn(1.0f, __fsqrt_rn(l2));
        nx = __fmul_rn(nx, inv);
        ny = __fmul_rn(ny, inv);
        nz = __fmul_rn(nz, inv);
    }
    const float dp = __fadd_rn(__fadd_rn(__fmul_rn(nx, v.x), __fmul_rn(ny, v.y)), __fmul_rn(nz, v.z));
    const float k2 = __fmul_rn(2.0f, dp);
    v.x = __fsub_rn(v.x, __fmul_rn(k2, nx));
    v.y = __fsub_rn(v.y, __fmul_rn(k2, ny));
    v.z = __fsub_rn(v.z, __fmul_rn(k2, nz));
}

// Block form: thread t of the block updates target number i0 + t (body
// order[i0 + t], or i0 + t without an order) against all n bodies, staged
// in tiles by TMA bulk copies (double-buffered mbarriers, bounded waits).
// Every thread of the block calls it.  Writes vel only when every wait
// succeeded.
__device__ __forceinline__ void collide_block(const float4 *__restrict__ pos, float4 *__restrict__ vel,
                                              const int *__restrict__ order, int n, int i0, Ctrl *ctrl) {
    __shared__ __align__(128) float4 tile[2][kCollideTile];
    __shared__ __align__(8) uint64_t bar[2];
    const int it = i0 + (int)threadIdx.x;
    const int i = it < n ? (order ? order[it] : it) : n;
    const float4 me = i < n ? pos[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 v = i < n ? vel[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float rr = contact_distance();
    const bool me_finite = finite3(me);
    const int ntiles = (n + kCollideTile - 1) / kCollideTile;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int t, int stage) {
        const int cnt = min(kCollideTile, n - t * kCollideTile);
        const uint32_t bytes = (uint32_t)cnt * 16u;
        mbar_expect_tx(&bar[stage], bytes);
        bulk_g2s(&tile[stage][0], pos + (size_t)t * kCollideTile, bytes, &bar[stage]);
    };
    if (threadIdx.x == 0 && ntiles > 0) issue(0, 0);
    bool ok = true;
    for (int t = 0; t < ntiles; ++t) {
        const int stage = t & 1;
        if (threadIdx.x == 0 && t + 1 < ntiles) issue(t + 1, stage ^ 1);
        if (!mbar_wait_bounded(&bar[stage], (uint32_t)((t >> 1) & 1), ctrl)) ok = false;
        const int cnt = min(kCollideTile, n - t * kCollideTile);
        const int j0 = t * kCollideTile;
        // the one-axis rejections only for finite tiles (every thread reads
        // the tile once more; a barrier per 256 bodies)
        const bool tile_finite =
            __syncthreads_and(!ok || (int)threadIdx.x >= cnt || finite3(tile[stage][threadIdx.x]));
        const bool fast = me_finite && tile_finite;
        if (ok)
            for (int j = 0; j < cnt; ++j) {
                const float4 q = tile[stage][j];
                if (j0 + j == i || !in_contact(me, q, rr, fast)) continue;
                reflect(me, q, v);
            }
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0 && t + 1 < ntiles)
                mbar_wait_bounded(&bar[stage ^ 1], (uint32_t)(((t + 1) >> 1) & 1), ctrl);
            ok = false;
            break;
        }
    }
    if (ok && i < n) vel[i] = v;
}

// Warp form, for systems too small to fill the GPU with blocks of targets:
// one warp per target i, lane L tests body j0 + L; the contacts of each
// group of 32 are then applied by every lane in ascending j (a ballot and a
// broadcast of the contact's position), the same sequence of reflections as
// the block form.  All 32 lanes call it.
__device__ __forceinline__ void collide_warp(const float4 *__restrict__ pos, float4 *__restrict__ vel, int n, int i,
                                             int lane) {
    if (i >= n) return;  // warp-uniform
    const float4 me = pos[i];
    float4 v = vel[i];
    const float rr = contact_distance();
    const bool me_finite = finite3(me);
    for (int j0 = 0; j0 < n; j0 += 32) {
        const int j = j0 + lane;
        const float4 q = j < n ? __ldg(&pos[j]) : me;
        const bool fast = me_finite && finite3(q);
        unsigned hit = __ballot_sync(0xffffffffu, j < n && j != i && in_contact(me, q, rr, fast));
        while (hit) {
            const int b = __ffs(hit) - 1;
            hit &= hit - 1;
            const float4 qb = make_float4(__shfl_sync(0xffffffffu, q.x, b), __shfl_sync(0xffffffffu, q.y, b),
                                          __shfl_sync(0xffffffffu, q.z, b), __shfl_sync(0xffffffffu, q.w, b));
            reflect(me, qb, v);
        }
    }
    if (lane == 0) vel[i] = v;
}

}  // namespace nbgb
