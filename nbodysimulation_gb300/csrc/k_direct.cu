// k_direct.cu -- all-pairs kernels: the direct sums (update /
// update_local, kernels/brute_force_update.cl), the collision update
// (kernels/collision_update.cl) and copy_vertices (kernels/copy_vertices.cl),
// plus the host-layout pack/unpack kernels.
//
// The tiled kernels stage j-tiles of packed {x,y,z,m} bodies into shared
// memory with TMA bulk copies (cp.async.bulk ... mbarrier::complete_tx),
// double-buffered, no cluster and no multicast; each thread keeps kI target
// bodies in registers so one broadcast shared-memory load feeds kI
// interactions.  Small systems split the j range over gridDim.y blocks and
// combine partial accelerations with float atomics before a separate
// integrate pass.
#include "collide_device.cuh"
#include "tma.cuh"

namespace nbgb {

constexpr int kTile = 256;          // bodies per staged tile (4 KiB)
constexpr int kDirectThreads = 256;  // allocation-free all-pairs kernel
constexpr int kTiledThreads = 64;    // tiled direct sum: small blocks, many per SM, even load

// ---- pair interactions ----
template <bool kQuirk, bool kEpsZero>
__device__ __forceinline__ void pair(const float4 me, const float4 q, float eps2, float &ax, float &ay, float &az) {
    const float dx = q.x - me.x, dy = q.y - me.y, dz = q.z - me.z;
    if constexpr (!kQuirk) {
        const float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
        const float r = rsqrt_fast(d2);
        float F = (q.w * r) * (r * r);
        if constexpr (kEpsZero) F = d2 > 0.0f ? F : 0.0f;
        ax = fmaf(dx, F, ax);
        ay = fmaf(dy, F, ay);
        az = fmaf(dz, F, az);
    } else {
        // the reference's brute-force arithmetic: n = normalize(r),
        // s = m / (|n|^2 + e^2) (brute_force_update.cl:54-60, 114-123);
        // the zero vector normalises to zero, so the self pair adds nothing
        const float l2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        const float inv = l2 > 0.0f ? rsqrtf(l2) : 0.0f;
        const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
        const float dist_sqr = fmaf(nz, nz, fmaf(ny, ny, fmaf(nx, nx, eps2)));
        const float s = __fdividef(q.w, dist_sqr);
        ax = fmaf(nx, s, ax);
        ay = fmaf(ny, s, ay);
        az = fmaf(nz, s, az);
    }
}

template <int kMethod>
__device__ __forceinline__ void integrate_one(const DevSim &s, const StepParams &p, int b, const float4 P, float ax,
                                              float ay, float az) {
    const float dt = p.dt;
    const float4 v = s.vel[b];
    float4 x = P, vo = v;
    if constexpr (kMethod == 2) {
        vo.x = __fadd_rn(v.x, __fmul_rn(ax, dt));
        vo.y = __fadd_rn(v.y, __fmul_rn(ay, dt));
        vo.z = __fadd_rn(v.z, __fmul_rn(az, dt));
        x.x = __fadd_rn(P.x, __fmul_rn(vo.x, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(vo.y, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(vo.z, dt));
        s.acc[b] = make_float4(ax, ay, az, 0.0f);
    } else if constexpr (kMethod == 1) {
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
    } else if constexpr (kMethod == 3) {
        const float h = p.kdk_primed ? dt : __fmul_rn(dt, 0.5f);
        vo.x = __fadd_rn(v.x, __fmul_rn(ax, h));
        vo.y = __fadd_rn(v.y, __fmul_rn(ay, h));
        vo.z = __fadd_rn(v.z, __fmul_rn(az, h));
        x.x = __fadd_rn(P.x, __fmul_rn(vo.x, dt));
        x.y = __fadd_rn(P.y, __fmul_rn(vo.y, dt));
        x.z = __fadd_rn(P.z, __fmul_rn(vo.z, dt));
        s.acc[b] = make_float4(ax, ay, az, 0.0f);
    }
    s.vel[b] = vo;
    s.body_next[b] = x;
}

// ---------------------------------------------------------------------------
// direct_global: one thread per body, j straight from global memory through
// L1 (update, brute_force_update.cl:3-105), no shared-memory staging.  When
// the bodies alone do not fill the GPU (the reference runs this variant at
// N = 4096: 32 blocks for 152 SMs), gridDim.y blocks split the j range and
// add partial accelerations into `part` (float atomics) for a separate
// integrate pass.
// ---------------------------------------------------------------------------
constexpr int kGlobalThreads = 128;
template <int kMethod, bool kQuirk, bool kEpsZero>
__global__ void __launch_bounds__(kGlobalThreads) k_direct_global(DevSim s, StepParams p, float eps, float4 *part) {
    const int n = s.n;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int per = (n + gridDim.y - 1) / gridDim.y;
    const int j0 = blockIdx.y * per, j1 = min(n, j0 + per);
    const float4 me = s.body_cur[i];
    const float eps2 = eps * eps;
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    for (int j = j0; j < j1; ++j) {
        const float4 q = __ldg(&s.body_cur[j]);
        if (!kQuirk && kEpsZero && j == i) continue;
        pair<kQuirk, false>(me, q, eps2, ax, ay, az);
    }
    if (gridDim.y == 1) {
        integrate_one<kMethod>(s, p, i, me, ax * p.G, ay * p.G, az * p.G);
    } else {
        atomicAdd(&part[i].x, ax);
        atomicAdd(&part[i].y, ay);
        atomicAdd(&part[i].z, az);
    }
}

// ---------------------------------------------------------------------------
// direct_tiled (update_local, brute_force_update.cl:128-228): TMA-staged
// j-tiles.  The reference's tile loop reloads tile 0 and skips the wrong body
// (:167-184); here every j is visited once.
//
// A block is kG groups of 64 threads that share the same 64*kI targets and
// split the j range between them: each stage brings kG consecutive tiles,
// group g takes the g-th, and at the end the groups' partial sums are added
// in group order (deterministic).  More warps per target set hide the MUFU
// and shared-memory latencies without more shared-memory loads per pair.
// gridDim.y > 1 splits the j range over blocks as well and accumulates the
// partial accelerations into `part` (float atomics).
// ---------------------------------------------------------------------------
template <int kI, int kG, int kMethod, bool kQuirk, bool kEpsZero>
__global__ void __launch_bounds__(kTiledThreads *kG) k_direct_tiled(DevSim s, StepParams p, float eps, float4 *part) {
    __shared__ __align__(128) float4 tile[2][kG][kTile];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ float red[kG > 1 ? kG - 1 : 1][3 * kI][kTiledThreads];
    const int n = s.n;
    const int grp = threadIdx.x / kTiledThreads, gl = threadIdx.x % kTiledThreads;
    const int ntiles = (n + kTile - 1) / kTile;
    const int per_split = (ntiles + gridDim.y - 1) / gridDim.y;
    const int t0 = blockIdx.y * per_split;
    const int t1 = min(ntiles, t0 + per_split);
    const int nst = (t1 - t0 + kG - 1) / kG;  // stages of kG tiles
    const float eps2 = eps * eps;
    int idx[kI];
    float4 me[kI];
    float ax[kI], ay[kI], az[kI];
#pragma unroll
    for (int r = 0; r < kI; ++r) {
        idx[r] = blockIdx.x * (kTiledThreads * kI) + r * kTiledThreads + gl;
        me[r] = idx[r] < n ? s.body_cur[idx[r]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ax[r] = ay[r] = az[r] = 0.0f;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int st, int stage) {
        uint32_t total = 0;
#pragma unroll
        for (int g = 0; g < kG; ++g) {
            const int t = t0 + st * kG + g;
            if (t < t1) total += (uint32_t)min(kTile, n - t * kTile) * 16u;
        }
        mbar_expect_tx(&bar[stage], total);
#pragma unroll
        for (int g = 0; g < kG; ++g) {
            const int t = t0 + st * kG + g;
            if (t < t1)
                bulk_g2s(&tile[stage][g][0], s.body_cur + (size_t)t * kTile,
                         (uint32_t)min(kTile, n - t * kTile) * 16u, &bar[stage]);
        }
    };
    if (threadIdx.x == 0 && nst > 0) issue(0, 0);
    bool ok = true;
    for (int st = 0; st < nst; ++st) {
        const int stage = st & 1;
        if (threadIdx.x == 0 && st + 1 < nst) issue(st + 1, stage ^ 1);
        if (!mbar_wait_bounded(&bar[stage], (uint32_t)((st >> 1) & 1), s.ctrl)) ok = false;
        const int t = t0 + st * kG + grp;
        const int cnt = t < t1 ? min(kTile, n - t * kTile) : 0;
        const float4 *tl = tile[stage][grp];
        if (cnt == kTile) {
#pragma unroll 4
            for (int j = 0; j < kTile; ++j) {
                const float4 q = tl[j];
#pragma unroll
                for (int r = 0; r < kI; ++r) pair<kQuirk, kEpsZero>(me[r], q, eps2, ax[r], ay[r], az[r]);
            }
        } else {
            for (int j = 0; j < cnt; ++j) {
                const float4 q = tl[j];
#pragma unroll
                for (int r = 0; r < kI; ++r) pair<kQuirk, kEpsZero>(me[r], q, eps2, ax[r], ay[r], az[r]);
            }
        }
        if (!__syncthreads_and(ok)) {
            // drain the copies already issued for the next stage before leaving
            if (threadIdx.x == 0 && st + 1 < nst)
                mbar_wait_bounded(&bar[stage ^ 1], (uint32_t)(((st + 1) >> 1) & 1), s.ctrl);
            ok = false;
            break;
        }
    }
    if (!ok) return;
    if constexpr (kG > 1) {
        if (grp > 0) {
#pragma unroll
            for (int r = 0; r < kI; ++r) {
                red[grp - 1][3 * r][gl] = ax[r];
                red[grp - 1][3 * r + 1][gl] = ay[r];
                red[grp - 1][3 * r + 2][gl] = az[r];
            }
        }
        __syncthreads();
        if (grp > 0) return;
#pragma unroll
        for (int g = 1; g < kG; ++g) {
#pragma unroll
            for (int r = 0; r < kI; ++r) {
                ax[r] += red[g - 1][3 * r][gl];
                ay[r] += red[g - 1][3 * r + 1][gl];
                az[r] += red[g - 1][3 * r + 2][gl];
            }
        }
    }
#pragma unroll
    for (int r = 0; r < kI; ++r) {
        if (idx[r] >= n) continue;
        if (gridDim.y == 1) {
            integrate_one<kMethod>(s, p, idx[r], me[r], ax[r] * p.G, ay[r] * p.G, az[r] * p.G);
        } else {
            atomicAdd(&part[idx[r]].x, ax[r]);
            atomicAdd(&part[idx[r]].y, ay[r]);
            atomicAdd(&part[idx[r]].z, az[r]);
        }
    }
}

template <int kMethod>
__global__ void k_integrate_partial(DevSim s, StepParams p, const float4 *part) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const float4 a = part[i];
    integrate_one<kMethod>(s, p, i, s.body_cur[i], a.x * p.G, a.y * p.G, a.z * p.G);
}

// ---------------------------------------------------------------------------
// collision update (update_collision_local, kernels/collision_update.cl:17-83;
// collide_device.cuh).  It reads the positions the integrator of the same step
// wrote, as the reference runs it after the force kernel
// (src/MyApp.cpp:593-596).  A step that failed keeps its step-start state,
// so the update does not run then.  Block form: one target per thread;
// warp form (systems too small to fill the GPU with blocks): one target per
// warp, 32 bodies tested at a time.  Both give the same bits.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kCollideThreads) k_collision(DevSim s, const int *order) {
    if (read_status(s.ctrl)) return;  // block-uniform, before any barrier
    collide_block(s.body_next, s.vel, order, s.n, blockIdx.x * kCollideThreads, s.ctrl);
}

__global__ void __launch_bounds__(kCollideWarps * 32) k_collision_warp(DevSim s) {
    if (read_status(s.ctrl)) return;  // warp-uniform
    const int lane = threadIdx.x & 31;
    collide_warp(s.body_next, s.vel, s.n, blockIdx.x * kCollideWarps + (threadIdx.x >> 5), lane);
}

__global__ void k_copy_vertices(const float4 *__restrict__ b, int n, float4 *__restrict__ dst) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = b[i];
        dst[i] = make_float4(p.x, p.y, p.z, 1.0f);
    }
}

// The reference's packed float[3N] arrays <-> the float4 body layout.  A
// block moves tiles of kPackTile bodies; when the float[3N] arrays are 16-byte
// aligned, a whole tile's 3 * kPackTile floats move as contiguous float4
// loads or stores through shared memory (the arrays may be pinned host
// memory the device reads or writes directly, where full-width accesses
// matter), otherwise as one float at a time.
constexpr int kPackTile = 256;
constexpr int kPackVec = kPackTile * 3 / 4;  // float4 per tile of float[3]

__global__ void __launch_bounds__(kPackTile) k_pack(const float *__restrict__ pos3, const float *__restrict__ mass,
                                                    const float *__restrict__ vel3, float4 *body, float4 *vel,
                                                    float4 *acc, int n, int vec) {
    __shared__ float4 tp[kPackVec], tv[kPackVec];
    const float *fp = reinterpret_cast<const float *>(tp), *fv = reinterpret_cast<const float *>(tv);
    const int t = threadIdx.x;
    const int ntiles = (n + kPackTile - 1) / kPackTile;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const size_t i0 = (size_t)tile * kPackTile;
        const size_t i = i0 + t;
        const bool full = vec && i0 + kPackTile <= (size_t)n;  // block-uniform
        if (full && t < kPackVec) {
            if (pos3) tp[t] = reinterpret_cast<const float4 *>(pos3 + 3 * i0)[t];
            if (vel3) tv[t] = reinterpret_cast<const float4 *>(vel3 + 3 * i0)[t];
        }
        __syncthreads();
        if (i < (size_t)n) {
            if (pos3) {
                const float m = mass ? mass[i] : body[i].w;
                body[i] = full ? make_float4(fp[3 * t], fp[3 * t + 1], fp[3 * t + 2], m)
                               : make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], m);
            } else if (mass) {
                body[i].w = mass[i];
            }
            if (vel) {
                float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                if (vel3) v = full ? make_float4(fv[3 * t], fv[3 * t + 1], fv[3 * t + 2], 0.0f)
                                   : make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.0f);
                vel[i] = v;
            }
            if (acc) acc[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        __syncthreads();  // the tile is read before the next one is staged
    }
}

// one float4 array -> one float[3N] array, tile at i0 (block-uniform `full`)
__device__ __forceinline__ void unpack_tile(const float4 *__restrict__ src, float *dst, size_t i0, int n, bool full,
                                            float4 *tile) {
    const int t = threadIdx.x;
    const size_t i = i0 + t;
    if (full) {
        float *f = reinterpret_cast<float *>(tile);
        const float4 v = src[i];
        f[3 * t] = v.x;
        f[3 * t + 1] = v.y;
        f[3 * t + 2] = v.z;
        __syncthreads();
        if (t < kPackVec) reinterpret_cast<float4 *>(dst + 3 * i0)[t] = tile[t];
        __syncthreads();
    } else if (i < (size_t)n) {
        const float4 v = src[i];
        dst[3 * i] = v.x;
        dst[3 * i + 1] = v.y;
        dst[3 * i + 2] = v.z;
    }
}

__global__ void __launch_bounds__(kPackTile) k_unpack(const float4 *__restrict__ body, const float4 *__restrict__ vel,
                                                      const float4 *__restrict__ acc, float *pos3, float *vel3,
                                                      float *acc3, int n, int vec) {
    __shared__ float4 tile[kPackVec];
    const int ntiles = (n + kPackTile - 1) / kPackTile;
    for (int k = blockIdx.x; k < ntiles; k += gridDim.x) {
        const size_t i0 = (size_t)k * kPackTile;
        const bool full = vec && i0 + kPackTile <= (size_t)n;  // block-uniform
        if (pos3) unpack_tile(body, pos3, i0, n, full, tile);
        if (vel3) unpack_tile(vel, vel3, i0, n, full, tile);
        if (acc3) unpack_tile(acc, acc3, i0, n, full, tile);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
template <int kMethod, bool kQuirk, bool kEpsZero>
static cudaError_t launch_direct_t(const DevSim &s, const StepParams &p, float eps, int tiled, int sm_count,
                                   cudaStream_t st, float4 *part) {
    const int n = s.n;
    if (!tiled) {
        const int bx = (n + kGlobalThreads - 1) / kGlobalThreads;
        int split = (sm_count * 6 + bx - 1) / bx;
        if (split > (n + 63) / 64) split = (n + 63) / 64;  // at least 64 j per block
        if (split <= 1) {
            k_direct_global<kMethod, kQuirk, kEpsZero><<<dim3(bx, 1), kGlobalThreads, 0, st>>>(s, p, eps, part);
            return cudaGetLastError();
        }
        cudaError_t e = cudaMemsetAsync(part, 0, sizeof(float4) * (size_t)n, st);
        if (e != cudaSuccess) return e;
        k_direct_global<kMethod, kQuirk, kEpsZero><<<dim3(bx, split), kGlobalThreads, 0, st>>>(s, p, eps, part);
        k_integrate_partial<kMethod><<<(n + 255) / 256, 256, 0, st>>>(s, p, part);
        return cudaGetLastError();
    }
    // bodies per thread: the most that still gives at least six blocks per
    // SM (every block does the same work, so many small blocks keep the SMs
    // evenly loaded), two j-groups per block; below that, split the j range
    // over gridDim.y
    const int want = sm_count * 6;
    const int bx4 = (n + kTiledThreads * 4 - 1) / (kTiledThreads * 4);
    const int bx3 = (n + kTiledThreads * 3 - 1) / (kTiledThreads * 3);
    const int bx2 = (n + kTiledThreads * 2 - 1) / (kTiledThreads * 2);
    const int bx1 = (n + kTiledThreads - 1) / kTiledThreads;
    const int ntiles = (n + kTile - 1) / kTile;
    if (bx4 >= want) {
        // every block does the same work, so the busiest SM holds
        // ceil(blocks / SMs) of them: 3 targets per thread when that evens
        // the SMs out enough to pay for the extra shared-memory load per pair
        // (N = 262,144: 1024 blocks of 4 -> 7 on the busiest SM, 28 target
        // rows; 1366 blocks of 3 -> 9, 27)
        const long long cost4 = 4LL * ((bx4 + sm_count - 1) / sm_count);
        const long long cost3 = 3LL * ((bx3 + sm_count - 1) / sm_count);
        if (cost3 < cost4) {
            k_direct_tiled<3, 2, kMethod, kQuirk, kEpsZero><<<dim3(bx3, 1), 2 * kTiledThreads, 0, st>>>(s, p, eps,
                                                                                                     part);
            return cudaGetLastError();
        }
        k_direct_tiled<4, 2, kMethod, kQuirk, kEpsZero><<<dim3(bx4, 1), 2 * kTiledThreads, 0, st>>>(s, p, eps, part);
        return cudaGetLastError();
    }
    if (bx2 >= want) {
        k_direct_tiled<2, 2, kMethod, kQuirk, kEpsZero><<<dim3(bx2, 1), 2 * kTiledThreads, 0, st>>>(s, p, eps, part);
        return cudaGetLastError();
    }
    int split = (want + bx1 - 1) / bx1;
    if (split > ntiles) split = ntiles;
    if (split < 1) split = 1;
    if (split == 1) {
        k_direct_tiled<1, 1, kMethod, kQuirk, kEpsZero><<<dim3(bx1, 1), kTiledThreads, 0, st>>>(s, p, eps, part);
        return cudaGetLastError();
    }
    cudaError_t e = cudaMemsetAsync(part, 0, sizeof(float4) * (size_t)n, st);
    if (e != cudaSuccess) return e;
    k_direct_tiled<1, 1, kMethod, kQuirk, kEpsZero><<<dim3(bx1, split), kTiledThreads, 0, st>>>(s, p, eps, part);
    k_integrate_partial<kMethod><<<(n + 255) / 256, 256, 0, st>>>(s, p, part);
    return cudaGetLastError();
}

template <int kMethod>
static cudaError_t launch_direct_m(const DevSim &s, const StepParams &p, float eps, int tiled, int quirk,
                                   int sm_count, cudaStream_t st, float4 *part) {
    const bool ez = !(eps > 0.0f);
    if (quirk) return launch_direct_t<kMethod, true, false>(s, p, eps, tiled, sm_count, st, part);
    if (ez) return launch_direct_t<kMethod, false, true>(s, p, eps, tiled, sm_count, st, part);
    return launch_direct_t<kMethod, false, false>(s, p, eps, tiled, sm_count, st, part);
}

// `p.eps` is the softening to use; s.part (N float4) holds the partial sums
// of a split j range.
cudaError_t launch_direct(const DevSim &s, const StepParams &p, int tiled, int quirk, int sm_count,
                          cudaStream_t st) {
    float4 *part = s.part;
    switch (p.method) {
    case 1: return launch_direct_m<1>(s, p, p.eps, tiled, quirk, sm_count, st, part);
    case 2: return launch_direct_m<2>(s, p, p.eps, tiled, quirk, sm_count, st, part);
    case 3: return launch_direct_m<3>(s, p, p.eps, tiled, quirk, sm_count, st, part);
    default: return launch_direct_m<0>(s, p, p.eps, tiled, quirk, sm_count, st, part);
    }
}

cudaError_t launch_collision(const DevSim &s, int tree, int sm_count, cudaStream_t st) {
    const int blocks = (s.n + kCollideThreads - 1) / kCollideThreads;
    if (blocks < collide_warp_form_below(sm_count))
        k_collision_warp<<<(s.n + kCollideWarps - 1) / kCollideWarps, kCollideWarps * 32, 0, st>>>(s);
    else
        k_collision<<<blocks, kCollideThreads, 0, st>>>(s, tree ? s.sorted : nullptr);
    return cudaGetLastError();
}

cudaError_t launch_copy_vertices(const float4 *body, int n, float4 *dst, cudaStream_t st) {
    k_copy_vertices<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(body, n, dst);
    return cudaGetLastError();
}

static bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

cudaError_t launch_pack(const float *pos3, const float *mass, const float *vel3, float4 *body, float4 *vel,
                        float4 *acc, int n, cudaStream_t st) {
    const int tiles = (n + kPackTile - 1) / kPackTile;
    const int blocks = tiles < 4096 ? tiles : 4096;
    const int vec = aligned16(pos3) && aligned16(vel3);
    k_pack<<<blocks > 0 ? blocks : 1, kPackTile, 0, st>>>(pos3, mass, vel3, body, vel, acc, n, vec);
    return cudaGetLastError();
}

cudaError_t launch_unpack(const float4 *body, const float4 *vel, const float4 *acc, float *pos3, float *vel3,
                          float *acc3, int n, cudaStream_t st) {
    const int tiles = (n + kPackTile - 1) / kPackTile;
    const int blocks = tiles < 4096 ? tiles : 4096;
    const int vec = aligned16(pos3) && aligned16(vel3) && aligned16(acc3);
    k_unpack<<<blocks > 0 ? blocks : 1, kPackTile, 0, st>>>(body, vel, acc, pos3, vel3, acc3, n, vec);
    return cudaGetLastError();
}

}  // namespace nbgb

namespace nbgb {

// ===========================================================================
// Allocation-free all-pairs accelerations (nb_direct_accel_noalloc).
//
// For callers that must not allocate device memory: a host engine that owns
// the whole device-memory budget and hands the library only its own buffers,
// or a frame loop where a cudaMalloc (which can synchronise the device and
// take an allocator lock) is not allowed.  The caller passes the bodies and
// the output; the one piece of scratch the split all-pairs sum needs -- the
// partial accelerations of the j slices -- lives in a file-scope device
// array of fixed size, together with a status word for the bounded waits.
// Every GPU that loads this library holds that array (1 MiB + 80 B) until
// the process exits.  All calls share it: calls that overlap on the GPU race.
// ===========================================================================
constexpr int kNoAllocMaxBodies = 65536;  // = NB_NOALLOC_MAX_BODIES
static __device__ __align__(256) float4 g_noalloc_part[kNoAllocMaxBodies];
static __device__ __align__(256) Ctrl g_noalloc_ctrl;

// The tiled all-pairs kernel above with the j range split over gridDim.y and
// every slice adding its partial sums into `part`; no integrator.
template <bool kEpsZero>
__global__ void __launch_bounds__(kDirectThreads) k_noalloc_partial(const float4 *__restrict__ body, int n,
                                                                     float eps2, float4 *part, Ctrl *ctrl) {
    __shared__ __align__(128) float4 tile[2][kTile];
    __shared__ __align__(8) uint64_t bar[2];
    const int ntiles = (n + kTile - 1) / kTile;
    const int per_split = (ntiles + gridDim.y - 1) / gridDim.y;
    const int t0 = blockIdx.y * per_split;
    const int t1 = min(ntiles, t0 + per_split);
    const int i = blockIdx.x * kDirectThreads + threadIdx.x;
    const float4 me = i < n ? body[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float ax = 0.0f, ay = 0.0f, az = 0.0f;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int t, int stage) {
        const int cnt = min(kTile, n - t * kTile);
        const uint32_t bytes = (uint32_t)cnt * 16u;
        mbar_expect_tx(&bar[stage], bytes);
        bulk_g2s(&tile[stage][0], body + (size_t)t * kTile, bytes, &bar[stage]);
    };
    if (threadIdx.x == 0 && t0 < t1) issue(t0, 0);
    bool ok = true;
    for (int t = t0; t < t1; ++t) {
        const int it = t - t0;
        const int stage = it & 1;
        if (threadIdx.x == 0 && t + 1 < t1) issue(t + 1, stage ^ 1);
        if (!mbar_wait_bounded(&bar[stage], (uint32_t)((it >> 1) & 1), ctrl)) ok = false;
        const int cnt = min(kTile, n - t * kTile);
        for (int j = 0; j < cnt; ++j) pair<false, kEpsZero>(me, tile[stage][j], eps2, ax, ay, az);
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0 && t + 1 < t1)
                mbar_wait_bounded(&bar[stage ^ 1], (uint32_t)(((it + 1) >> 1) & 1), ctrl);
            ok = false;
            break;
        }
    }
    if (!ok || i >= n) return;
    atomicAdd(&part[i].x, ax);
    atomicAdd(&part[i].y, ay);
    atomicAdd(&part[i].z, az);
}

__global__ void k_noalloc_finish(const float4 *__restrict__ part, int n, float G, float4 *__restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 a = part[i];
    out[i] = make_float4(a.x * G, a.y * G, a.z * G, 0.0f);
}

}  // namespace nbgb

#include <mutex>

#include "../../include/nbgb.h"

static_assert(nbgb::kNoAllocMaxBodies == NB_NOALLOC_MAX_BODIES, "the scratch must hold the documented limit");

namespace {
// Device addresses of the two arrays, looked up once per device with that
// device current.  In host code the array names are host-side stand-ins, not
// device addresses, so only these looked-up pointers are passed to kernels.
// The addresses are kept for the life of the process: a cudaDeviceReset (or
// a reset of the device's primary context) unloads the module, after which
// this entry point must not be called on that device again.
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void *g_noalloc_part_ptr[kMaxDevices] = {};
void *g_noalloc_ctrl_ptr[kMaxDevices] = {};

bool noalloc_setup(int dev, float4 **part, nbgb::Ctrl **ctrl) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_part_ptr[dev]) {
        void *p = nullptr, *c = nullptr;
        if (cudaGetSymbolAddress(&p, nbgb::g_noalloc_part) != cudaSuccess) return false;
        if (cudaGetSymbolAddress(&c, nbgb::g_noalloc_ctrl) != cudaSuccess) return false;
        g_noalloc_part_ptr[dev] = p;
        g_noalloc_ctrl_ptr[dev] = c;
    }
    *part = static_cast<float4 *>(g_noalloc_part_ptr[dev]);
    *ctrl = static_cast<nbgb::Ctrl *>(g_noalloc_ctrl_ptr[dev]);
    return true;
}
}  // namespace

extern "C" nb_status nb_direct_accel_noalloc(const float *d_body4, int32_t n, float eps, float G, float *d_acc4,
                                            void *stream) {
    using namespace nbgb;
    if (!d_body4 || !d_acc4 || n < 1 || !(eps >= 0.0f)) return NB_ERR_INVALID_ARGUMENT;
    if (n > kNoAllocMaxBodies) return NB_ERR_INVALID_ARGUMENT;  // beyond the fixed scratch
    if (((uintptr_t)d_body4 & 15u) || ((uintptr_t)d_acc4 & 15u)) return NB_ERR_INVALID_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return NB_ERR_NO_DEVICE;
    float4 *part = nullptr;
    Ctrl *ctrl = nullptr;
    if (!noalloc_setup(dev, &part, &ctrl)) return NB_ERR_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the scratch keeps the previous call's contents: clear what must start at 0
    if (cudaMemsetAsync(part, 0, sizeof(float4) * (size_t)n, st) != cudaSuccess) return NB_ERR_CUDA;
    if (cudaMemsetAsync(ctrl, 0, sizeof(Ctrl), st) != cudaSuccess) return NB_ERR_CUDA;
    int sm_count = 0;
    cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
    const int bx = (n + kDirectThreads - 1) / kDirectThreads;
    const int ntiles = (n + kTile - 1) / kTile;
    int split = (2 * sm_count + bx - 1) / bx;
    if (split > ntiles) split = ntiles;
    if (split < 1) split = 1;
    const float eps2 = eps * eps;
    const float4 *body = reinterpret_cast<const float4 *>(d_body4);
    if (eps > 0.0f) k_noalloc_partial<false><<<dim3(bx, split), kDirectThreads, 0, st>>>(body, n, eps2, part, ctrl);
    else k_noalloc_partial<true><<<dim3(bx, split), kDirectThreads, 0, st>>>(body, n, eps2, part, ctrl);
    k_noalloc_finish<<<bx, kDirectThreads, 0, st>>>(part, n, G, reinterpret_cast<float4 *>(d_acc4));
    if (cudaGetLastError() != cudaSuccess) return NB_ERR_CUDA;
    // wait, then read the status of the bounded waits (no allocation: a
    // stack variable receives it)
    int status = 0;
    if (cudaMemcpyAsync(&status, &ctrl->status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return NB_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return NB_ERR_CUDA;
    return status ? (nb_status)status : NB_OK;
}
