// k_batch.cu -- one launch per stage for many independent systems of uneven
// N.  Every kernel walks the batch's table of systems (SysDesc): the work
// of all systems is laid end to end in one index space per stage (bodies in
// chunks, cell slots, warp groups, direct-sum target blocks) and a thread
// finds its system with a binary search in the stage's prefix table.
// Barnes-Hut systems run the same per-item code as the single-system
// kernels (bh_device.cuh, force_device.cuh); small systems take the
// TMA-tiled direct sum.  A step is: reset, bbox, top-level counts, top cells,
// build, used-cell scan, summarize, sort, force, direct, flip -- captured
// once into a CUDA graph by the host.
#include "bh_device.cuh"
#include "collide_device.cuh"
#include "force_device.cuh"
#include "tma.cuh"

namespace nbgb {

// ---------------------------------------------------------------------------
// reset (init, kernels/init.cl:26-33) for every Barnes-Hut system
// ---------------------------------------------------------------------------
__global__ void k_batch_reset(BatchTables t) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t.nsys) return;
    const SysDesc &d = t.sys[k];
    if (!d.active || d.kind != kSysBH || !system_live(d.v.ctrl)) return;
    const DevSim &s = d.v;
    Ctrl *c = s.ctrl;
    c->bbox_key[0] = c->bbox_key[1] = c->bbox_key[2] = 0xFFFFFFFFu;
    c->bbox_key[3] = c->bbox_key[4] = c->bbox_key[5] = 0u;
    int4 *row = reinterpret_cast<int4 *>(&s.child[s.cap * 8]);
    row[0] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
    row[1] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
    c->bottom = s.n + s.cap;
    c->max_depth = 0;
    c->work = 0;
    s.arrive[s.cap] = 0;
    s.start[s.cap] = 0;
    s.count[s.cap] = 0;
    s.parent[s.cap] = -1;
}

// ---------------------------------------------------------------------------
// bbox: one block per chunk of one system; order-preserving integer keys,
// one atomic per component per block (as k_bbox)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_batch_bbox(BatchTables t) {
    const int k = find_system(t.chunk_prefix, t.nsys, blockIdx.x);
    const SysDesc &d = t.sys[k];
    if (!system_live(d.v.ctrl)) return;  // block-uniform
    const DevSim s = system_view(d);
    const int i0 = (blockIdx.x - d.chunk_begin) * d.chunk;
    const int i1 = min(s.n, i0 + d.chunk);
    unsigned mn0 = 0xFFFFFFFFu, mn1 = 0xFFFFFFFFu, mn2 = 0xFFFFFFFFu, mx0 = 0u, mx1 = 0u, mx2 = 0u;
    int bad = -1;
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const float4 p = __ldg(&s.body_cur[i]);
        if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) bad = i;
        const unsigned kx = f2key(p.x), ky = f2key(p.y), kz = f2key(p.z);
        mn0 = min(mn0, kx); mx0 = max(mx0, kx);
        mn1 = min(mn1, ky); mx1 = max(mx1, ky);
        mn2 = min(mn2, kz); mx2 = max(mx2, kz);
    }
    mn0 = __reduce_min_sync(0xffffffffu, mn0);
    mn1 = __reduce_min_sync(0xffffffffu, mn1);
    mn2 = __reduce_min_sync(0xffffffffu, mn2);
    mx0 = __reduce_max_sync(0xffffffffu, mx0);
    mx1 = __reduce_max_sync(0xffffffffu, mx1);
    mx2 = __reduce_max_sync(0xffffffffu, mx2);
    __shared__ unsigned red[8][6];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[w][0] = mn0; red[w][1] = mn1; red[w][2] = mn2;
        red[w][3] = mx0; red[w][4] = mx1; red[w][5] = mx2;
    }
    if (bad >= 0) set_status(s.ctrl, kStNonFinite, bad);
    __syncthreads();
    if (threadIdx.x < 6) {
        const int c = threadIdx.x;
        unsigned v = red[0][c];
        for (int j = 1; j < 8; ++j) v = c < 3 ? min(v, red[j][c]) : max(v, red[j][c]);
        if (c < 3) atomicMin(&s.ctrl->bbox_key[c], v);
        else atomicMax(&s.ctrl->bbox_key[c], v);
    }
}

// ---------------------------------------------------------------------------
// build: one block per chunk of one system (insert_body), one max-depth
// atomic per block.  Lock holders are always running threads, so no
// co-residency is needed.
// ---------------------------------------------------------------------------
template <class Geo, bool kRef>
__device__ __forceinline__ int build_chunk(const DevSim &s, int i0, int i1) {
    float box[6];
    load_box(s.ctrl, box);
    const Geo root_g = Geo::root(box);
    int local_max = 0;
    const long long cap = tree_spin_cap(s.ctrl);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int depth = insert_body<Geo, kRef>(s, root_g, i, cap);
        if (depth < 0) return -1;
        local_max = max(local_max, depth);
    }
    return local_max;
}

// the same from the top levels (insert_from_top)
__device__ __forceinline__ int build_chunk_top(const DevSim &s, const TopTables &top, int i0, int i1) {
    float box[6];
    load_box(s.ctrl, box);
    const GeoCube root_g = GeoCube::root(box);
    int local_max = 0;
    const long long cap = tree_spin_cap(s.ctrl);
    for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
        const int depth = insert_from_top(s, top, root_g, i, cap);
        if (depth < 0) return -1;
        local_max = max(local_max, depth);
    }
    return local_max;
}

// ---------------------------------------------------------------------------
// top levels of every cubic-root tree that has them (top_levels): region
// counts per chunk of bodies in shared-memory bins, then one block per tree
// creates its top cells (top_cells_block); the build then starts every
// insertion below them
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_batch_top_count(BatchTables t) {
    __shared__ int bins[1 << (3 * kBatchTopMaxLevels)];
    const int k = find_system(t.chunk_prefix, t.nsys, blockIdx.x);
    const SysDesc &d = t.sys[k];
    // block-uniform, before any barrier: only earlier kernels set the status
    if (d.top.levels == 0 || !system_live(d.v.ctrl) || read_status(d.v.ctrl)) return;
    const DevSim s = system_view(d);
    float box[6];
    load_box(s.ctrl, box);
    const int i0 = (blockIdx.x - d.chunk_begin) * d.chunk;
    top_count_range(s, d.top, GeoCube::root(box), i0, min(s.n, i0 + d.chunk), blockDim.x, bins);
}

static_assert((1 << (3 * kBatchTopMaxLevels)) <= 32 * 256, "top_cells_block: at most 32 regions a thread");
__global__ void __launch_bounds__(256) k_batch_top_cells(BatchTables t) {
    const SysDesc &d = t.sys[blockIdx.x];
    if (!d.active || d.kind != kSysBH || d.top.levels == 0 || !system_live(d.v.ctrl)) return;
    top_cells_block(system_view(d), d.top);
}

__global__ void __launch_bounds__(256) k_batch_build(BatchTables t) {
    const int k = find_system(t.chunk_prefix, t.nsys, blockIdx.x);
    const SysDesc &d = t.sys[k];
    const DevSim s = system_view(d);
    if (read_status(s.ctrl) || !system_live(s.ctrl)) return;
    const int i0 = (blockIdx.x - d.chunk_begin) * d.chunk;
    const int i1 = min(s.n, i0 + d.chunk);
    const int depth = d.p.tree_ref     ? build_chunk<RefBox, true>(s, i0, i1)
                      : d.top.levels ? build_chunk_top(s, d.top, i0, i1)
                                     : build_chunk<GeoCube, false>(s, i0, i1);
    if (depth < 0) return;
    const unsigned am = __activemask();
    const int wmax = __reduce_max_sync(am, depth);
    if ((threadIdx.x & 31) == __ffs(am) - 1) atomicMax(&s.ctrl->max_depth, wmax);
}

// ---------------------------------------------------------------------------
// used cells: after the build, every tree's allocated cells [bottom, root]
// are laid end to end (one exclusive scan over the systems, one block), so
// summarize and sort visit only cells that exist.  A tree whose step failed,
// or that has no steps left, contributes none.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_batch_used(BatchTables t) {
    __shared__ int warp_sum[kScanThreads / 32];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < t.nsys; base += kScanThreads) {
        const int k = base + threadIdx.x;
        int used = 0;
        if (k < t.nsys) {
            const SysDesc &d = t.sys[k];
            const Ctrl *c = d.v.ctrl;
            if (d.active && d.kind == kSysBH && system_live(c) && !read_status(c))
                used = d.v.n + d.v.cap - c->bottom + 1;
        }
        int incl = used;  // inclusive scan: warps, then warp totals
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) warp_sum[w] = incl;
        __syncthreads();
        if (w == 0) {
            int v = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += u;
            }
            warp_sum[lane] = v;  // inclusive over warps
        }
        __syncthreads();
        const int before = carry + (w > 0 ? warp_sum[w - 1] : 0) + incl - used;
        if (k < t.nsys) t.used_prefix[k] = before;
        __syncthreads();
        if (threadIdx.x == kScanThreads - 1) carry = before + used;
        __syncthreads();
    }
    if (threadIdx.x == 0) t.used_prefix[t.nsys] = carry;
}

// ---------------------------------------------------------------------------
// summarize: one allocated cell per thread over all trees
// ---------------------------------------------------------------------------
template <bool kQuad>
__global__ void __launch_bounds__(256) k_batch_summarize(BatchTables t) {
    const int total = t.used_prefix[t.nsys];
    const int stride = gridDim.x * blockDim.x;
    int k = 0, lo = 0, hi = 0;  // the system of the last x and its range (x only grows)
    int first = 0, par = 0;     // that system's first allocated cell and buffer parity, read once
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < total; x += stride) {
        if (x >= hi) {
            k = find_system(t.used_prefix, t.nsys, x);
            lo = t.used_prefix[k];
            hi = t.used_prefix[k + 1];
            first = t.sys[k].v.ctrl->bottom;
            par = system_parity(t.sys[k]);
        }
        summarize_from<kQuad>(system_view_par(t.sys[k], par), first + (x - lo));
    }
}

// ---------------------------------------------------------------------------
// sort: inside every tree the cells are visited from the root downward (a
// parent before its children); the grid is no larger than what is
// co-resident, so every bounded wait in sort_cell is for a cell another
// running thread handles in an earlier or the same round.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_batch_sort(BatchTables t) {
    const int total = t.used_prefix[t.nsys];
    const int stride = gridDim.x * blockDim.x;
    int k = 0, lo = 0, hi = 0;  // the system of the last x and its range (x only grows)
    bool skip = false;          // that system's status and wait limit, read once per system
    long long cap = 0;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < total; x += stride) {
        if (x >= hi) {
            k = find_system(t.used_prefix, t.nsys, x);
            lo = t.used_prefix[k];
            hi = t.used_prefix[k + 1];
            const Ctrl *c = t.sys[k].v.ctrl;
            skip = read_status(c) != 0;
            cap = tree_spin_cap(c);
        }
        if (skip) continue;
        const DevSim &s = t.sys[k].v;  // the sort reads no body buffer
        if (!sort_cell(s, s.n + s.cap - (x - lo), cap)) skip = true;
    }
}

// ---------------------------------------------------------------------------
// force: warps take groups from one batch-wide counter; a warp recomputes its
// thresholds whenever its next group belongs to another system.  A system
// whose step failed keeps its step-start state.
// ---------------------------------------------------------------------------
// Shared memory of one warp of the batched force kernel.  The block has a
// runtime number of warps (TreeShape::force_warps), so the warps' records are
// laid out one after another in dynamic shared memory.
template <bool kQuad>
struct BatchForceWarp {
    float dq[kMaxDepth];
    int stack[kStack];
    float4 bpm[8 * kBatch], cpm[8 * kBatch], cmeta[8 * kBatch], cqa[kQuad ? 8 * kBatch : 1];
    // the current system's buffers and parameters: the walk reads them from
    // shared memory where the single-system kernel reads its kernel
    // parameters, instead of holding them in registers
    DevSim view;
    StepParams par;
    // the current system, its first group and its mode (0 walk, 1 keep the
    // step-start state of a failed step, 2 inert): in shared memory, so
    // nothing of the outer loop stays live in registers during a walk
    int cur, begin, mode;
};
constexpr int kBatchForceMaxWarps = 8;

// Register budget: at most 48 a thread for the monopole walks (ten resident
// blocks of four warps) and 64 with quadrupoles; neither spills.
template <int kMethod, bool kComp, bool kQuad>
__global__ void __launch_bounds__(kBatchForceMaxWarps * 32, kQuad ? 4 : 5) k_batch_force(BatchTables t) {
    extern __shared__ __align__(16) unsigned char force_smem[];
    BatchForceWarp<kQuad> &me = reinterpret_cast<BatchForceWarp<kQuad> *>(force_smem)[threadIdx.x >> 5];
    float *const s_dq_w = me.dq;
    DevSim &s_view_w = me.view;
    StepParams &s_par_w = me.par;
    int &s_cur_w = me.cur, &s_begin_w = me.begin, &s_mode_w = me.mode;
    const int lane = threadIdx.x & 31;
    if (lane == 0) s_cur_w = -1;
    __syncwarp();
    while (true) {
        int gg = 0;
        if (lane == 0) gg = atomicAdd(t.work, 1);
        gg = __shfl_sync(0xffffffffu, gg, 0);
        if (gg >= t.groups) break;
        const int k = find_system(t.group_prefix, t.nsys, gg);
        if (k != s_cur_w) {
            __syncwarp();  // the previous system's view and thresholds are no longer read
            if (lane == 0) {
                const SysDesc &d = t.sys[k];
                const DevSim v = system_view(d);
                StepParams p = d.p;
                p.kdk_primed = v.ctrl->kdk_primed;
                s_view_w = v;
                s_par_w = p;
                int sk = 0;
                if (!system_live(v.ctrl)) {
                    sk = 2;
                } else if (read_status(v.ctrl)) {
                    sk = 1;
                } else if (v.ctrl->max_depth >= kMaxDepth) {
                    set_status(v.ctrl, kStDepth, v.ctrl->max_depth);
                    sk = 1;
                }
                float box[6];
                load_box(v.ctrl, box);
                make_thresholds(box, p.theta, p.eps, p.crit_ref, s_dq_w);
                s_cur_w = k;
                s_begin_w = d.group_begin;
                s_mode_w = sk;
            }
            __syncwarp();
        }
        const int g = gg - s_begin_w;
        const int mode = s_mode_w;
        const DevSim &s = s_view_w;
        if (mode == 2) continue;
        if (mode == 1) {  // keep the step-start state
            const int i = g * 32 + lane;
            if (i < s.n) s.body_next[i] = s.body_cur[i];
            continue;
        }
        const WarpStage ws{me.stack, me.bpm, me.cpm, me.cmeta, me.cqa};
        force_group<kMethod, kComp, false, kQuad>(s, s_par_w, s_dq_w, g, lane, ws);
    }
}

// ---------------------------------------------------------------------------
// direct: one block per kThreads*kI targets of one system; j-tiles of kTileB
// bodies staged by TMA bulk copies (double-buffered mbarriers); Plummer
// softening; fused integrator.  kI, kThreads and kTileB come from the
// autotuner.
// ---------------------------------------------------------------------------
template <int kI, int kThreads, int kTileB>
__global__ void __launch_bounds__(kThreads) k_batch_direct(BatchTables t) {
    __shared__ __align__(128) float4 tile[2][kTileB];
    __shared__ __align__(8) uint64_t bar[2];
    const int k = find_system(t.dblock_prefix, t.nsys, blockIdx.x);
    const SysDesc &d = t.sys[k];
    if (!system_live(d.v.ctrl)) return;  // block-uniform, before any barrier
    const DevSim s = system_view(d);
    StepParams p = d.p;
    p.kdk_primed = s.ctrl->kdk_primed;
    const int n = s.n;
    const int base = (blockIdx.x - d.dblock_begin) * (kThreads * kI);
    const float eps2 = p.eps * p.eps;
    int idx[kI];
    float4 me[kI];
    float ax[kI], ay[kI], az[kI];
#pragma unroll
    for (int r = 0; r < kI; ++r) {
        idx[r] = base + r * kThreads + threadIdx.x;
        me[r] = idx[r] < n ? s.body_cur[idx[r]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        ax[r] = ay[r] = az[r] = 0.0f;
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int ntiles = (n + kTileB - 1) / kTileB;
    auto issue = [&](int tt, int stage) {
        const int cnt = min(kTileB, n - tt * kTileB);
        const uint32_t bytes = (uint32_t)cnt * 16u;
        mbar_expect_tx(&bar[stage], bytes);
        bulk_g2s(&tile[stage][0], s.body_cur + (size_t)tt * kTileB, bytes, &bar[stage]);
    };
    if (threadIdx.x == 0 && ntiles > 0) issue(0, 0);
    bool ok = true;
    for (int tt = 0; tt < ntiles; ++tt) {
        const int stage = tt & 1;
        if (threadIdx.x == 0 && tt + 1 < ntiles) issue(tt + 1, stage ^ 1);
        if (!mbar_wait_bounded(&bar[stage], (uint32_t)((tt >> 1) & 1), s.ctrl)) ok = false;
        const int cnt = min(kTileB, n - tt * kTileB);
        const float4 *tl = tile[stage];
#pragma unroll 4
        for (int j = 0; j < cnt; ++j) {
            const float4 q = tl[j];
#pragma unroll
            for (int r = 0; r < kI; ++r) {
                const float dx = q.x - me[r].x, dy = q.y - me[r].y, dz = q.z - me[r].z;
                const float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                const float rr = rsqrt_fast(d2);
                const float F = (q.w * rr) * (rr * rr);
                ax[r] = fmaf(dx, F, ax[r]);
                ay[r] = fmaf(dy, F, ay[r]);
                az[r] = fmaf(dz, F, az[r]);
            }
        }
        if (!__syncthreads_and(ok)) {
            if (threadIdx.x == 0 && tt + 1 < ntiles)
                mbar_wait_bounded(&bar[stage ^ 1], (uint32_t)(((tt + 1) >> 1) & 1), s.ctrl);
            ok = false;
            break;
        }
    }
#pragma unroll
    for (int r = 0; r < kI; ++r) {
        if (idx[r] >= n) continue;
        if (!ok) {
            s.body_next[idx[r]] = me[r];
            continue;
        }
        const float gx = ax[r] * p.G, gy = ay[r] * p.G, gz = az[r] * p.G;
        switch (p.method) {
        case 1: integrate_body<1>(s, p, idx[r], me[r], gx, gy, gz); break;
        case 2: integrate_body<2>(s, p, idx[r], me[r], gx, gy, gz); break;
        case 3: integrate_body<3>(s, p, idx[r], me[r], gx, gy, gz); break;
        default: integrate_body<0>(s, p, idx[r], me[r], gx, gy, gz); break;
        }
    }
}

// ---------------------------------------------------------------------------
// flip: the next buffer becomes current; KDK systems are primed; one step
// of the system's budget is used
// ---------------------------------------------------------------------------
__global__ void k_batch_flip(BatchTables t) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t.nsys) return;
    const SysDesc &d = t.sys[k];
    if (!d.active) return;
    Ctrl *c = d.v.ctrl;
    const int budget = c->budget;
    if (budget == 0) return;
    c->parity ^= 1;
    if (d.p.method == 3) c->kdk_primed = 1;
    if (budget > 0) c->budget = budget - 1;
}

// ---------------------------------------------------------------------------
// collision update of every system that asks for it (update_collision_local,
// kernels/collision_update.cl:17-83): one block per kCollideBlockBodies
// targets of one system (a tree system's in the order of its sort), the
// block form of the standalone kernel
// (collide_device.cuh), after the force and direct stages have integrated
// and before the flip (src/MyApp.cpp:593-596,606-610,622-625).  Systems with
// no steps left or a failed step are skipped.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kCollideThreads) k_batch_collision(BatchTables t) {
    const int k = find_system(t.cblock_prefix, t.nsys, blockIdx.x);
    const SysDesc &d = t.sys[k];
    if (!system_live(d.v.ctrl) || read_status(d.v.ctrl)) return;  // block-uniform, before any barrier
    const DevSim s = system_view(d);
    collide_block(s.body_next, s.vel, d.kind == kSysBH ? s.sorted : nullptr, s.n,
                  (blockIdx.x - d.cblock_begin) * kCollideThreads, s.ctrl);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int resident(const void *fn, int threads, int sm_count) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * sm_count;
}

// Direct-sum variants the autotuner chooses from: {bodies per thread,
// threads per block, j-tile bodies}.
struct DirectVariant {
    int ki, threads, tile;
};
static const DirectVariant kDirectVariants[] = {{1, 128, 128}, {1, 128, 256}, {1, 256, 256}, {2, 128, 128},
                                                {2, 128, 256}, {2, 256, 256}, {4, 128, 256}, {4, 256, 256},
                                                {1, 64, 256},  {2, 64, 256},  {4, 64, 256}};
constexpr int kNumDirectVariants = sizeof(kDirectVariants) / sizeof(kDirectVariants[0]);

int batch_direct_variants() { return kNumDirectVariants; }
int batch_direct_block_bodies(int variant) {
    const DirectVariant &v = kDirectVariants[variant];
    return v.ki * v.threads;
}

static cudaError_t launch_direct_variant(const BatchTables &t, int variant, cudaStream_t st) {
    const int b = t.dblocks;
    switch (variant) {
    case 0: k_batch_direct<1, 128, 128><<<b, 128, 0, st>>>(t); break;
    case 1: k_batch_direct<1, 128, 256><<<b, 128, 0, st>>>(t); break;
    case 2: k_batch_direct<1, 256, 256><<<b, 256, 0, st>>>(t); break;
    case 3: k_batch_direct<2, 128, 128><<<b, 128, 0, st>>>(t); break;
    case 4: k_batch_direct<2, 128, 256><<<b, 128, 0, st>>>(t); break;
    case 5: k_batch_direct<2, 256, 256><<<b, 256, 0, st>>>(t); break;
    case 6: k_batch_direct<4, 128, 256><<<b, 128, 0, st>>>(t); break;
    case 7: k_batch_direct<4, 256, 256><<<b, 256, 0, st>>>(t); break;
    case 8: k_batch_direct<1, 64, 256><<<b, 64, 0, st>>>(t); break;
    case 9: k_batch_direct<2, 64, 256><<<b, 64, 0, st>>>(t); break;
    default: k_batch_direct<4, 64, 256><<<b, 64, 0, st>>>(t); break;
    }
    return cudaGetLastError();
}

template <int kMethod, bool kComp, bool kQuad>
static cudaError_t launch_batch_force_t(const BatchTables &t, const TreeShape &shape, int sm_count,
                                        cudaStream_t st) {
    int warps = shape.force_warps;
    if (warps < 1 || warps > kBatchForceMaxWarps) warps = kForceWarps;
    const int threads = warps * 32;
    const size_t smem = sizeof(BatchForceWarp<kQuad>) * (size_t)warps;
    const void *fn = (const void *)k_batch_force<kMethod, kComp, kQuad>;
    if (smem > 48 * 1024) {  // beyond the default dynamic shared memory of a block: opt in
        const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    long long blocks = (long long)per_sm * sm_count * (shape.force_grid_pct > 0 ? shape.force_grid_pct : 100) / 100;
    const int need = (t.groups + warps - 1) / warps;
    if (blocks > need) blocks = need;
    if (blocks < 1) blocks = 1;
    k_batch_force<kMethod, kComp, kQuad><<<(int)blocks, threads, smem, st>>>(t);
    return cudaGetLastError();
}

template <int kMethod>
static cudaError_t launch_batch_force_m(const BatchTables &t, int comp, int quad, const TreeShape &shape,
                                        int sm_count, cudaStream_t st) {
    if (quad) return comp ? launch_batch_force_t<kMethod, true, true>(t, shape, sm_count, st)
                          : launch_batch_force_t<kMethod, false, true>(t, shape, sm_count, st);
    return comp ? launch_batch_force_t<kMethod, true, false>(t, shape, sm_count, st)
                : launch_batch_force_t<kMethod, false, false>(t, shape, sm_count, st);
}

// bbox .. force of every tree system; *launches gets the kernel count
static cudaError_t launch_batch_tree_stages(const BatchTables &t, int method, int comp, int quad,
                                            const TreeShape &shape, int sm_count, cudaStream_t st,
                                            const StepFork *fork, bool branch, int *launches) {
    cudaError_t e = cudaSuccess;
    const int sb = (t.nsys + 127) / 128;
    k_batch_reset<<<sb, 128, 0, st>>>(t);
    k_batch_bbox<<<t.chunks, 256, 0, st>>>(t);
    k_batch_top_count<<<t.chunks, 256, 0, st>>>(t);
    k_batch_top_cells<<<t.nsys, 256, 0, st>>>(t);
    k_batch_build<<<t.chunks, 256, 0, st>>>(t);
    k_batch_used<<<1, kScanThreads, 0, st>>>(t);
    // many blocks, so the grid-stride tail is short (512 systems: 8 per SM
    // 4.79 ms, 32 per SM 2.90 ms)
    int sblocks = sm_count * 32;
    const int need = (t.cells + 255) / 256;
    if (sblocks > need) sblocks = need;
    if (quad) k_batch_summarize<true><<<sblocks, 256, 0, st>>>(t);
    else k_batch_summarize<false><<<sblocks, 256, 0, st>>>(t);
    if (branch && (e = cudaStreamWaitEvent(st, fork->join, 0)) != cudaSuccess) return e;
    int rblocks = resident((const void *)k_batch_sort, 256, sm_count);
    if (rblocks > need) rblocks = need;
    k_batch_sort<<<rblocks, 256, 0, st>>>(t);
    if ((e = cudaMemsetAsync(t.work, 0, sizeof(int), st)) != cudaSuccess) return e;
    switch (method) {
    case 1: e = launch_batch_force_m<1>(t, comp, quad, shape, sm_count, st); break;
    case 2: e = launch_batch_force_m<2>(t, comp, quad, shape, sm_count, st); break;
    case 3: e = launch_batch_force_m<3>(t, comp, quad, shape, sm_count, st); break;
    default: e = launch_batch_force_m<0>(t, comp, quad, shape, sm_count, st); break;
    }
    if (launches) *launches = 9;
    return e;
}



// One batched step.  Kernels with no work in this batch are not launched.
// Returns the number of kernels launched through *launches.
cudaError_t launch_batch_step(const BatchTables &t, int method, int comp, int quad, int direct_variant,
                              const TreeShape &shape, int sm_count, cudaStream_t st, const StepFork *fork,
                              int *launches, bool advance) {
    int nl = 0;
    cudaError_t e = cudaSuccess;
    const int sb = (t.nsys + 127) / 128;
    const bool branch = fork && fork->aux && t.chunks > 0 && t.dblocks > 0;
    if (branch) {  // the direct sum beside the tree stages
        if ((e = cudaEventRecord(fork->fork, st)) != cudaSuccess ||
            (e = cudaStreamWaitEvent(fork->aux, fork->fork, 0)) != cudaSuccess ||
            (e = launch_direct_variant(t, direct_variant, fork->aux)) != cudaSuccess ||
            (e = cudaEventRecord(fork->join, fork->aux)) != cudaSuccess)
            return e;
        nl += 1;
    }
    if (t.chunks > 0) {
        int tl = 0;
        if ((e = launch_batch_tree_stages(t, method, comp, quad, shape, sm_count, st, fork, branch, &tl)) !=
            cudaSuccess)
            return e;
        nl += tl;
    }
    if (t.dblocks > 0 && !branch) {
        if ((e = launch_direct_variant(t, direct_variant, st)) != cudaSuccess) return e;
        nl += 1;
    }
    if (!advance) {
        if (launches) *launches = nl;
        return cudaGetLastError();
    }
    if (t.cblocks > 0) {
        k_batch_collision<<<t.cblocks, kCollideThreads, 0, st>>>(t);
        nl += 1;
    }
    k_batch_flip<<<sb, 128, 0, st>>>(t);
    nl += 1;
    if (launches) *launches = nl;
    return cudaGetLastError();
}

__global__ void k_batch_clear(BatchTables t) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t.nsys) return;
    Ctrl *c = t.sys[k].v.ctrl;
    c->status = 0;
    c->status_info = 0;
    c->interactions = 0;
    c->opened = 0;
    c->cell_interactions = 0;
}

cudaError_t launch_batch_clear(const BatchTables &t, cudaStream_t st) {
    k_batch_clear<<<(t.nsys + 127) / 128, 128, 0, st>>>(t);
    return cudaGetLastError();
}

}  // namespace nbgb
