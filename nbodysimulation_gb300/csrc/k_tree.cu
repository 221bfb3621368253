// k_tree.cu -- bounding box, octree build, centre-of-mass summarisation and
// in-order sort of the Barnes-Hut step.
//
// Reference stages: boundary_reduce (kernels/boundary_reduce.cl), init
// (kernels/init.cl), build_tree (kernels/build_tree.cl, build_tree.hcl),
// saturate_tree (kernels/saturate_tree.cl) and the empty sort
// (kernels/sort.cl).  Each is re-designed for sm_103a; the differences that
// change results are listed at each kernel.
#include <algorithm>

#include "bh_device.cuh"

namespace nbgb {

// ---------------------------------------------------------------------------
// reset: the per-step part of init (kernels/init.cl:26-33).  The reference
// also rewrites every child slot of every node (init.cl:17-19, 32 B per node
// and step); here a cell's eight slots are cleared by the thread that
// allocates it, so only the root needs it.  The status word is cleared by the
// host once per nb_step call, so an error stays visible to the later steps.
// ---------------------------------------------------------------------------
__global__ void k_reset(DevSim s) {
    Ctrl *c = s.ctrl;
    const int t = threadIdx.x;
    if (t < 3) c->bbox_key[t] = 0xFFFFFFFFu;
    else if (t < 6) c->bbox_key[t] = 0u;
    if (t < 8) s.child[s.cap * 8 + t] = kEmpty;
    if (t == 0) {
        c->bottom = s.n + s.cap;
        c->max_depth = 0;
        c->work = 0;
        s.arrive[s.cap] = 0;
        s.start[s.cap] = 0;
        s.count[s.cap] = 0;
        s.parent[s.cap] = -1;
    }
}

// ---------------------------------------------------------------------------
// bbox: exact component-wise min/max over all bodies.  The reference's
// two-kernel reduction samples only 2*WG bodies as wired (the host passes
// the position buffer to parallel_reduce_root, src/MyApp.cpp:282); this is
// the true reduction.  Floats are reduced as order-preserving integer keys
// (IMNMX, exact, -0 < +0), warp shuffles, then one atomic per component per
// block.  HBM-bound: 16 B read per body.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bbox(const float4 *__restrict__ b, int n, Ctrl *c) {
    unsigned mn0 = 0xFFFFFFFFu, mn1 = 0xFFFFFFFFu, mn2 = 0xFFFFFFFFu, mx0 = 0u, mx1 = 0u, mx2 = 0u;
    int bad = -1;
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float4 p = __ldg(&b[i]);
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
    if (bad >= 0) set_status(c, kStNonFinite, bad);
    __syncthreads();
    if (threadIdx.x < 6) {
        const int k = threadIdx.x;
        unsigned v = red[0][k];
        const int nw = blockDim.x >> 5;
        for (int j = 1; j < nw; ++j) v = k < 3 ? min(v, red[j][k]) : max(v, red[j][k]);
        if (k < 3) atomicMin(&c->bbox_key[k], v);
        else atomicMax(&c->bbox_key[k], v);
    }
}

// ---------------------------------------------------------------------------
// build: one body per thread, grid-stride (insert_body, bh_device.cuh).
// ---------------------------------------------------------------------------
template <class Geo, bool kRef>
__global__ void __launch_bounds__(256) k_build(DevSim s) {
    Ctrl *ctrl = s.ctrl;
    if (read_status(ctrl)) return;
    float box[6];
    load_box(ctrl, box);
    const Geo root_g = Geo::root(box);
    int local_max = 0;
    const long long cap = tree_spin_cap(ctrl);
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += stride) {
        const int depth = insert_body<Geo, kRef>(s, root_g, i, cap);
        if (depth < 0) return;
        local_max = max(local_max, depth);
    }
    const unsigned am = __activemask();
    const int wmax = __reduce_max_sync(am, local_max);
    if ((threadIdx.x & 31) == __ffs(am) - 1) atomicMax(&ctrl->max_depth, wmax);
}

// ---------------------------------------------------------------------------
// top levels (cubic-root tree): count, cells, then the build from them.
// ---------------------------------------------------------------------------
// Counts per block in shared memory (8^L bins, dynamic), then one global
// atomic per non-empty bin: regions of a dense centre hold tens of thousands
// of bodies, which one global counter each would serialise.
constexpr int kTopCountThreads = 1024;
__global__ void __launch_bounds__(kTopCountThreads) k_top_count(DevSim s, TopTables t) {
    extern __shared__ int bins[];
    Ctrl *ctrl = s.ctrl;
    if (read_status(ctrl)) return;  // block-uniform, before any barrier
    float box[6];
    load_box(ctrl, box);
    top_count_range(s, t, GeoCube::root(box), blockIdx.x * blockDim.x, s.n, gridDim.x * blockDim.x, bins);
}

constexpr int kTopCellsThreads = 1024;
static_assert((1 << (3 * kTopMaxLevels)) <= 32 * kTopCellsThreads, "top_cells_block: at most 32 regions a thread");
// levels 1..L-1 in one block, then level L (most of the cells) over a grid
__global__ void __launch_bounds__(kTopCellsThreads) k_top_cells(DevSim s, TopTables t) {
    top_cells_block(s, t, t.deep);
}

__global__ void __launch_bounds__(256) k_top_leaf(DevSim s, TopTables t) {
    top_leaf_cells(s, t, t.deep, blockIdx.x * blockDim.x + threadIdx.x);
}

// build from the top levels, one body per thread, grid-stride
__global__ void __launch_bounds__(256) k_build_top(DevSim s, TopTables t) {
    Ctrl *ctrl = s.ctrl;
    if (read_status(ctrl)) return;
    float box[6];
    load_box(ctrl, box);
    const GeoCube root_g = GeoCube::root(box);
    int local_max = 0;
    const long long cap = tree_spin_cap(ctrl);
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += stride) {
        const int depth = insert_from_top(s, t, root_g, i, cap);
        if (depth < 0) return;
        local_max = max(local_max, depth);
    }
    const unsigned am = __activemask();
    const int wmax = __reduce_max_sync(am, local_max);
    if ((threadIdx.x & 31) == __ffs(am) - 1) atomicMax(&ctrl->max_depth, wmax);
}

// ---------------------------------------------------------------------------
// summarize: one cell of [bottom, root] per thread (summarize_from).
// ---------------------------------------------------------------------------
template <bool kQuad>
__global__ void __launch_bounds__(256) k_summarize(DevSim s) {
    if (read_status(s.ctrl)) return;
    const int root = s.n + s.cap;
    const int bottom = s.ctrl->bottom;
    const int stride = gridDim.x * blockDim.x;
    for (int k = bottom + (int)(blockIdx.x * blockDim.x + threadIdx.x); k <= root; k += stride)
        summarize_from<kQuad>(s, k);
}

// ---------------------------------------------------------------------------
// sort: cells visited from the root downward (descending index: a parent was
// allocated before its children), so every wait in sort_cell is for a cell
// handled earlier; launched on a grid no larger than what is co-resident.
// The result is the depth-first listing of bodies in slot order, which the
// oracle's orc_sort reproduces exactly.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_sort(DevSim s) {
    Ctrl *ctrl = s.ctrl;
    if (read_status(ctrl)) return;
    const int root = s.n + s.cap;
    const int bottom = ctrl->bottom;
    const long long cap = tree_spin_cap(ctrl);
    const int stride = gridDim.x * blockDim.x;
    for (int k = root - (int)(blockIdx.x * blockDim.x + threadIdx.x); k >= bottom; k -= stride)
        if (!sort_cell(s, k, cap)) return;
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int resident_blocks(const void *fn, int threads, int sm_count) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * sm_count;
}

cudaError_t launch_reset(const DevSim &s, cudaStream_t st) {
    k_reset<<<1, 32, 0, st>>>(s);
    return cudaGetLastError();
}

cudaError_t launch_bbox(const DevSim &s, int sm_count, cudaStream_t st) {
    int blocks = sm_count * 4;
    const int need = (s.n + 255) / 256;
    if (blocks > need) blocks = need > 0 ? need : 1;
    k_bbox<<<blocks, 256, 0, st>>>(s.body_cur, s.n, s.ctrl);
    return cudaGetLastError();
}

cudaError_t launch_build(const DevSim &s, const TopTables &top, int tree_ref, int sm_count, cudaStream_t st,
                         int *launches) {
    const int need = (s.n + 255) / 256;
    if (!tree_ref && top.levels >= 2 && top.levels <= kTopMaxLevels) {
        const size_t bins_bytes = sizeof(int) << (3 * top.levels);
        if (bins_bytes > 48 * 1024) {  // the 8^5-bin table needs the opt-in shared memory size (current device)
            const cudaError_t e = cudaFuncSetAttribute(k_top_count, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       (int)bins_bytes);
            if (e != cudaSuccess) return e;
        }
        const int cblocks = std::max(1, std::min(sm_count, (s.n + kTopCountThreads - 1) / kTopCountThreads));
        k_top_count<<<cblocks, kTopCountThreads, bins_bytes, st>>>(s, top);
        k_top_cells<<<1, kTopCellsThreads, 0, st>>>(s, top);  // all levels in the block when top.deep is null
        if (top.deep) k_top_leaf<<<((1 << (3 * top.levels)) + 255) / 256, 256, 0, st>>>(s, top);
        // two blocks per SM, as for the build from the root (262k-body ball:
        // 0.12 ms against 0.14 ms on the whole co-resident grid; 4M: equal)
        int blocks = std::min(resident_blocks((const void *)k_build_top, 256, sm_count), 2 * sm_count);
        if (blocks > need) blocks = need > 0 ? need : 1;
        k_build_top<<<blocks, 256, 0, st>>>(s, top);
        *launches = top.deep ? 4 : 3;
        return cudaGetLastError();
    }
    *launches = 1;
    const void *fn = tree_ref ? (const void *)k_build<RefBox, true> : (const void *)k_build<GeoCube, false>;
    // two blocks per SM: threads that start at the root together contend for
    // its first cells, and fewer of them insert faster (measured build time
    // with 1 / 2 / 4 / 8 blocks per SM: 262k-body ball 0.20 / 0.20 / 0.30 /
    // 0.32 ms, 1M 0.60 / 0.41 / 0.49 / 0.54 ms, 4M 2.25 / 1.26 / 1.24 / 1.32 ms)
    int blocks = std::min(resident_blocks(fn, 256, sm_count), 2 * sm_count);
    if (blocks > need) blocks = need > 0 ? need : 1;
    if (tree_ref) k_build<RefBox, true><<<blocks, 256, 0, st>>>(s);
    else k_build<GeoCube, false><<<blocks, 256, 0, st>>>(s);
    return cudaGetLastError();
}

cudaError_t launch_summarize(const DevSim &s, int quadrupole, int sm_count, cudaStream_t st) {
    // many blocks: a cell's cost varies (the last arriver climbs), so a long
    // grid-stride tail hurts (4M, quadrupoles: 8 per SM 0.70 ms, 32 per SM 0.65)
    int blocks = sm_count * 32;
    const int need = (s.cap + 1 + 255) / 256;
    if (blocks > need) blocks = need > 0 ? need : 1;
    if (quadrupole) k_summarize<true><<<blocks, 256, 0, st>>>(s);
    else k_summarize<false><<<blocks, 256, 0, st>>>(s);
    return cudaGetLastError();
}

cudaError_t launch_sort(const DevSim &s, int sm_count, cudaStream_t st) {
    int blocks = resident_blocks((const void *)k_sort, 256, sm_count);
    const int need = (s.cap + 1 + 255) / 256;
    if (blocks > need) blocks = need;
    k_sort<<<blocks, 256, 0, st>>>(s);
    return cudaGetLastError();
}

}  // namespace nbgb
