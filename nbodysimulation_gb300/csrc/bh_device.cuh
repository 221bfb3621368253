// bh_device.cuh -- the per-item work of the Barnes-Hut stages as device
// functions, shared by the single-system kernels (k_tree.cu, k_force.cu)
// and the batched kernels that walk a table of systems (k_batch.cu).
//
// Reference stages: build_tree (kernels/build_tree.cl, build_tree.hcl),
// saturate_tree (kernels/saturate_tree.cl), the empty sort
// (kernels/sort.cl) and calculate_force_local (kernels/calculate_forces.cl).
#pragma once
#include <cooperative_groups.h>

#include "nbgb_internal.cuh"

namespace nbgb {

namespace bh_cg = cooperative_groups;

// ---------------------------------------------------------------------------
// Geometry of the build.  Both policies keep `g` = the region of the slot the
// body is about to enter, so the split can give a new cell that region.
// ---------------------------------------------------------------------------
struct GeoCube {  // Burtscher: cubic root, child centre = centre -/+ r/2
    float cx, cy, cz, r;
    __device__ __forceinline__ int octant(float x, float y, float z) const {
        return (y < cy ? 4 : 0) + (x < cx ? 2 : 0) + (z < cz ? 1 : 0);
    }
    __device__ __forceinline__ void descend(float x, float y, float z) {
        r = __fmul_rn(r, 0.5f);
        cx = __fadd_rn(cx, x < cx ? -r : r);
        cy = __fadd_rn(cy, y < cy ? -r : r);
        cz = __fadd_rn(cz, z < cz ? -r : r);
    }
    __device__ static GeoCube root(const float box[6]) {
        const float ex = box[3] - box[0], ey = box[4] - box[1], ez = box[5] - box[2];
        float m = ex > ey ? ex : ey;
        m = m > ez ? m : ez;
        return GeoCube{__fmul_rn(__fadd_rn(box[0], box[3]), 0.5f), __fmul_rn(__fadd_rn(box[1], box[4]), 0.5f),
                       __fmul_rn(__fadd_rn(box[2], box[5]), 0.5f), __fmul_rn(0.5f, m)};
    }
};

struct RefBox {  // the reference: calculateOctantIdx / adjustBoundaryValues
    float mnx, mny, mnz, mxx, mxy, mxz;
    // build_tree.hcl:14-29 -- 4*(dy<0) + 2*(dx<0) + (dz<0), centre (max+min)/2
    __device__ __forceinline__ int octant(float x, float y, float z) const {
        const float cx = __fmul_rn(__fadd_rn(mxx, mnx), 0.5f);
        const float cy = __fmul_rn(__fadd_rn(mxy, mny), 0.5f);
        const float cz = __fmul_rn(__fadd_rn(mxz, mnz), 0.5f);
        return (y < cy ? 4 : 0) + (x < cx ? 2 : 0) + (z < cz ? 1 : 0);
    }
    // build_tree.hcl:31-54, y bounds following the x difference (:42-46)
    __device__ __forceinline__ void descend(float x, float y, float z) {
        const float cx = __fmul_rn(__fadd_rn(mxx, mnx), 0.5f);
        const float cy = __fmul_rn(__fadd_rn(mxy, mny), 0.5f);
        const float cz = __fmul_rn(__fadd_rn(mxz, mnz), 0.5f);
        if (x > cx) mnx = cx; else mxx = cx;
        if (x > cx) mny = cy; else mxy = cy;
        if (z > cz) mnz = cz; else mxz = cz;
        (void)y;
    }
    __device__ static RefBox root(const float box[6]) { return RefBox{box[0], box[1], box[2], box[3], box[4], box[5]}; }
};

// ---------------------------------------------------------------------------
// Octree insertion of body i (Burtscher; kernels/build_tree.cl:42-161).
// Empty slot: CAS(-1 -> body).  Slot holding a body: CAS(body -> LOCKED),
// grow a chain of cells until the two bodies separate, publish the chain with
// one release store of its top cell.  Cells come from the system's downward
// counter with warp-aggregated atomicSub (one atomic per converged group of
// splitting threads).  A fresh cell's eight slots, parent link, arrival
// counter and sort start are set by the allocating thread before
// publication.  Retries are bounded (tree_spin_cap) and watch the status word; a
// cell overflow or an over-deep chain restores the locked slot and records
// the status.  Returns the body's depth, or -1 when the build must stop.
//
// Reference semantics (kRef): the first probe is slot 0 of the super-root
// without an octant test (build_tree.cl:57-65); the root region is the
// bounding box; boxes halve as adjustBoundaryValues does.
//
// insert_from is the insertion loop: body i (position P) enters slot `slot`
// of published cell `node` at depth `depth`; g is already that slot's region.
// insert_body starts it at the root.
// ---------------------------------------------------------------------------
template <class Geo>
__device__ __forceinline__ int insert_from(const DevSim &s, Geo g, int node, int slot, int depth, const float4 P,
                                           int i, long long spin_cap) {
    Ctrl *ctrl = s.ctrl;
    const int n = s.n;
    int *cslot = &s.child[(node - n) * 8 + slot];
    int ch = ld_volatile(cslot);
    long long spins = 0;
    unsigned pause = 32;
    while (true) {
        while (ch >= n) {  // descend through published cells
            node = ch;
            slot = g.octant(P.x, P.y, P.z);
            g.descend(P.x, P.y, P.z);
            ++depth;
            cslot = &s.child[(node - n) * 8 + slot];
            ch = ld_volatile(cslot);
        }
        if (ch == kEmpty) {
            if (atomicCAS(cslot, kEmpty, i) == kEmpty) return depth;
        } else if (ch >= 0) {
            if (atomicCAS(cslot, ch, kLocked) == ch) {
                const int og = ch;
                const float4 O = s.body_cur[og];
                Geo og_g = g;
                int patch = -1, link_node = node, link_slot = slot, c2;
                int fail = 0;
                do {
                    bh_cg::coalesced_group grp = bh_cg::coalesced_threads();
                    int base = 0;
                    if (grp.thread_rank() == 0) base = atomicSub(&ctrl->bottom, (int)grp.size());
                    base = grp.shfl(base, 0);
                    const int cell = base - 1 - (int)grp.thread_rank();
                    ++depth;
                    if (cell < n) { fail = kStCellOverflow; break; }
                    if (depth > 2 * kMaxDepth) { fail = kStDepth; break; }
                    patch = max(patch, cell);
                    const int c = cell - n;
                    int4 *row = reinterpret_cast<int4 *>(&s.child[c * 8]);
                    row[0] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
                    row[1] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
                    s.parent[c] = link_node;
                    s.arrive[c] = 0;
                    s.start[c] = -1;
                    if (patch != cell) s.child[(link_node - n) * 8 + link_slot] = cell;
                    const int oslot = og_g.octant(O.x, O.y, O.z);
                    og_g.descend(O.x, O.y, O.z);
                    s.child[c * 8 + oslot] = og;
                    slot = g.octant(P.x, P.y, P.z);
                    g.descend(P.x, P.y, P.z);
                    link_node = cell;
                    link_slot = slot;
                    c2 = (slot == oslot) ? og : kEmpty;
                } while (c2 >= 0);
                if (fail) {
                    st_volatile(cslot, og);  // release the lock unchanged
                    set_status(ctrl, fail, i);
                    return -1;
                }
                s.child[(link_node - n) * 8 + link_slot] = i;
                __threadfence();
                st_volatile(cslot, patch);  // publish the chain
                return depth;
            }
        }
        if (++spins > spin_cap) {
            set_status(ctrl, kStSpinTimeout, i);
            return -1;
        }
        if ((spins & 1023) == 0 && read_status(ctrl)) return -1;
        if (ch == kLocked) {  // another thread is splitting this slot: back off
            __nanosleep(pause);
            if (pause < 2048) pause <<= 1;
        }
        ch = ld_volatile(cslot);
    }
}

template <class Geo, bool kRef>
__device__ __forceinline__ int insert_body(const DevSim &s, const Geo &root_g, int i, long long spin_cap) {
    const float4 P = s.body_cur[i];
    Geo g = root_g;
    int slot = 0;
    if constexpr (!kRef) {
        slot = g.octant(P.x, P.y, P.z);
        g.descend(P.x, P.y, P.z);
    }
    return insert_from<Geo>(s, g, s.n + s.cap, slot, 0, P, i, spin_cap);
}

// ---------------------------------------------------------------------------
// Top levels of the cubic-root tree, built before the insertions.  The cell
// of a region exists in the insertion tree exactly when the region holds at
// least two bodies, so counting the bodies of every region of level L (8^L
// regions, the same octant() / descend() steps as an insertion) gives every
// cell of levels 1..L.  Those cells are allocated level by level (a parent
// gets a higher index than its children, as in the insertions) and published
// before the build; each body then starts its insertion at the deepest
// existing cell of its level-L path.  The tree, its depth and its cell count
// are the ones the insertions alone give; only the cell numbering differs.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int top_region(GeoCube g, const float4 P, int levels) {
    int id = 0;
    for (int l = 0; l < levels; ++l) {
        id = id * 8 + g.octant(P.x, P.y, P.z);
        g.descend(P.x, P.y, P.z);
    }
    return id;
}

// first region of level l (>= 1) in a table of the regions of levels 1..4
__device__ __forceinline__ int top_offset(int l) { return ((1 << (3 * l)) - 8) / 7; }

// Exclusive prefix sum of v over the block (blockDim.x a multiple of 32,
// at most 1024); *total gets the sum.  Every thread of the block calls it.
__device__ __forceinline__ int block_exclusive_sum(int v, int *warp_tot, int *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        int x = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += u;
        }
        if (lane < nw) warp_tot[lane] = x;  // inclusive over warps
    }
    __syncthreads();
    const int before = (w > 0 ? warp_tot[w - 1] : 0) + incl - v;
    *total = warp_tot[nw - 1];
    __syncthreads();  // warp_tot is reused by the next call
    return before;
}

// Level-L region counts of bodies [i0 + threadIdx.x, i1) with stride `stride`
// into the block's shared bins (8^L ints), then one global atomic per
// non-empty bin.  Every thread of the block calls it.
__device__ __forceinline__ void top_count_range(const DevSim &s, const TopTables &t, const GeoCube &root_g, int i0,
                                                int i1, int stride, int *bins) {
    const int nbins = 1 << (3 * t.levels);
    for (int r = threadIdx.x; r < nbins; r += blockDim.x) bins[r] = 0;
    __syncthreads();
    for (int i = i0 + threadIdx.x; i < i1; i += stride)
        atomicAdd(&bins[top_region(root_g, __ldg(&s.body_cur[i]), t.levels)], 1);
    __syncthreads();
    for (int r = threadIdx.x; r < nbins; r += blockDim.x)
        if (bins[r]) atomicAdd(&t.count[r], bins[r]);
}

// One block: region counts of levels L-1..1 from the level-L counts, then
// the cells of levels 1..L top down (each level's cells numbered below the
// previous level's), then the start entry of every level-L region.  Clears
// the level-L counts for the next step in every case.  With deep_out, the
// block stops after level L-1 and leaves that level's entries in deep_out
// (8^(L-1) ints) and the counts in place for top_leaf_cells.  Every thread of
// the block calls it; blockDim.x is a power of two with 8^L <= 32 *
// blockDim.x, so a thread takes at most 32 regions of a level and a level has
// at most kTopRegions / 32 (round, warp) pairs.
__device__ __forceinline__ void top_cells_block(const DevSim &s, const TopTables &t, int *deep_out = nullptr) {
    __shared__ int cnt_sh[kTopInner];   // body counts, regions of levels 1..L-1
    __shared__ int deep_sh[kTopInner];  // (level << 26) | deepest existing cell of the region's path
    __shared__ int rank_sh[kTopRegions / 32];  // per (round, warp): new cells before it
    __shared__ int warp_tot[32];
    __shared__ int s_skip, s_bottom;
    Ctrl *ctrl = s.ctrl;
    const int L = t.levels, n = s.n, root = n + s.cap;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int n_last = 1 << (3 * L);
    if (tid == 0) {
        s_skip = read_status(ctrl);
        s_bottom = ctrl->bottom;
    }
    __syncthreads();
    if (!s_skip) {
        for (int l = L - 1; l >= 1; --l) {
            const int nr = 1 << (3 * l);
            int *dst = cnt_sh + top_offset(l);
            for (int r = tid; r < nr; r += nt) {
                int sum = 0;
                if (l == L - 1) {
                    const int4 a = reinterpret_cast<const int4 *>(t.count)[2 * r];
                    const int4 b = reinterpret_cast<const int4 *>(t.count)[2 * r + 1];
                    sum = a.x + a.y + a.z + a.w + b.x + b.y + b.z + b.w;
                } else {
                    const int *src = cnt_sh + top_offset(l + 1) + 8 * r;
#pragma unroll
                    for (int j = 0; j < 8; ++j) sum += src[j];
                }
                dst[r] = sum;
            }
            __syncthreads();
        }
        const int lane = tid & 31, w = tid >> 5, nw = nt >> 5;
        const unsigned below = (1u << lane) - 1u;
        const int last = deep_out ? L - 1 : L;
        for (int l = 1; l <= last; ++l) {
            // region r = j * nt + tid in round j; a level's cells are numbered
            // bottom - 1 - rank with rank in (round, warp, lane) order, so a
            // warp's new cells are consecutive and its writes coalesce
            const int nr = 1 << (3 * l);
            const int rounds = (nr + nt - 1) / nt, m = rounds * nw;  // rounds <= 32: 8^L <= 32 * blockDim.x
            const int *cnt = l < L ? cnt_sh + top_offset(l) : t.count;
            unsigned make_bits = 0;  // bit j: region j * nt + tid gets a cell
#pragma unroll 8
            for (int j = 0; j < rounds; ++j) {  // independent loads, then the votes
                const int r = j * nt + tid;
                if (r < nr && cnt[r] >= 2) make_bits |= 1u << j;
            }
            for (int j = 0; j < rounds; ++j) {
                const unsigned b = __ballot_sync(0xffffffffu, (make_bits >> j) & 1u);
                if (lane == 0) rank_sh[j * nw + w] = __popc(b);
            }
            __syncthreads();
            int total = 0;  // exclusive scan of rank_sh[0, m) in place
            for (int base = 0; base < m; base += nt) {
                const int v = base + tid < m ? rank_sh[base + tid] : 0;
                int part = 0;
                const int ex = block_exclusive_sum(v, warp_tot, &part);
                if (base + tid < m) rank_sh[base + tid] = total + ex;
                total += part;
            }
            __syncthreads();
            const int bottom = s_bottom;
            if (bottom - total < n) {  // block-uniform: more top cells than the capacity
                if (tid == 0) set_status(ctrl, kStCellOverflow, l);
                s_skip = 1;
                break;
            }
            for (int j = 0; j < rounds; ++j) {
                const int r = j * nt + tid;
                const bool make = (make_bits >> j) & 1u;
                const unsigned b = __ballot_sync(0xffffffffu, make);
                if (r >= nr) continue;
                const int pe = l == 1 ? root : deep_sh[top_offset(l - 1) + (r >> 3)];
                int e = pe;
                if (make) {  // the parent region holds these bodies too: its cell exists
                    const int cell = bottom - 1 - (rank_sh[j * nw + w] + __popc(b & below));
                    const int c = cell - n;
                    int4 *row = reinterpret_cast<int4 *>(&s.child[c * 8]);
                    row[0] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
                    row[1] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
                    const int parent = pe & ((1 << 26) - 1);
                    s.parent[c] = parent;
                    s.arrive[c] = 0;
                    s.start[c] = -1;
                    s.child[(parent - n) * 8 + (r & 7)] = cell;
                    e = (l << 26) | cell;
                }
                if (l < L) deep_sh[top_offset(l) + r] = e;
                else t.start[r] = e;
                if (deep_out && l == last) deep_out[r] = e;
            }
            __syncthreads();
            if (tid == 0) s_bottom = bottom - total;
            __syncthreads();
        }
    }
    __syncthreads();
    if (!deep_out)
        for (int r = tid; r < n_last; r += nt) t.count[r] = 0;
    if (tid == 0 && !s_skip) ctrl->bottom = s_bottom;
}

// The cells of level L after top_cells_block(..., deep): one region per
// thread, warp-aggregated numbering from the cell counter (below every cell
// of the upper levels), the start entries, and the counts cleared.
__device__ __forceinline__ void top_leaf_cells(const DevSim &s, const TopTables &t, const int *deep, int r) {
    Ctrl *ctrl = s.ctrl;
    const int n = s.n, nr = 1 << (3 * t.levels);
    const bool skip = read_status(ctrl) != 0;  // grid-uniform: only earlier kernels set it
    const int cnt = r < nr ? t.count[r] : 0;
    const bool make = !skip && cnt >= 2;
    const unsigned am = __activemask();
    const unsigned b = __ballot_sync(am, make);
    const int leader = __ffs(am) - 1, lane = threadIdx.x & 31;
    int base = 0;
    if (lane == leader && b) base = atomicSub(&ctrl->bottom, __popc(b));
    base = __shfl_sync(am, base, leader);
    if (r >= nr) return;
    t.count[r] = 0;
    if (skip) return;
    const int pe = deep[r >> 3];
    int e = pe;
    if (make) {
        const int cell = base - 1 - __popc(b & ((1u << lane) - 1u));
        if (cell < n) {  // more top cells than the capacity
            set_status(ctrl, kStCellOverflow, t.levels);
            return;
        }
        const int c = cell - n;
        int4 *row = reinterpret_cast<int4 *>(&s.child[c * 8]);
        row[0] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
        row[1] = make_int4(kEmpty, kEmpty, kEmpty, kEmpty);
        const int parent = pe & ((1 << 26) - 1);
        s.parent[c] = parent;
        s.arrive[c] = 0;
        s.start[c] = -1;
        s.child[(parent - n) * 8 + (r & 7)] = cell;
        e = (t.levels << 26) | cell;
    }
    t.start[r] = e;
}

// Insertion of body i from the deepest existing top cell of its level-L path.
__device__ __forceinline__ int insert_from_top(const DevSim &s, const TopTables &t, const GeoCube &root_g, int i,
                                               long long spin_cap) {
    const float4 P = s.body_cur[i];
    const int e = __ldg(&t.start[top_region(root_g, P, t.levels)]);
    const int lv = (int)((unsigned)e >> 26), node = e & ((1 << 26) - 1);
    GeoCube g = root_g;
    for (int l = 0; l < lv; ++l) g.descend(P.x, P.y, P.z);
    const int slot = g.octant(P.x, P.y, P.z);
    g.descend(P.x, P.y, P.z);
    return insert_from<GeoCube>(s, g, node, slot, lv, P, i, spin_cap);
}

__device__ __forceinline__ void load_children(const int *child, int c, int chs[8], int &nch, int &nbody, int n) {
    const int4 a0 = *reinterpret_cast<const int4 *>(&child[c * 8]);
    const int4 a1 = *reinterpret_cast<const int4 *>(&child[c * 8 + 4]);
    chs[0] = a0.x; chs[1] = a0.y; chs[2] = a0.z; chs[3] = a0.w;
    chs[4] = a1.x; chs[5] = a1.y; chs[6] = a1.z; chs[7] = a1.w;
    nch = 0;
    nbody = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        nch += chs[j] >= 0;
        nbody += (chs[j] >= 0) & (chs[j] < n);
    }
}

// ---------------------------------------------------------------------------
// Summarisation starting at cell node k: bottom-up centre of mass with
// L2-resident arrival counters.  The cell's own thread adds the number of its
// body children to the counter in one atomic; a completed child cell adds
// one.  Whoever brings the counter to the number of children computes the
// cell and then arrives at the parent, and so on up to the root.  No thread
// ever waits (saturate_tree.cl spins on child masses, :96-117).  Children are
// summed in slot order -- mass += m, centre += x*m, centre *= 1/mass, each
// rounded separately (saturate_tree.cl:84-87,129-133) -- so the result does
// not depend on the schedule and matches the oracle bit for bit.  The
// completing thread also writes the compacted child list and the packed child
// {x,y,z,m} line (and quadrupoles) the force walk reads (the reference
// compacts in place, saturate_tree.cl:57-63, and skips the move when a
// child's index equals its new slot number; that defect is not reproduced).
// Fences: release before every counter update, acquire after the update that
// completes a cell; child-cell data written in this kernel is read through L2.
// ---------------------------------------------------------------------------
template <bool kQuad>
__device__ __forceinline__ void summarize_from(const DevSim &s, int k) {
    const int n = s.n, root = n + s.cap;
    int node = k;
    int chs[8], nch, nbody;
    load_children(s.child, node - n, chs, nch, nbody, n);
    if (nbody == 0) return;  // completed by its child cells
    if (nbody != nch) {
        const int old = atomicAdd(&s.arrive[node - n], nbody);
        if (old + nbody != nch) return;
        __threadfence();
    }
    while (true) {
        const int c = node - n;
        float M = 0.0f, cx = 0.0f, cy = 0.0f, cz = 0.0f;
        int cnt = 0, w = 0;
        // children in slot order; the compacted list and packed lines go to
        // the cell's rows.  The monopole kernel stores them as they come
        // (fewer registers, more warps); the quadrupole pass needs them again,
        // so that kernel gathers them in registers and stores whole rows.
        int wc[kQuad ? 8 : 1];
        float4 wp[kQuad ? 8 : 1];
        int *wrow = &s.wchild[c * 8];
        float4 *prow = &s.wpm[c * 8];
        if constexpr (kQuad) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                wc[j] = kEmpty;
                wp[j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int ch = chs[j];
            if (ch < 0) continue;
            float4 pm;
            int cc;
            if (ch < n) {
                pm = s.body_cur[ch];
                cc = 1;
            } else {
                pm = __ldcg(&s.cell_pm[ch - n]);
                cc = __ldcg(&s.count[ch - n]);
            }
            M = __fadd_rn(M, pm.w);
            cx = __fadd_rn(cx, __fmul_rn(pm.x, pm.w));
            cy = __fadd_rn(cy, __fmul_rn(pm.y, pm.w));
            cz = __fadd_rn(cz, __fmul_rn(pm.z, pm.w));
            cnt += cc;
            if constexpr (kQuad) {
                // w <= j, so a static index write through a select chain
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (q == w) { wc[q] = ch; wp[q] = pm; }
            } else {
                wrow[w] = ch;
                prow[w] = pm;
            }
            ++w;
        }
        if constexpr (kQuad) {
            int4 *r4 = reinterpret_cast<int4 *>(wrow);
            r4[0] = make_int4(wc[0], wc[1], wc[2], wc[3]);
            r4[1] = make_int4(wc[4], wc[5], wc[6], wc[7]);
#pragma unroll
            for (int q = 0; q < 8; ++q) prow[q] = wp[q];
        } else {
            for (int q = w; q < 8; ++q) {
                wrow[q] = kEmpty;
                prow[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
        }
        const float inv = __frcp_rn(M);
        const float X = __fmul_rn(cx, inv), Y = __fmul_rn(cy, inv), Z = __fmul_rn(cz, inv);
        s.count[c] = cnt;
        s.cell_pm[c] = make_float4(X, Y, Z, M);
        if constexpr (kQuad) {
            // traceless quadrupole about the centre of mass, children in
            // slot order: Q += Q_child + m (3 d d^T - |d|^2 I), d = x_child - X
            float q0 = 0.0f, q1 = 0.0f, q2 = 0.0f, q3 = 0.0f, q4 = 0.0f, q5 = 0.0f;
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int ch = wc[j];
                if (ch < 0) break;
                const float4 pm = wp[j];
                float4 oa = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                float4 ob = oa;
                if (ch >= n) {
                    oa = __ldcg(&s.cell_q[2 * (ch - n)]);
                    ob = __ldcg(&s.cell_q[2 * (ch - n) + 1]);
                }
                s.wqa[c * 8 + j] = oa;
                s.wqb[c * 8 + j] = make_float2(ob.x, ob.y);
                const float m = pm.w;
                const float dx = __fsub_rn(pm.x, X), dy = __fsub_rn(pm.y, Y), dz = __fsub_rn(pm.z, Z);
                const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
                const float tx = __fmul_rn(3.0f, dx), ty = __fmul_rn(3.0f, dy);
                q0 = __fadd_rn(q0, __fmaf_rn(m, __fmaf_rn(tx, dx, -r2), oa.x));
                q1 = __fadd_rn(q1, __fmaf_rn(m, __fmaf_rn(ty, dy, -r2), oa.y));
                q2 = __fadd_rn(q2, __fmaf_rn(m, __fmaf_rn(__fmul_rn(3.0f, dz), dz, -r2), oa.z));
                q3 = __fadd_rn(q3, __fmaf_rn(m, __fmul_rn(tx, dy), oa.w));
                q4 = __fadd_rn(q4, __fmaf_rn(m, __fmul_rn(tx, dz), ob.x));
                q5 = __fadd_rn(q5, __fmaf_rn(m, __fmul_rn(ty, dz), ob.y));
            }
            s.cell_q[2 * c] = make_float4(q0, q1, q2, q3);
            s.cell_q[2 * c + 1] = make_float4(q4, q5, 0.0f, 0.0f);
        }
        if (node == root) return;
        const int p = s.parent[c];
        load_children(s.child, p - n, chs, nch, nbody, n);
        __threadfence();
        const int old = atomicAdd(&s.arrive[p - n], 1);
        if (old + 1 != nch) return;
        __threadfence();
        node = p;
    }
}

// ---------------------------------------------------------------------------
// Sort step for cell node k (Burtscher's in-order placement; the reference's
// kernels/sort.cl is empty): wait -- bounded -- until the parent has
// published the cell's start, then hand each child cell a start (running sum
// of counts in slot order) and place each child body.  Returns false when
// the sort must stop (the status word is set).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool sort_cell(const DevSim &s, int k, long long spin_cap) {
    Ctrl *ctrl = s.ctrl;
    const int n = s.n;
    const int c = k - n;
    int st = ld_volatile(&s.start[c]);
    long long spins = 0;
    unsigned pause = 32;  // back off: many waiting threads must not flood L2 with polls
    while (st < 0) {
        if (++spins > spin_cap) {
            set_status(ctrl, kStSpinTimeout, k);
            return false;
        }
        if ((spins & 1023) == 0 && read_status(ctrl)) return false;
        __nanosleep(pause);
        if (pause < 1024) pause <<= 1;
        st = ld_volatile(&s.start[c]);
    }
    const int4 a0 = *reinterpret_cast<const int4 *>(&s.wchild[c * 8]);
    const int4 a1 = *reinterpret_cast<const int4 *>(&s.wchild[c * 8 + 4]);
    const int chs[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const int ch = chs[j];
        if (ch < 0) break;
        if (ch >= n) {
            st_volatile(&s.start[ch - n], st);
            st += s.count[ch - n];
        } else {
            if ((unsigned)st >= (unsigned)n) {  // inconsistent counts: never write past sorted[]
                set_status(ctrl, kStSpinTimeout, st);
                return false;
            }
            s.sorted[st] = ch;
            ++st;
        }
    }
    return true;
}

}  // namespace nbgb
