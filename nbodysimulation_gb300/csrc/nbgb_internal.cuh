// nbgb_internal.cuh -- device data layout and helpers shared by the kernels.
//
// Layout in HBM (one system of N bodies, C cells):
//   body_pm[2][N]  float4 {x,y,z,m}     positions double-buffered per step
//   vel[N], acc[N] float4               velocity / last acceleration (w unused)
//   node index space: bodies [0,N), cells [N, N+C), root N+C (the
//   reference's index space, src/MyApp.cpp:71-83); cell arrays are indexed
//   by cell - N and have C+1 entries (the root is the last one).
//   child[(C+1)*8]   int   octant slots written by the build
//   wchild[(C+1)*8]  int   the same children compacted in slot order
//   wpm[(C+1)*8]     float4 {x,y,z,m} of those children, packed per cell so
//                    the force walk reads one 128-byte line per opened cell
//   cell_pm[C+1]     float4 centre of mass + mass
//   count/start/arrive/parent[C+1] int (parent: of a cell), sorted[N] int
//   Ctrl             bbox keys, allocation counter, max depth, status
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace nbgb {

constexpr int kMaxDepth = 64;
// targets per block of the collision update's block form (one thread each)
constexpr int kCollideBlockBodies = 256;
constexpr int kLocked = -2;
constexpr int kEmpty = -1;

// device status codes (same values as nb_status)
constexpr int kStOk = 0;
constexpr int kStCellOverflow = 4;
constexpr int kStDepth = 5;
constexpr int kStSpinTimeout = 6;
constexpr int kStNonFinite = 7;

// bounded waits: iterations before a device wait gives up with kStSpinTimeout
constexpr long long kSpinCap = 1LL << 24;

struct Ctrl {
    unsigned bbox_key[6];  // order-preserving keys: min xyz, max xyz
    int bottom;            // lowest allocated cell index
    int max_depth;
    int work;              // dynamic work counter of the force pass
    int parity;            // batched systems: which body buffer is current
    int kdk_primed;        // batched systems: a KDK half-kick has happened
    int budget;            // batched systems: steps left (< 0 unlimited, 0 inert)
    int spin_cap;          // > 0: iteration cap of the tree stages' waits (a test hook); 0: kSpinCap
    int pad0[1];
    // cleared by the host once per nb_step call (everything from here on)
    int status;
    int status_info;
    unsigned long long interactions;  // body-node interactions of the force passes
    unsigned long long opened;        // cells opened by the force passes
    unsigned long long cell_interactions;  // the part of `interactions` with cells
};

struct DevSim {
    int n;
    int cap;
    const float4 *body_cur;
    float4 *body_next;
    float4 *vel;
    float4 *acc;
    int *parent;
    int *child;
    int *wchild;
    float4 *wpm;
    float4 *cell_pm;
    int *count;
    int *start;
    int *arrive;
    int *sorted;
    float4 *part;    // N partial accelerations of a split direct sum
    float4 *cell_q;  // 2 per cell: {xx, yy, zz, xy}, {xz, yz, 0, 0} about the centre of mass
    float4 *wqa;     // (C+1)*8: quadrupole {xx, yy, zz, xy} of each packed child (0 for bodies)
    float2 *wqb;     // (C+1)*8: {xz, yz} of each packed child
    Ctrl *ctrl;
};

struct StepParams {
    float dt;
    float G;
    float theta;
    float eps;
    int method;      // 1 leapfrog as written, 2 euler, 3 kdk
    int kdk_primed;
    int tree_ref;    // reference tree semantics
    int crit_ref;    // reference opening thresholds
    int quadrupole;  // accepted cells add their quadrupole term
};

__device__ __forceinline__ unsigned f2key(float f) {
    unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float key2f(unsigned k) {
    unsigned b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(b);
}

// Reciprocal square root on the MUFU unit with subnormal inputs flushed
// (PTX rsqrt.approx.ftz.f32).  The pair sums only take it of d^2 + eps^2,
// which is normal or zero; without the flush the compiler wraps the MUFU
// instruction in a rescaling for subnormal inputs that costs issue slots in
// the innermost loops.
__device__ __forceinline__ float rsqrt_fast(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void set_status(Ctrl *c, int code, int info) {
    if (atomicCAS(&c->status, 0, code) == 0) c->status_info = info;
}
__device__ __forceinline__ int read_status(const Ctrl *c) {
    return *(volatile const int *)&c->status;
}

__device__ __forceinline__ int ld_volatile(const int *p) { return *(volatile const int *)p; }

// Iteration cap of the build's lock retries and the sort's wait for a
// parent, read once per thread (the Ctrl line is busy with the build's
// allocation atomics).  The TMA waits keep kSpinCap: they must outlast their
// own copies.
__device__ __forceinline__ long long tree_spin_cap(const Ctrl *c) {
    const int v = c->spin_cap;
    return v > 0 ? (long long)v : kSpinCap;
}
__device__ __forceinline__ void st_volatile(int *p, int v) { *(volatile int *)p = v; }

// Opening thresholds per depth, as in the oracle's orc_bh_thresholds.
__device__ __forceinline__ void make_thresholds(const float box[6], float theta, float eps, int crit_ref,
                                                float *dq) {
    float radius = 0.5f * fmaxf(fmaxf(box[3] - box[0], box[4] - box[1]), box[5] - box[2]);
    float d0;
    if (crit_ref) {
        d0 = theta > 0.0f ? __fdiv_rn(__fmul_rn(radius, radius), theta) : __fmul_rn(radius, radius);
    } else {
        float itolsq = __fdiv_rn(1.0f, __fmul_rn(theta, theta));
        d0 = __fmul_rn(__fmul_rn(radius, radius), itolsq);
    }
    float add = crit_ref ? eps : __fmul_rn(eps, eps);
    float base = d0;
    for (int i = 0; i < kMaxDepth; ++i) {
        dq[i] = __fadd_rn(base, add);
        base = __fmul_rn(0.25f, base);
    }
}

__device__ __forceinline__ void load_box(const Ctrl *c, float box[6]) {
    for (int k = 0; k < 6; ++k) box[k] = key2f(c->bbox_key[k]);
}

// One system of a batch (nb_batch / nb_server): its buffers, its step
// parameters and where its work starts in the batch-wide index spaces.
enum SysKind { kSysBH = 0, kSysDirect = 1 };
// Per-system tables of the top levels of the cubic-root tree (k_tree.cu):
// body counts of the 8^levels regions of the deepest top level (zero between
// steps) and, per region, the packed (level << 26) | cell its bodies start
// their insertion at.  levels = 0: every insertion starts at the root.
struct TopTables {
    int *count;
    int *start;
    int levels;
    int *deep;  // 8^(levels-1) entries of level levels-1 when the last level is built by a grid (else null)
};
constexpr int kTopMaxLevels = 5;                  // 8^5 = 32768 regions
constexpr int kTopRegions = 1 << (3 * kTopMaxLevels);
constexpr int kTopInner = (kTopRegions - 8) / 7;  // regions of levels 1..4: 8 + 64 + 512 + 4096
// top levels for a tree of n bodies: about 8 bodies or more per region of the
// deepest level, at most kTopMaxLevels, none below 2 (262,144-body ball:
// build 0.102 ms with 5 levels, 0.116 ms with 4)
inline int top_levels_for(int n) {
    int l = 0;
    while (l < kTopMaxLevels && (8LL << (3 * (l + 1))) <= (long long)n) ++l;
    return l >= 2 ? l : 0;
}
// batched trees count in shared-memory bins per block of bodies, so at most
// 4 levels (4096 bins, 16 KB)
constexpr int kBatchTopMaxLevels = 4;
inline int batch_top_levels_for(int n) {
    const int l = top_levels_for(n);
    return l < kBatchTopMaxLevels ? l : kBatchTopMaxLevels;
}

struct SysDesc {
    DevSim v;          // pointers; body_cur / body_next come from body[] and ctrl->parity
    float4 *body[2];
    StepParams p;      // theta, eps, G, dt, method, tree_ref, crit_ref, quadrupole
    int kind;          // SysKind
    int active;        // 0: skipped by every stage
    int body_begin;    // prefix over all systems' bodies
    int chunk_begin;   // prefix over BH systems' bbox/build chunks
    int cell_begin;    // prefix over BH systems' cell slots (cap + 1)
    int group_begin;   // prefix over BH systems' warp groups
    int dblock_begin;  // prefix over direct systems' target blocks
    int cblock_begin;  // prefix over colliding systems' collision blocks
    int collide;       // the collision update runs after the force and integrate stages
    int chunk;         // bodies per bbox / build block (batch_chunk)
    TopTables top;     // top-level tables; levels = 0: insertions from the root
};

// Prefix tables (nsys + 1 entries each) and totals of a batch.
struct BatchTables {
    const SysDesc *sys;
    int nsys;
    const int *chunk_prefix, *cell_prefix, *group_prefix, *dblock_prefix, *cblock_prefix;
    int chunks, cells, groups, dblocks, cblocks;
    int *work;         // batch-wide force work counter
    int *used_prefix;  // nsys + 1: prefix over the cells each tree allocated this step (device-written)
};

__device__ __forceinline__ int find_system(const int *prefix, int nsys, int x) {
    int lo = 0, hi = nsys;  // largest k with prefix[k] <= x and prefix[k+1] > x
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&prefix[mid]) <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// A batched system with no steps left takes no part in any stage.
__device__ __forceinline__ bool system_live(const Ctrl *c) { return ld_volatile(&c->budget) != 0; }

__device__ __forceinline__ DevSim system_view_par(const SysDesc &d, int par) {
    DevSim v = d.v;
    v.body_cur = d.body[par];
    v.body_next = d.body[par ^ 1];
    return v;
}

__device__ __forceinline__ int system_parity(const SysDesc &d) { return ld_volatile(&d.v.ctrl->parity) & 1; }

__device__ __forceinline__ DevSim system_view(const SysDesc &d) { return system_view_par(d, system_parity(d)); }

// Launch helpers implemented in the kernel translation units.
struct LaunchShape {
    int blocks;
    int threads;
};

cudaError_t launch_reset(const DevSim &s, cudaStream_t st);
cudaError_t launch_bbox(const DevSim &s, int sm_count, cudaStream_t st);
// Launches the build (the top-level count and cells first when top.levels >
// 0 and the tree is the cubic-root one); *launches gets the kernel count.
cudaError_t launch_build(const DevSim &s, const TopTables &top, int tree_ref, int sm_count, cudaStream_t st,
                         int *launches);
cudaError_t launch_summarize(const DevSim &s, int quadrupole, int sm_count, cudaStream_t st);
cudaError_t launch_sort(const DevSim &s, int sm_count, cudaStream_t st);
cudaError_t launch_force(const DevSim &s, const StepParams &p, int compensated, int sm_count, cudaStream_t st);
cudaError_t launch_direct(const DevSim &s, const StepParams &p, int tiled, int quirk, int sm_count,
                          cudaStream_t st);
// tree != 0: s.sorted holds this step's in-order sort (targets handed out in it)
cudaError_t launch_collision(const DevSim &s, int tree, int sm_count, cudaStream_t st);
cudaError_t launch_copy_vertices(const float4 *body, int n, float4 *dst, cudaStream_t st);
cudaError_t launch_pack(const float *pos3, const float *mass, const float *vel3, float4 *body, float4 *vel,
                        float4 *acc, int n, cudaStream_t st);
cudaError_t launch_unpack(const float4 *body, const float4 *vel, const float4 *acc, float *pos3, float *vel3,
                          float *acc3, int n, cudaStream_t st);
cudaError_t launch_export_tree(const DevSim &s, int *children_full, float *pos_full, float *mass_full,
                               int *count_full, float *quad_full, cudaStream_t st);
cudaError_t launch_force_probe(const float4 *body, int n, const int *sample, int ns, double eps, double G,
                               double *out3, cudaStream_t st);
cudaError_t launch_diagnostics(const float4 *body, const float4 *vel, int n, int with_potential, double eps,
                               double G, double *out9, cudaStream_t st);

// batched systems (k_batch.cu)
// Bodies per bbox / build block of a batched tree.  Threads that start at a
// root together contend for its first cells, so fewer per tree is better
// once the batch as a whole has threads enough: 4096 when the batch's trees
// hold 4M bodies or more, or for a tree of 2^19 bodies or more; 1024
// otherwise (measured: a 512-system batch of 27M bodies builds in 3.6 ms
// with 4096 and 6.6 ms with 1024; a lone 131k-body tree steps in 0.67 ms
// with 1024 and 0.81 ms with 4096).
inline int batch_chunk(int n, long long batch_tree_bodies) {
    return (n >= (1 << 19) || batch_tree_bodies >= (4LL << 20)) ? 4096 : 1024;
}
int batch_direct_variants();
int batch_direct_block_bodies(int variant);
// Optional second stream of a captured batched step: the small systems'
// direct sum runs on it beside the tree stages up to the summarisation (a
// parallel branch of the graph); the sort, whose waits assume its whole grid
// is resident, starts after both.
struct StepFork {
    cudaStream_t aux;
    cudaEvent_t fork, join;
};
// Launch shapes of a batched step that do not change any result (the tree
// and every sum are the same for all of them), so the autotuner may choose
// them and a batched system stays bit-identical to a standalone handle.
struct TreeShape {
    int force_warps = 4;       // warps per block of the batched force kernel: 2, 4 or 8
    int force_grid_pct = 100;  // percent of the resident force blocks launched
    int build_chunk = 0;       // bodies per bbox / build block of every tree; 0: batch_chunk's rule
    int top_levels = kBatchTopMaxLevels;  // at most this many top levels built first
};
// advance = false leaves out the collision update and the flip: the tree
// stages and the direct sums as a step runs them (the direct sums beside the
// tree stages on fork->aux), which is what the autotuner times with dt = 0.
cudaError_t launch_batch_step(const BatchTables &t, int method, int comp, int quad, int direct_variant,
                              const TreeShape &shape, int sm_count, cudaStream_t st, const StepFork *fork,
                              int *launches, bool advance = true);
// clears the status word and work counters of every system (once per call)
cudaError_t launch_batch_clear(const BatchTables &t, cudaStream_t st);

}  // namespace nbgb
