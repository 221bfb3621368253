// sysmem.cuh -- the device buffers of one system carved from a shared arena
// (batched systems and served requests): the same arrays, with the same
// sizes, as a standalone handle holds, laid out back to back with every
// array 256-byte aligned (TMA bulk copies need 16 bytes).
#pragma once
#include <cstddef>

#include "../../include/nbgb.h"
#include "nbgb_internal.cuh"

namespace nbgb {

struct SysMem {
    int n = 0, cap = 0;
    bool tree = false, quad = false;
    float4 *body[2] = {nullptr, nullptr};
    float4 *vel = nullptr, *acc = nullptr, *part = nullptr;
    int *parent = nullptr, *child = nullptr, *wchild = nullptr, *count = nullptr, *start = nullptr,
        *arrive = nullptr, *sorted = nullptr;
    float4 *wpm = nullptr, *cell_pm = nullptr, *cell_q = nullptr, *wqa = nullptr;
    float2 *wqb = nullptr;
    int *top = nullptr;  // top-level tables (batch_top_levels_for): counts, then start entries
    int top_levels = 0;
    Ctrl *ctrl = nullptr;
};

inline size_t sysmem_align(size_t x) { return (x + 255) & ~(size_t)255; }

// Cells of a batched tree: max(2N, 4096) rounded up to 16.  The standalone
// handle's floor of 1024 cells per SM (src/MyApp.cpp:75-79) would give every
// small system of a large batch ~150k cells.
inline int sysmem_default_capacity(int n) {
    long long c = 2LL * n;
    if (c < 4096) c = 4096;
    return (int)((c + 15) / 16 * 16);
}

// Bytes the system needs; when base is non-null the pointers are set to
// consecutive pieces of [base, base + bytes).  The owner clears the top-level
// counts (sysmem_top_counts) once before the first step; every step leaves
// them at zero.
inline size_t sysmem_layout(SysMem &m, char *base) {
    size_t off = 0;
    auto take = [&](auto *&p, size_t count) {
        using T = std::remove_reference_t<decltype(*p)>;
        off = sysmem_align(off);
        p = base && count ? reinterpret_cast<T *>(base + off) : nullptr;
        off += sizeof(T) * count;
    };
    const size_t n = (size_t)m.n;
    take(m.body[0], n);
    take(m.body[1], n);
    take(m.vel, n);
    take(m.acc, n);
    if (m.tree) {
        const size_t cells = (size_t)m.cap + 1;
        take(m.parent, cells);
        take(m.child, cells * 8);
        take(m.wchild, cells * 8);
        take(m.wpm, cells * 8);
        take(m.cell_pm, cells);
        take(m.count, cells);
        take(m.start, cells);
        take(m.arrive, cells);
        take(m.sorted, n);
        if (m.quad) {
            take(m.cell_q, cells * 2);
            take(m.wqa, cells * 8);
            take(m.wqb, cells * 8);
        }
        m.top_levels = batch_top_levels_for(m.n);
        if (m.top_levels) take(m.top, (size_t)2 << (3 * m.top_levels));
    }
    return sysmem_align(off);
}

// the top-level count table of a tree (nullptr, 0 when it has none)
inline void sysmem_top_counts(const SysMem &m, int **p, size_t *bytes) {
    *p = m.top;
    *bytes = m.top ? sizeof(int) << (3 * m.top_levels) : 0;
}

inline size_t sysmem_bytes(int n, bool tree, bool quad, int cap) {
    SysMem m;
    m.n = n;
    m.tree = tree;
    m.quad = quad;
    m.cap = cap;
    return sysmem_layout(m, nullptr);
}

// Descriptor of a system: its buffers and the step parameters of its config
// (the same choices as the standalone step).
// The top-level tables of a system building min(m.top_levels, cap) top
// levels (none for the reference tree semantics, which always insert from
// the root).  The count table (8^levels entries, zero between steps) and the
// start table lie at fixed places for any level count -- the start table
// after room for the counts of m.top_levels -- so a step with fewer levels
// never leaves start entries where a later step with more levels counts.
inline void sysdesc_set_top(SysDesc &d, const SysMem &m, bool tree_ref, int cap) {
    const int top = tree_ref ? 0 : (m.top_levels < cap ? m.top_levels : cap);
    d.top = TopTables{top ? m.top : nullptr, top ? m.top + (1 << (3 * m.top_levels)) : nullptr, top, nullptr};
}

inline SysDesc sysmem_desc(const SysMem &m, const nb_config &c, float dt) {
    SysDesc d{};
    DevSim &v = d.v;
    v.n = m.n;
    v.cap = m.cap;
    v.body_cur = m.body[0];
    v.body_next = m.body[1];
    v.vel = m.vel;
    v.acc = m.acc;
    v.parent = m.parent;
    v.child = m.child;
    v.wchild = m.wchild;
    v.wpm = m.wpm;
    v.cell_pm = m.cell_pm;
    v.count = m.count;
    v.start = m.start;
    v.arrive = m.arrive;
    v.sorted = m.sorted;
    v.part = m.part;
    v.cell_q = m.cell_q;
    v.wqa = m.wqa;
    v.wqb = m.wqb;
    v.ctrl = m.ctrl;
    sysdesc_set_top(d, m, c.tree_semantics == NB_TREE_REFERENCE, kBatchTopMaxLevels);
    d.body[0] = m.body[0];
    d.body[1] = m.body[1];
    StepParams &p = d.p;
    p.dt = dt;
    p.G = c.gravitational_constant;
    p.theta = c.theta;
    p.method = c.numerical_method;
    p.kdk_primed = 0;
    p.tree_ref = c.tree_semantics == NB_TREE_REFERENCE;
    p.crit_ref = c.theta_semantics == NB_THETA_REFERENCE;
    p.quadrupole = m.quad ? 1 : 0;
    p.eps = m.tree ? c.epsilon : (c.direct_epsilon >= 0.0f ? c.direct_epsilon : c.epsilon);
    d.kind = m.tree ? kSysBH : kSysDirect;
    d.collide = c.collision ? 1 : 0;
    d.active = 1;
    return d;
}

// The batch-wide index spaces: bbox/build chunks, cell slots, force warp
// groups, direct-sum blocks, collision blocks.
constexpr int kBatchSpaces = 5;
// host-written prefix tables, nsys + 1 entries each
inline size_t batch_prefix_ints(int nsys) { return (size_t)kBatchSpaces * (size_t)(nsys + 1); }
// on the device they are followed by the device-written table of used cells
inline size_t batch_prefix_device_ints(int nsys) { return (size_t)(kBatchSpaces + 1) * (size_t)(nsys + 1); }

// Where every system's work starts in the batch-wide index spaces (direct-sum
// blocks of `direct_block` bodies, collision blocks of kCollideBlockBodies,
// bbox / build chunks of chunk_override bodies when > 0, else batch_chunk's).
// Fills the *_begin fields of sys, the prefix tables (nsys + 1 entries each,
// back to back in pref) and their totals.
inline void batch_prefixes(SysDesc *sys, int nsys, int direct_block, int *pref, int totals[kBatchSpaces],
                           int chunk_override = 0) {
    int *chunk = pref, *cell = pref + (nsys + 1), *group = pref + 2 * (nsys + 1), *dblock = pref + 3 * (nsys + 1),
        *cblock = pref + 4 * (nsys + 1);
    chunk[0] = cell[0] = group[0] = dblock[0] = cblock[0] = 0;
    long long tree_bodies = 0;
    for (int k = 0; k < nsys; ++k)
        if (sys[k].active && sys[k].kind == kSysBH) tree_bodies += sys[k].v.n;
    int body = 0;
    for (int k = 0; k < nsys; ++k) {
        SysDesc &d = sys[k];
        const int n = d.v.n;
        d.body_begin = body;
        d.chunk_begin = chunk[k];
        d.cell_begin = cell[k];
        d.group_begin = group[k];
        d.dblock_begin = dblock[k];
        d.cblock_begin = cblock[k];
        const bool bh = d.active && d.kind == kSysBH, direct = d.active && d.kind == kSysDirect;
        d.chunk = chunk_override > 0 ? chunk_override : batch_chunk(n, tree_bodies);
        chunk[k + 1] = chunk[k] + (bh ? (n + d.chunk - 1) / d.chunk : 0);
        cell[k + 1] = cell[k] + (bh ? d.v.cap + 1 : 0);
        group[k + 1] = group[k] + (bh ? (n + 31) / 32 : 0);
        dblock[k + 1] = dblock[k] + (direct ? (n + direct_block - 1) / direct_block : 0);
        cblock[k + 1] = cblock[k] + (d.active && d.collide ? (n + kCollideBlockBodies - 1) / kCollideBlockBodies : 0);
        body += n;
    }
    totals[0] = chunk[nsys];
    totals[1] = cell[nsys];
    totals[2] = group[nsys];
    totals[3] = dblock[nsys];
    totals[4] = cblock[nsys];
}

// d_pref holds the prefix tables of batch_prefixes followed by room for the
// device-written table of used cells: batch_prefix_device_ints(nsys) ints.
inline BatchTables batch_tables(const SysDesc *d_sys, int nsys, int *d_pref, const int totals[kBatchSpaces],
                                int *work) {
    BatchTables t{};
    t.sys = d_sys;
    t.nsys = nsys;
    t.chunk_prefix = d_pref;
    t.cell_prefix = d_pref + (nsys + 1);
    t.group_prefix = d_pref + 2 * (nsys + 1);
    t.dblock_prefix = d_pref + 3 * (nsys + 1);
    t.cblock_prefix = d_pref + 4 * (nsys + 1);
    t.chunks = totals[0];
    t.cells = totals[1];
    t.groups = totals[2];
    t.dblocks = totals[3];
    t.cblocks = totals[4];
    t.work = work;
    t.used_prefix = d_pref + kBatchSpaces * (nsys + 1);
    return t;
}

}  // namespace nbgb
