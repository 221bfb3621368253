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
// consecutive pieces of [base, base + bytes).
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
    }
    return sysmem_align(off);
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
    d.active = 1;
    return d;
}

}  // namespace nbgb
