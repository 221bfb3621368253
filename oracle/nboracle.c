/*
 * nboracle.c -- TEST INFRASTRUCTURE: the CPU oracle.
 *
 * A plain-C restatement of the reference's per-step N-body kernels
 * (Ace-of-Heartz/NBodySimulation, the kernels/ .cl files).  It is the checker for the
 * GB300 library and is used only by tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py; nothing in the product links or calls it.
 *
 * Each function names the reference file:line it restates.  Where the
 * reference has a defect, the restatement keeps it behind a named switch so
 * the oracle can be pinned against the reference's own kernels (built here
 * by oracle/ref/ into oracle/_ref/) and, with the switch off, state the
 * corrected semantics the GPU library implements.
 *
 * Index space (reference layout, src/MyApp.cpp:71-83,219-235): bodies
 * [0,N), cells (N, N+nodes), root / super-root N+nodes.  pos[3*(N+nodes+1)],
 * mass[N+nodes+1], children[8*(N+nodes+1)] indexed node*8+slot.
 *
 * Build with -ffp-contract=off: every a*b+c below is two roundings unless it
 * is written as fmaf().
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "nboracle.h"

int orc_version(void) { return 1; }

int orc_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------ */
/* Bounding box                                                        */
/* ------------------------------------------------------------------ */

/* True component-wise min/max over all bodies: what boundary_reduce
 * (kernels/boundary_reduce.cl:6-160) is meant to compute. */
void orc_bbox_exact(const float *pos3, long n, float out6[6]) {
    for (int k = 0; k < 3; ++k) {
        float lo = pos3[k], hi = pos3[k];
        uint32_t klo = orc_fkey(lo), khi = klo;
        for (long i = 1; i < n; ++i) {
            float v = pos3[i * 3 + k];
            uint32_t kv = orc_fkey(v);
            if (kv < klo) { klo = kv; lo = v; }
            if (kv > khi) { khi = kv; hi = v; }
        }
        out6[k] = lo;
        out6[3 + k] = hi;
    }
}

/* The box as wired: parallel_reduce_root is handed cl_p
 * (src/MyApp.cpp:282) and reduces p[6l..6l+2] (min slots) and
 * p[6l+3..6l+5] (max slots) for l < workgroup size
 * (kernels/boundary_reduce.cl:112-159). */
void orc_bbox_sampled(const float *p, int wg, float out6[6]) {
    for (int k = 0; k < 6; ++k) out6[k] = p[k];
    for (int l = 1; l < wg; ++l)
        for (int k = 0; k < 3; ++k) {
            float vmin = p[l * 6 + k], vmax = p[l * 6 + 3 + k];
            out6[k] = vmin < out6[k] ? vmin : out6[k];
            out6[3 + k] = out6[3 + k] < vmax ? vmax : out6[3 + k];
        }
}

/* ------------------------------------------------------------------ */
/* Octree build                                                         */
/* ------------------------------------------------------------------ */

/* calculateOctantIdx (kernels/build_tree.hcl:14-29): 2-2*dy/|dy| +
 * 1-dx/|dx| + 0.5-0.5*dz/|dz| is 4*(dy<0) + 2*(dx<0) + (dz<0) for non-zero
 * differences (a difference of exactly zero is NaN there; inputs avoid it).
 * diff<0 is the same predicate as pos<centre for IEEE subtraction. */
static inline int orc_octant_ref(const float p[3], const float bmin[3], const float bmax[3]) {
    float cx = (bmax[0] + bmin[0]) / 2.0f, cy = (bmax[1] + bmin[1]) / 2.0f, cz = (bmax[2] + bmin[2]) / 2.0f;
    return ((p[1] - cy) < 0.0f ? 4 : 0) + ((p[0] - cx) < 0.0f ? 2 : 0) + ((p[2] - cz) < 0.0f ? 1 : 0);
}

/* adjustBoundaryValues (kernels/build_tree.hcl:31-54), including its defect: the y
 * bounds follow the sign of the x difference (:42-46). */
static inline void orc_adjust_ref(const float p[3], float bmin[3], float bmax[3]) {
    float c[3];
    for (int k = 0; k < 3; ++k) c[k] = (bmax[k] + bmin[k]) / 2.0f;
    float dx = p[0] - c[0], dz = p[2] - c[2];
    if (dx > 0) bmin[0] = c[0]; else bmax[0] = c[0];
    if (dx > 0) bmin[1] = c[1]; else bmax[1] = c[1];
    if (dz > 0) bmin[2] = c[2]; else bmax[2] = c[2];
}

/* Geometric semantics (orc_cube, orc_octant_geo, orc_descend_geo in
 * nboracle.h): a cubic root around the box centre with half-width 0.5*max
 * extent (Burtscher), the reference's octant numbering. */
void orc_root_cube(const float box6[6], float out4[4]) {
    float ex = box6[3] - box6[0], ey = box6[4] - box6[1], ez = box6[5] - box6[2];
    float m = ex > ey ? ex : ey;
    m = m > ez ? m : ez;
    out4[0] = (box6[0] + box6[3]) * 0.5f;
    out4[1] = (box6[1] + box6[4]) * 0.5f;
    out4[2] = (box6[2] + box6[5]) * 0.5f;
    out4[3] = 0.5f * m;
}

/* Sequential restatement of build_tree (kernels/build_tree.cl:42-161) in body
 * order.  The octree of distinct points does not depend on insertion order
 * (a cell's box is a function of its path), so this is a valid oracle for
 * the reference's and the GPU's concurrent builds in canonical path form.
 *
 * sem == ORC_SEM_REFERENCE reproduces the dummy level (the first probe at the
 * super-root always takes slot 0, build_tree.cl:57-65), the y-bound defect
 * and the box-halving arithmetic.
 * sem == ORC_SEM_GEOMETRIC: cubic root, no dummy level.
 * Writes children (reference layout), cell centres to node_pos, -1 to cell
 * masses, body_depth[N]; returns the final `bottom` via *bottom_out.
 * Cells are allocated downward from N+nodes-1; `cell <= N` is an overflow
 * (build_tree.cl:109). */
int orc_tree_build(int sem, const float *pos3, int n, int nodes, const float box6[6],
                   float *node_pos, float *node_mass, int *children, int *body_depth,
                   int *bottom_out, int *max_depth_out) {
    const int root = n + nodes;
    const long total = (long)n + nodes + 1;
    for (long i = 0; i < total * 8; ++i) children[i] = ORC_EMPTY;
    int bottom = root;
    int max_depth = 1;
    float rc[4];
    orc_root_cube(box6, rc);
    if (sem == ORC_SEM_REFERENCE) {
        node_pos[root * 3 + 0] = (box6[0] + box6[3]) / 2.0f;
        node_pos[root * 3 + 1] = (box6[1] + box6[4]) / 2.0f;
        node_pos[root * 3 + 2] = (box6[2] + box6[5]) / 2.0f;
    } else {
        node_pos[root * 3 + 0] = rc[0];
        node_pos[root * 3 + 1] = rc[1];
        node_pos[root * 3 + 2] = rc[2];
    }
    node_mass[root] = -1.0f;

    for (int p = 0; p < n; ++p) {
        const float *P = pos3 + (long)p * 3;
        int depth = 0;
        int node = root, slot = 0, child;
        float bmin[3] = {box6[0], box6[1], box6[2]}, bmax[3] = {box6[3], box6[4], box6[5]};
        orc_cube q = {{rc[0], rc[1], rc[2]}, rc[3]};
        if (sem == ORC_SEM_REFERENCE) {
            child = children[node * 8 + 0];
            while (child >= n) {
                node = child;
                slot = orc_octant_ref(P, bmin, bmax);
                child = children[node * 8 + slot];
                orc_adjust_ref(P, bmin, bmax);
                ++depth;
            }
        } else {
            slot = orc_octant_geo(P, &q);
            child = children[node * 8 + slot];
            while (child >= n) {
                node = child;
                orc_descend_geo(P, &q);
                ++depth;
                slot = orc_octant_geo(P, &q);
                child = children[node * 8 + slot];
            }
        }
        if (child == ORC_EMPTY) {
            children[node * 8 + slot] = p;
        } else {
            /* split (build_tree.cl:92-147) */
            const int og = child;
            const float *O = pos3 + (long)og * 3;
            const int locked = node * 8 + slot;
            int patch = -1;
            float omin[3] = {bmin[0], bmin[1], bmin[2]}, omax[3] = {bmax[0], bmax[1], bmax[2]};
            orc_cube oq = q;
            int c2;
            do {
                const int cell = --bottom;
                ++depth;
                if (cell <= n) { *bottom_out = bottom; return ORC_ERR_CELL_OVERFLOW; }
                if (depth > 4 * ORC_MAX_DEPTH) { *bottom_out = bottom; return ORC_ERR_DEPTH; }
                patch = cell > patch ? cell : patch;
                if (sem == ORC_SEM_REFERENCE) {
                    node_pos[cell * 3 + 0] = (bmax[0] + bmin[0]) / 2.0f;
                    node_pos[cell * 3 + 1] = (bmax[1] + bmin[1]) / 2.0f;
                    node_pos[cell * 3 + 2] = (bmax[2] + bmin[2]) / 2.0f;
                } else {
                    /* the new cell is the slot-`slot` child of `node` */
                    orc_descend_geo(P, &q);
                    orc_descend_geo(O, &oq);
                    node_pos[cell * 3 + 0] = q.c[0];
                    node_pos[cell * 3 + 1] = q.c[1];
                    node_pos[cell * 3 + 2] = q.c[2];
                }
                node_mass[cell] = -1.0f;
                if (patch != cell) children[node * 8 + slot] = cell;
                int oslot;
                if (sem == ORC_SEM_REFERENCE) {
                    oslot = orc_octant_ref(O, omin, omax);
                    orc_adjust_ref(O, omin, omax);
                } else {
                    oslot = orc_octant_geo(O, &oq);
                }
                children[cell * 8 + oslot] = og;
                node = cell;
                if (sem == ORC_SEM_REFERENCE) {
                    slot = orc_octant_ref(P, bmin, bmax);
                    orc_adjust_ref(P, bmin, bmax);
                } else {
                    slot = orc_octant_geo(P, &q);
                }
                c2 = children[node * 8 + slot];
            } while (c2 >= 0);
            children[node * 8 + slot] = p;
            children[locked] = patch;
        }
        body_depth[p] = depth;
        if (depth > max_depth) max_depth = depth;
    }
    *bottom_out = bottom;
    *max_depth_out = max_depth;
    return ORC_OK;
}

/* Canonical octant-path form: for every body, the child slots from the
 * root (super-root in reference semantics) down to the body.  paths is
 * [n][maxlen] int8 padded with -1; depth[b] = path length, -1 if the body
 * is not reachable, -2 if its path is longer than maxlen. */
int orc_tree_paths(const int *children, int n, int root, int maxlen, signed char *paths, int *depth) {
    for (long i = 0; i < (long)n * maxlen; ++i) paths[i] = -1;
    for (int i = 0; i < n; ++i) depth[i] = -1;
    int st_node[1024], st_slot[1024];
    signed char cur[1024];
    int sp = 0;
    st_node[0] = root;
    st_slot[0] = 0;
    int found = 0;
    while (sp >= 0) {
        if (st_slot[sp] >= 8) { --sp; continue; }
        int s = st_slot[sp]++;
        int ch = children[(long)st_node[sp] * 8 + s];
        if (ch < 0) continue;
        cur[sp] = (signed char)s;
        if (ch < n) {
            if (depth[ch] != -1) return -1; /* body reachable twice */
            if (sp + 1 > maxlen) { depth[ch] = -2; continue; }
            depth[ch] = sp + 1;
            memcpy(paths + (long)ch * maxlen, cur, sp + 1);
            ++found;
        } else {
            if (sp + 1 >= 1024) return -2;
            ++sp;
            st_node[sp] = ch;
            st_slot[sp] = 0;
        }
    }
    return found;
}

/* ------------------------------------------------------------------ */
/* Centre-of-mass summarisation                                         */
/* ------------------------------------------------------------------ */

/* Restates saturate_tree (kernels/saturate_tree.cl:39-145) bottom-up over
 * cells [bottom, N+nodes] in ascending index (a cell's children were
 * allocated after it, so they have lower indices).  Children are summed in
 * slot order: mass += m_c, centre += x_c*m_c, then centre * (1/mass)
 * (:84-87,129-133).  body_count = sum over child cells of (count-1) plus the
 * number of used slots (:77-80,93).
 * compaction_bug != 0 keeps the reference's defect (the move is skipped when the child's INDEX
 * equals the slot number, :60); 0 compacts correctly. */
int orc_saturate(int compaction_bug, int n, int nodes, int bottom, float *node_pos, float *node_mass,
                 int *children, int *body_count) {
    return orc_saturate_range(compaction_bug, n, bottom, n + nodes, node_pos, node_mass, children, body_count);
}

/* The same over the cells [lo, hi] only, ascending: every child of a cell in
 * the range is a body or a cell below it that is already summarised. */
int orc_saturate_range(int compaction_bug, int n, int lo, int hi, float *node_pos, float *node_mass,
                       int *children, int *body_count) {
    for (int c = lo; c <= hi; ++c) {
        int *row = children + (long)c * 8;
        float M = 0.0f, cx = 0.0f, cy = 0.0f, cz = 0.0f;
        int count = 0, used = 0;
        for (int s = 0; s < 8; ++s) {
            int ch = row[s];
            if (ch < 0) continue;
            int move = compaction_bug ? (ch != used) : (s != used);
            if (move) {
                row[s] = -1;
                row[used] = ch;
            }
            float m = node_mass[ch];
            if (m < 0.0f) return ORC_ERR_ARG; /* child not summarised: order violated */
            if (ch >= n) count += body_count[ch] - 1;
            M = M + m;
            cx = cx + node_pos[ch * 3 + 0] * m;
            cy = cy + node_pos[ch * 3 + 1] * m;
            cz = cz + node_pos[ch * 3 + 2] * m;
            ++used;
        }
        count += used;
        body_count[c] = count;
        float inv = 1.0f / M;
        node_pos[c * 3 + 0] = cx * inv;
        node_pos[c * 3 + 1] = cy * inv;
        node_pos[c * 3 + 2] = cz * inv;
        node_mass[c] = M;
    }
    return ORC_OK;
}

/* Traceless quadrupole of every cell about its centre of mass (an addition:
 * the reference is monopole only).  Bottom-up in slot order:
 * Q += Q_child + m_child (3 d d^T - |d|^2 I), d = x_child - x_cell; a body has
 * Q = 0.  quad[6*node] = {xx, yy, zz, xy, xz, yz}. */
void orc_quadrupoles(int n, int nodes, int bottom, const float *node_pos, const float *node_mass,
                     const int *children, float *quad) {
    for (long i = 0; i < (long)(n + nodes + 1) * 6; ++i) quad[i] = 0.0f;
    orc_quadrupoles_range(n, bottom, n + nodes, node_pos, node_mass, children, quad);
}

/* The same for the cells [lo, hi] only, ascending (children first); the
 * entries of bodies are never read. */
void orc_quadrupoles_range(int n, int lo, int hi, const float *node_pos, const float *node_mass,
                           const int *children, float *quad) {
    for (int c = lo; c <= hi; ++c) {
        const int *row = children + (long)c * 8;
        const float X = node_pos[c * 3 + 0], Y = node_pos[c * 3 + 1], Z = node_pos[c * 3 + 2];
        float q[6] = {0, 0, 0, 0, 0, 0};
        for (int s = 0; s < 8; ++s) {
            const int ch = row[s];
            if (ch < 0) continue;
            const float m = node_mass[ch];
            const float dx = node_pos[ch * 3 + 0] - X, dy = node_pos[ch * 3 + 1] - Y, dz = node_pos[ch * 3 + 2] - Z;
            const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            const float t[6] = {fmaf(3.0f * dx, dx, -r2), fmaf(3.0f * dy, dy, -r2), fmaf(3.0f * dz, dz, -r2),
                                3.0f * dx * dy, 3.0f * dx * dz, 3.0f * dy * dz};
            for (int k = 0; k < 6; ++k) {
                const float own = ch >= n ? quad[(long)ch * 6 + k] : 0.0f;
                q[k] = q[k] + fmaf(m, t[k], own);
            }
        }
        for (int k = 0; k < 6; ++k) quad[(long)c * 6 + k] = q[k];
    }
}

/* ------------------------------------------------------------------ */
/* Sort (the reference's sort.cl is empty)                              */
/* ------------------------------------------------------------------ */

/* In-order body placement from subtree counts (Burtscher's sort): children
 * in slot order, a child cell reserves count[child] places, a child body
 * takes the next one.  That is a depth-first listing of bodies in slot
 * order, computed here with an explicit stack.  Returns bodies placed. */
int orc_sort(const int *children, int n, int root, int *sorted) {
    int st_node[1024], st_slot[1024];
    int sp = 0, k = 0;
    st_node[0] = root;
    st_slot[0] = 0;
    while (sp >= 0) {
        if (st_slot[sp] >= 8) { --sp; continue; }
        int ch = children[(long)st_node[sp] * 8 + st_slot[sp]++];
        if (ch < 0) continue;
        if (ch < n) {
            if (k < n) sorted[k] = ch;
            ++k;
        } else {
            if (sp + 1 >= 1024) return -1;
            ++sp;
            st_node[sp] = ch;
            st_slot[sp] = 0;
        }
    }
    return k;
}

/* ------------------------------------------------------------------ */
/* Barnes-Hut force                                                     */
/* ------------------------------------------------------------------ */

/* Per-depth opening thresholds.
 * ORC_CRIT_REFERENCE (kernels/calculate_forces.cl:45-61): r = half the
 *   largest box extent, dq[0] = r*r/theta (r*r if theta <= 0), dq[i] =
 *   0.25*dq[i-1], then every entry += eps (not eps^2).
 * ORC_CRIT_STANDARD (Burtscher): dq[0] = r*r*(1/theta^2), dq[i] =
 *   0.25*dq[i-1], every entry += eps^2. */
void orc_bh_thresholds(int criterion, const float box6[6], float theta, float eps, int max_depth,
                       float *dq /* ORC_MAX_DEPTH */) {
    float radius = 0.5f * fmaxf(fmaxf(box6[3] - box6[0], box6[4] - box6[1]), box6[5] - box6[2]);
    if (max_depth < 1) max_depth = 1;
    if (max_depth > ORC_MAX_DEPTH) max_depth = ORC_MAX_DEPTH;
    if (criterion == ORC_CRIT_REFERENCE) {
        dq[0] = theta > 0 ? radius * radius / theta : radius * radius;
    } else {
        float itolsq = 1.0f / (theta * theta);
        dq[0] = radius * radius * itolsq;
    }
    float add = criterion == ORC_CRIT_REFERENCE ? eps : eps * eps;
    int i;
    for (i = 1; i < ORC_MAX_DEPTH; ++i) {
        dq[i] = 0.25f * dq[i - 1];
        dq[i - 1] += add;
    }
    dq[i - 1] += add;
}

/* Warp-voted depth-first walk restating calculate_force_local
 * (kernels/calculate_forces.cl:84-147): per group of `vote_width` bodies a
 * shared (node, next-slot) stack; a child body is always accumulated, a
 * child cell is accumulated when EVERY body of the group has
 * d2 >= dq[depth] (work_group_all, :121) and pushed otherwise; an empty
 * slot pops (:140-142).  Groups are consecutive entries of `order`
 * (identity when NULL, i.e. the reference's g_id order); only the first
 * `norder` entries of `order` are walked (a sample of groups).
 *
 * arith == ORC_ARITH_REFERENCE: d2 = eps*eps + dx*dx + dy*dy + dz*dz,
 *   F = m*r*r*r with r = 1/sqrt(d2), acc += diff*F (:117-128).
 * arith == ORC_ARITH_FMA: d2 = fma(dz,dz,fma(dy,dy,fma(dx,dx,eps*eps))),
 *   F = (m*r)*(r*r), acc = fma(diff,F,acc) -- the GPU kernel's arithmetic.
 * skip_self: a body does not interact with itself (the reference includes
 *   the self pair, which adds exactly zero when eps > 0).
 * compensated: per-component TwoSum accumulation (acc = hi + lo).
 * quad: optional cell quadrupoles (6 per node, orc_quadrupoles); accepted
 *   cells then add the softened quadrupole term.
 * stats: optional {body interactions, cell interactions} (per lane).
 * acc3 receives G*acc.  Returns 0, or ORC_ERR_DEPTH on stack overflow. */
int orc_bh_force(const float *node_pos, const float *node_mass, const int *children, int n, int nodes,
                 const float *dq, float eps, float G, int arith, int vote_width, const int *order, int norder,
                 int skip_self, int compensated, const float *quad, long long *stats, float *acc3) {
    const int root = n + nodes;
    if (vote_width < 1 || vote_width > 64) return ORC_ERR_ARG;
    if (!order || norder <= 0 || norder > n) norder = n;
    const int ngroups = (norder + vote_width - 1) / vote_width;
    const float eps2 = eps * eps;
    int err = 0;
#pragma omp parallel for schedule(dynamic, 4)
    for (int g = 0; g < ngroups; ++g) {
        int lanes = norder - g * vote_width;
        if (lanes > vote_width) lanes = vote_width;
        int body[64];
        float px[64], py[64], pz[64];
        float ax[64], ay[64], az[64], lx[64], ly[64], lz[64];
        for (int l = 0; l < lanes; ++l) {
            int b = order ? order[g * vote_width + l] : g * vote_width + l;
            body[l] = b;
            px[l] = node_pos[b * 3 + 0];
            py[l] = node_pos[b * 3 + 1];
            pz[l] = node_pos[b * 3 + 2];
            ax[l] = ay[l] = az[l] = 0.0f;
            lx[l] = ly[l] = lz[l] = 0.0f;
        }
        int st_node[ORC_MAX_DEPTH], st_pos[ORC_MAX_DEPTH];
        int depth = 0;
        st_node[0] = root;
        st_pos[0] = 0;
        int local_err = 0;
        long long nb_body = 0, nb_cell = 0;
        while (depth >= 0 && !local_err) {
            int top;
            while ((top = st_pos[depth]) < 8) {
                int child = children[(long)st_node[depth] * 8 + top];
                st_pos[depth] = top + 1;
                if (child >= 0) {
                    const float cxp = node_pos[child * 3 + 0], cyp = node_pos[child * 3 + 1],
                                czp = node_pos[child * 3 + 2], cm = node_mass[child];
                    float d2v[64], dxv[64], dyv[64], dzv[64];
                    const float thr = dq[depth];
                    int all = 1;
                    /* lane loops are written without early exits so that the
                     * compiler can vectorise them; every lane's arithmetic is
                     * the scalar sequence above, so results do not change */
                    if (arith == ORC_ARITH_REFERENCE) {
                        for (int l = 0; l < lanes; ++l) {
                            const float dx = cxp - px[l], dy = cyp - py[l], dz = czp - pz[l];
                            const float d2 = eps2 + dx * dx + dy * dy + dz * dz;
                            dxv[l] = dx; dyv[l] = dy; dzv[l] = dz; d2v[l] = d2;
                            all &= d2 >= thr;
                        }
                    } else {
                        for (int l = 0; l < lanes; ++l) {
                            const float dx = cxp - px[l], dy = cyp - py[l], dz = czp - pz[l];
                            const float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
                            dxv[l] = dx; dyv[l] = dy; dzv[l] = dz; d2v[l] = d2;
                            all &= d2 >= thr;
                        }
                    }
                    if (child < n || all) {
                        /* F per lane; a body's own entry (skip_self) gets F = 0,
                         * which adds exactly nothing below */
                        float Fv[64], rv[64];
                        int self = 0;
                        for (int l = 0; l < lanes; ++l) {
                            const float r = 1.0f / sqrtf(d2v[l]);
                            float F = arith == ORC_ARITH_REFERENCE ? cm * r * r * r : (cm * r) * (r * r);
                            const int me = skip_self && child == body[l];
                            self += me;
                            rv[l] = r;
                            Fv[l] = me ? 0.0f : F;
                        }
                        if (!compensated) {
                            if (arith == ORC_ARITH_REFERENCE) {
                                for (int l = 0; l < lanes; ++l) {
                                    ax[l] = ax[l] + dxv[l] * Fv[l];
                                    ay[l] = ay[l] + dyv[l] * Fv[l];
                                    az[l] = az[l] + dzv[l] * Fv[l];
                                }
                            } else {
                                for (int l = 0; l < lanes; ++l) {
                                    ax[l] = fmaf(dxv[l], Fv[l], ax[l]);
                                    ay[l] = fmaf(dyv[l], Fv[l], ay[l]);
                                    az[l] = fmaf(dzv[l], Fv[l], az[l]);
                                }
                            }
                        } else {
                            /* TwoSum (Knuth): s = a+b exactly split into s + e */
                            for (int l = 0; l < lanes; ++l) {
                                const float tx = dxv[l] * Fv[l], ty = dyv[l] * Fv[l], tz = dzv[l] * Fv[l];
                                float s, bp, e;
                                s = ax[l] + tx; bp = s - ax[l]; e = (ax[l] - (s - bp)) + (tx - bp); ax[l] = s; lx[l] += e;
                                s = ay[l] + ty; bp = s - ay[l]; e = (ay[l] - (s - bp)) + (ty - bp); ay[l] = s; ly[l] += e;
                                s = az[l] + tz; bp = s - az[l]; e = (az[l] - (s - bp)) + (tz - bp); az[l] = s; lz[l] += e;
                            }
                        }
                        if (quad && child >= n) {
                            /* softened quadrupole of the cell about its centre of mass:
                             * a += 2.5 (d.Q.d) d / r^7 - Q d / r^5, d = x_cell - x_body */
                            const float *Q = quad + (long)child * 6; /* xx yy zz xy xz yz */
                            const float Qxx = Q[0], Qyy = Q[1], Qzz = Q[2], Qxy = Q[3], Qxz = Q[4], Qyz = Q[5];
                            for (int l = 0; l < lanes; ++l) {
                                const float dx = dxv[l], dy = dyv[l], dz = dzv[l], r = rv[l];
                                const float qx = fmaf(Qxz, dz, fmaf(Qxy, dy, Qxx * dx));
                                const float qy = fmaf(Qyz, dz, fmaf(Qyy, dy, Qxy * dx));
                                const float qz = fmaf(Qzz, dz, fmaf(Qyz, dy, Qxz * dx));
                                const float sq = fmaf(dz, qz, fmaf(dy, qy, dx * qx));
                                const float r2i = r * r;
                                const float r5 = (r * r2i) * r2i;
                                const float c1 = (2.5f * sq) * (r5 * r2i);
                                const float ux = fmaf(dx, c1, -qx * r5), uy = fmaf(dy, c1, -qy * r5),
                                            uz = fmaf(dz, c1, -qz * r5);
                                if (!compensated) {
                                    ax[l] += ux; ay[l] += uy; az[l] += uz;
                                } else {
                                    float s, bp, e;
                                    s = ax[l] + ux; bp = s - ax[l]; e = (ax[l] - (s - bp)) + (ux - bp); ax[l] = s; lx[l] += e;
                                    s = ay[l] + uy; bp = s - ay[l]; e = (ay[l] - (s - bp)) + (uy - bp); ay[l] = s; ly[l] += e;
                                    s = az[l] + uz; bp = s - az[l]; e = (az[l] - (s - bp)) + (uz - bp); az[l] = s; lz[l] += e;
                                }
                            }
                        }
                        if (stats) {
                            if (child < n) nb_body += lanes - self;
                            else nb_cell += lanes - self;
                        }
                    } else {
                        ++depth;
                        if (depth >= ORC_MAX_DEPTH) { local_err = 1; break; }
                        st_node[depth] = child;
                        st_pos[depth] = 0;
                    }
                } else {
                    depth = depth - 1 > 0 ? depth - 1 : 0;
                }
            }
            --depth;
        }
        if (local_err) {
#pragma omp atomic write
            err = ORC_ERR_DEPTH;
        }
        if (stats) {
#pragma omp atomic
            stats[0] += nb_body;
#pragma omp atomic
            stats[1] += nb_cell;
        }
        for (int l = 0; l < lanes; ++l) {
            float x = ax[l], y = ay[l], z = az[l];
            if (compensated) { x = x + lx[l]; y = y + ly[l]; z = z + lz[l]; }
            acc3[body[l] * 3 + 0] = x * G;
            acc3[body[l] * 3 + 1] = y * G;
            acc3[body[l] * 3 + 2] = z * G;
        }
    }
    return err;
}

/* ------------------------------------------------------------------ */
/* Direct sums                                                          */
/* ------------------------------------------------------------------ */

/* Plummer-softened gravity, the physics both the reference's BH kernel
 * (kernels/calculate_forces.cl:117-128) uses:
 * a_i = G * sum_{j != i} m_j r_ij (|r_ij|^2 + eps^2)^{-3/2}, FP32 with the
 * GPU kernel's FMA arithmetic, j ascending. */
void orc_direct_fp32(const float *pos3, const float *mass, int n, float eps, float G, int i0, int i1,
                     float *acc3) {
    const float eps2 = eps * eps;
#pragma omp parallel for schedule(static)
    for (int i = i0; i < i1; ++i) {
        float px = pos3[i * 3 + 0], py = pos3[i * 3 + 1], pz = pos3[i * 3 + 2];
        float ax = 0.0f, ay = 0.0f, az = 0.0f;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            float dx = pos3[j * 3 + 0] - px, dy = pos3[j * 3 + 1] - py, dz = pos3[j * 3 + 2] - pz;
            float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
            float r = 1.0f / sqrtf(d2);
            float F = (mass[j] * r) * (r * r);
            ax = fmaf(dx, F, ax);
            ay = fmaf(dy, F, ay);
            az = fmaf(dz, F, az);
        }
        acc3[i * 3 + 0] = ax * G;
        acc3[i * 3 + 1] = ay * G;
        acc3[i * 3 + 2] = az * G;
    }
}

/* The same sum in FP64 for the listed targets (accuracy oracle). */
void orc_direct_fp64(const float *pos3, const float *mass, int n, double eps, double G, const int *targets,
                     int nt, double *acc3) {
    const double eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16)
    for (int t = 0; t < nt; ++t) {
        int i = targets ? targets[t] : t;
        double px = pos3[i * 3 + 0], py = pos3[i * 3 + 1], pz = pos3[i * 3 + 2];
        double ax = 0.0, ay = 0.0, az = 0.0;
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            double dx = (double)pos3[j * 3 + 0] - px, dy = (double)pos3[j * 3 + 1] - py,
                   dz = (double)pos3[j * 3 + 2] - pz;
            double d2 = dx * dx + dy * dy + dz * dz + eps2;
            double r = 1.0 / sqrt(d2);
            double F = (double)mass[j] * r * r * r;
            ax += dx * F;
            ay += dy * F;
            az += dz * F;
        }
        acc3[t * 3 + 0] = ax * G;
        acc3[t * 3 + 1] = ay * G;
        acc3[t * 3 + 2] = az * G;
    }
}

/* normalize as the OpenCL built-in with its zero-vector special case. */
static inline void orc_normalize(float v[3]) {
    float l2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (l2 == 0.0f) return;
    float inv = 1.0f / sqrtf(l2);
    v[0] = v[0] * inv; v[1] = v[1] * inv; v[2] = v[2] * inv;
}

/* calc_body_body / the inner loop of update: d = normalize(pj - pi),
 * dist_sqr = |d|^2 + eps^2, s = m_j / pow(dist_sqr, 3/2) with 3/2 == 1
 * (kernels/brute_force_update.cl:54-60,114-123). */
static inline void orc_quirk_pair(const float *pi, const float *pj, float mj, float eps, float a[3]) {
    float d[3] = {pj[0] - pi[0], pj[1] - pi[1], pj[2] - pi[2]};
    orc_normalize(d);
    float dist_sqr = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + eps * eps;
    float s = mj / powf(dist_sqr, 1.0f);
    a[0] = a[0] + d[0] * s;
    a[1] = a[1] + d[1] * s;
    a[2] = a[2] + d[2] * s;
}

/* update (kernels/brute_force_update.cl:31-63): every j != i, eps 0.01. */
void orc_direct_quirk_global(const float *pos3, const float *mass, int n, float G, float *acc3) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        float a[3] = {0.0f, 0.0f, 0.0f};
        for (int j = 0; j < n; ++j) {
            if (j == i) continue;
            orc_quirk_pair(pos3 + i * 3, pos3 + j * 3, mass[j], 0.01f, a);
        }
        acc3[i * 3 + 0] = a[0] * G;
        acc3[i * 3 + 1] = a[1] * G;
        acc3[i * 3 + 2] = a[2] * G;
    }
}

/* update_local (kernels/brute_force_update.cl:144-185), eps 0.1.
 * tile_schedule != 0 restates the tile schedule as written, defined for
 * n % wg == 0: iteration 0 loads tile 0 and skips j == i; iteration t >= 1
 * loads tile t-1 and skips slot j when i == t*wg + j; N/wg + 1 iterations.
 * tile_schedule == 0: every j != i once, ascending. */
int orc_direct_quirk_local(const float *pos3, const float *mass, int n, int wg, int tile_schedule, float G, float *acc3) {
    if (tile_schedule && (wg <= 0 || n % wg != 0)) return ORC_ERR_ARG;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        float a[3] = {0.0f, 0.0f, 0.0f};
        if (!tile_schedule) {
            for (int j = 0; j < n; ++j)
                if (j != i) orc_quirk_pair(pos3 + i * 3, pos3 + j * 3, mass[j], 0.1f, a);
        } else {
            int iters = n / wg + 1;
            for (int t = 0; t < iters; ++t) {
                int tile = t == 0 ? 0 : t - 1;
                for (int j = 0; j < wg; ++j) {
                    if (i == t * wg + j) continue;
                    int b = tile * wg + j;
                    orc_quirk_pair(pos3 + i * 3, pos3 + b * 3, mass[b], 0.1f, a);
                }
            }
        }
        acc3[i * 3 + 0] = a[0] * G;
        acc3[i * 3 + 1] = a[1] * G;
        acc3[i * 3 + 2] = a[2] * G;
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* Integrators (kernels/calculate_forces.cl:150-182,                   */
/* kernels/brute_force_update.cl:69-101)                                */
/* ------------------------------------------------------------------ */

/* method ORC_EULER: accs = a; v = v + a*dt; x = x + v*dt.
 * method ORC_LEAPFROG as written: vh = v + accs*dt*0.5; x = x + vh*dt;
 *   v = vh + a*dt*0.5; accs is read but not written.
 * method ORC_KDK (the corrected leapfrog, an opt-in deviation): velocities
 *   live at half steps; v += a*dt on a primed step, a*dt*0.5 on the first;
 *   x = x + v*dt; accs = a.  `primed` says which.
 * Any other method changes nothing (the as-wired BH path binds NumberOfBodies as the method). */
void orc_integrate(int method, int primed, int n, float dt, const float *acc_new3, float *accs3, float *vel3,
                   float *pos3, int pos_stride) {
#pragma omp parallel for schedule(static) if (n >= 65536)
    for (int i = 0; i < n; ++i) {
        float *x = pos3 + (long)i * pos_stride, *v = vel3 + i * 3, *ap = accs3 + i * 3;
        const float *a = acc_new3 + i * 3;
        if (method == ORC_EULER) {
            for (int k = 0; k < 3; ++k) {
                ap[k] = a[k];
                v[k] = v[k] + a[k] * dt;
                x[k] = x[k] + v[k] * dt;
            }
        } else if (method == ORC_LEAPFROG) {
            for (int k = 0; k < 3; ++k) {
                float vh = v[k] + ap[k] * dt * 0.5f;
                x[k] = x[k] + vh * dt;
                v[k] = vh + a[k] * dt * 0.5f;
            }
        } else if (method == ORC_KDK) {
            float h = primed ? dt : dt * 0.5f;
            for (int k = 0; k < 3; ++k) {
                ap[k] = a[k];
                v[k] = v[k] + a[k] * h;
                x[k] = x[k] + v[k] * dt;
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Collision (kernels/collision_update.cl:3-82)                          */
/* ------------------------------------------------------------------ */

/* calc_collision_traj (:3-15): if |pi - pj| > ri + rj keep v, else reflect
 * v <- v - 2 dot(n, v) n with n = normalize(pj - pi).  Reflections apply in
 * j order to the running v_i; positions are read-only.  Radii are 0.015
 * (:59,65).  tile_schedule != 0 uses update_local's tile schedule as written (n % wg == 0);
 * otherwise every j != i once, ascending. */
int orc_collision(const float *pos3, float *vel3, int n, int wg, int tile_schedule) {
    if (tile_schedule && (wg <= 0 || n % wg != 0)) return ORC_ERR_ARG;
    const float rr = 0.015f + 0.015f;
    float *out = (float *)malloc(sizeof(float) * 3 * (size_t)n);
    if (!out) return ORC_ERR_ARG;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const float *pi = pos3 + i * 3;
        float v[3] = {vel3[i * 3 + 0], vel3[i * 3 + 1], vel3[i * 3 + 2]};
        int iters = tile_schedule ? n / wg + 1 : 1;
        for (int t = 0; t < iters; ++t) {
            int tile = t == 0 ? 0 : t - 1;
            int jn = tile_schedule ? wg : n;
            for (int j = 0; j < jn; ++j) {
                int b;
                if (tile_schedule) {
                    if (i == t * wg + j) continue;
                    b = tile * wg + j;
                } else {
                    if (j == i) continue;
                    b = j;
                }
                const float *pj = pos3 + b * 3;
                float d[3] = {pj[0] - pi[0], pj[1] - pi[1], pj[2] - pi[2]};
                float nrm[3] = {d[0], d[1], d[2]};
                orc_normalize(nrm);
                float e[3] = {pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]};
                float dist = sqrtf(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                if (dist > rr) continue;
                float dp = nrm[0] * v[0] + nrm[1] * v[1] + nrm[2] * v[2];
                float k2 = 2.0f * dp;
                v[0] = v[0] - k2 * nrm[0];
                v[1] = v[1] - k2 * nrm[1];
                v[2] = v[2] - k2 * nrm[2];
            }
        }
        out[i * 3 + 0] = v[0];
        out[i * 3 + 1] = v[1];
        out[i * 3 + 2] = v[2];
    }
    memcpy(vel3, out, sizeof(float) * 3 * (size_t)n);
    free(out);
    return ORC_OK;
}

/* copy_vertices (kernels/copy_vertices.cl:12-16): float4{x,y,z,1}. */
void orc_copy_vertices(const float *pos3, int n, float *out4) {
    for (int i = 0; i < n; ++i) {
        out4[i * 4 + 0] = pos3[i * 3 + 0];
        out4[i * 4 + 1] = pos3[i * 3 + 1];
        out4[i * 4 + 2] = pos3[i * 3 + 2];
        out4[i * 4 + 3] = 1.0f;
    }
}
