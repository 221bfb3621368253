/*
 * nbpipeline.c -- TEST INFRASTRUCTURE: the oracle's kernels run as one whole
 * Barnes-Hut step on every host core.  This is the timed CPU baseline (the
 * reference's step as a CPU program: bbox -> init+build -> saturate -> sort
 * -> force+integrate, sequenced as CMyApp::Update does in src/MyApp.cpp:583-600)
 * and nothing else; nothing in the product links or calls it.
 *
 * Results are those of the sequential restatement in nboracle.c, bit for
 * bit: the same tree (a cell's box is a function of its path, so the octree
 * of distinct points does not depend on the order or grouping of the
 * insertions), the same slot-order sums, the same walk.  Only the numbering
 * of the cells differs.  How the work is split:
 *
 *   bbox       per-thread min/max keys, combined (exact, order-free);
 *   build      every body's region among the 8^L cubes of level L is found
 *              in parallel; the cells of levels 1..L-1 follow from the region
 *              counts (a cell exists exactly where two or more bodies share
 *              its cube); each level-L region with two or more bodies is
 *              built by one thread into a private buffer, with the
 *              insertions of orc_tree_build (kernels/build_tree.cl:42-161),
 *              then renumbered into one contiguous range of cell indices;
 *   saturate   and the quadrupoles: the regions' ranges in parallel, then
 *              the top cells (orc_saturate_range, kernels/saturate_tree.cl:39-145);
 *   sort       the top cells' depth-first order gives each region its first
 *              place; the regions are listed in parallel (orc_sort);
 *   force      orc_bh_force over the sorted bodies (OpenMP over warp groups,
 *              kernels/calculate_forces.cl:84-147); Euler update
 *              (kernels/calculate_forces.cl:168-181) in parallel.
 *
 * Geometric tree semantics and the standard opening criterion only: the
 * configuration the GPU library's bench runs.
 *
 * Also here: the seeded initial-condition streams of the library's generator
 * (normal positions, equal or lognormal masses), restated so that the CPU
 * baseline builds the same input bytes without loading the library.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "nboracle.h"

/* ------------------------------------------------------------------ */
/* Seeded initial conditions                                            */
/* ------------------------------------------------------------------ */

/* SplitMix64 counter stream, uniforms in (0, 1], Box-Muller normals in
 * double with the sine kept as the next normal: the streams of
 * nbodysimulation_gb300/csrc/ic.cpp (nb_generate_ic), read in one
 * sequential pass (which is the sequence its parallel chunks produce). */
typedef struct { uint64_t s; int have; double spare; } orc_normal;

static const uint64_t ORC_GOLDEN = 0x9E3779B97F4A7C15ULL;

static inline uint64_t orc_sm_next(uint64_t *s) {
    uint64_t z = (*s += ORC_GOLDEN);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline double orc_uniform(uint64_t *s) { return ((orc_sm_next(s) >> 11) + 1) * (1.0 / 9007199254740992.0); }
static inline double orc_normal_next(orc_normal *g) {
    if (g->have) {
        g->have = 0;
        return g->spare;
    }
    const double u1 = orc_uniform(&g->s), u2 = orc_uniform(&g->s);
    const double rad = sqrt(-2.0 * log(u1));
    const double a = 6.283185307179586 * u2;
    g->spare = rad * sin(a);
    g->have = 1;
    return rad * cos(a);
}

enum { ORC_POS_UNIFORM = 1, ORC_POS_NORMAL_SIGMA = 3 };
enum { ORC_MASS_EQUAL = 1, ORC_MASS_LOGNORMAL = 2 };

/* pos_mode ORC_POS_UNIFORM: normal(0, R) per axis (the library's
 * NB_UNIFORM_POS, src/MyApp.cpp:384-396); ORC_POS_NORMAL_SIGMA: normal(0,
 * sigma[k]) per axis.  mass_mode ORC_MASS_EQUAL: 1/n; ORC_MASS_LOGNORMAL:
 * exp(msigma * normal) normalised to a total of 1.  Returns 0, or
 * ORC_ERR_ARG for a mode the restatement does not cover. */
int orc_generate_ic(int n, uint64_t seed, int pos_mode, const float sigma[3], float R, int mass_mode, float msigma,
                    float *pos3, float *mass) {
    if (n < 0) return ORC_ERR_ARG;
    if (pos3) {
        orc_normal g = {seed ^ 0x706f736974696f6eULL, 0, 0.0};
        if (pos_mode == ORC_POS_NORMAL_SIGMA) {
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) pos3[3 * i + k] = (float)((double)sigma[k] * orc_normal_next(&g));
        } else if (pos_mode == ORC_POS_UNIFORM) {
            for (long i = 0; i < 3L * n; ++i) pos3[i] = (float)((double)R * orc_normal_next(&g));
        } else {
            return ORC_ERR_ARG;
        }
    }
    if (mass) {
        if (mass_mode == ORC_MASS_EQUAL) {
            for (int i = 0; i < n; ++i) mass[i] = 1.0f / (float)n;
        } else if (mass_mode == ORC_MASS_LOGNORMAL) {
            double *m = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
            if (!m) return ORC_ERR_ARG;
            orc_normal g = {seed ^ 0x6d61737365730000ULL, 0, 0.0};
            double tot = 0.0;
            for (int i = 0; i < n; ++i) m[i] = exp((double)msigma * orc_normal_next(&g));
            for (int i = 0; i < n; ++i) tot += m[i];
            for (int i = 0; i < n; ++i) mass[i] = (float)(m[i] / tot);
            free(m);
        } else {
            return ORC_ERR_ARG;
        }
    }
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* The parallel step                                                    */
/* ------------------------------------------------------------------ */

typedef struct {
    int *row; /* 8 ints per local cell: a body, -1, or n + local cell */
    long used, cap;
} orc_lbuf;

typedef struct {
    int n, nodes, levels, nreg, threads;
    float *node_pos, *node_mass, *quad, *acc_new;
    int *children, *body_count, *sorted;
    int *region_of, *reg_bodies, *reg_start;     /* n, n, nreg + 1 */
    int *cnt;                                    /* counts of every level: (8^(L+1) - 1) / 7 entries */
    int *top_idx;                                /* cell index of each region of levels 0..L-1 (-1: none) */
    int *reg_hi, *reg_cells, *reg_thread;        /* per level-L region: root cell, cell count, builder */
    long *reg_off;                               /* per level-L region: offset of its rows in its builder's buffer */
    int *reg_place;                              /* per level-L region: first place in the sorted order */
    int *reg_err;                                /* per level-L region: build status */
    orc_lbuf *buf;                               /* per thread */
    int top_lo, bottom, max_depth;
} orc_pipe;

static long orc_level_base(int l) { return ((1L << (3 * l)) - 1) / 7; } /* regions of the levels above l */

static int orc_pipe_levels(int n) {
    int l = 1;
    while (l < 5 && (256L << (3 * (l + 1))) <= (long)n) ++l;
    return l;
}

void orc_pipe_destroy(void *vp) {
    orc_pipe *p = (orc_pipe *)vp;
    if (!p) return;
    free(p->node_pos); free(p->node_mass); free(p->quad); free(p->acc_new);
    free(p->children); free(p->body_count); free(p->sorted);
    free(p->region_of); free(p->reg_bodies); free(p->reg_start); free(p->cnt); free(p->top_idx);
    free(p->reg_hi); free(p->reg_cells); free(p->reg_thread); free(p->reg_off); free(p->reg_place);
    free(p->reg_err);
    if (p->buf)
        for (int t = 0; t < p->threads; ++t) free(p->buf[t].row);
    free(p->buf);
    free(p);
}

/* A pipeline for n bodies and a budget of `nodes` cell slots (the reference's
 * index space: bodies [0,n), cells (n, n+nodes), root n+nodes). */
void *orc_pipe_create(int n, int nodes) {
    if (n < 2 || nodes < 2) return NULL;
    orc_pipe *p = (orc_pipe *)calloc(1, sizeof(orc_pipe));
    if (!p) return NULL;
    p->n = n;
    p->nodes = nodes;
    p->levels = orc_pipe_levels(n);
    p->nreg = 1 << (3 * p->levels);
#ifdef _OPENMP
    p->threads = omp_get_max_threads();
#else
    p->threads = 1;
#endif
    const size_t total = (size_t)n + (size_t)nodes + 1;
    const long levels_total = orc_level_base(p->levels + 1);
    p->node_pos = (float *)malloc(sizeof(float) * 3 * total);
    p->node_mass = (float *)malloc(sizeof(float) * total);
    p->quad = (float *)malloc(sizeof(float) * 6 * total);
    p->acc_new = (float *)malloc(sizeof(float) * 3 * (size_t)n);
    p->children = (int *)malloc(sizeof(int) * 8 * total);
    p->body_count = (int *)malloc(sizeof(int) * total);
    p->sorted = (int *)malloc(sizeof(int) * (size_t)n);
    p->region_of = (int *)malloc(sizeof(int) * (size_t)n);
    p->reg_bodies = (int *)malloc(sizeof(int) * (size_t)n);
    p->reg_start = (int *)malloc(sizeof(int) * (size_t)(p->nreg + 1));
    p->cnt = (int *)malloc(sizeof(int) * (size_t)levels_total);
    p->top_idx = (int *)malloc(sizeof(int) * (size_t)orc_level_base(p->levels));
    p->reg_hi = (int *)malloc(sizeof(int) * (size_t)p->nreg);
    p->reg_cells = (int *)malloc(sizeof(int) * (size_t)p->nreg);
    p->reg_thread = (int *)malloc(sizeof(int) * (size_t)p->nreg);
    p->reg_off = (long *)malloc(sizeof(long) * (size_t)p->nreg);
    p->reg_place = (int *)malloc(sizeof(int) * (size_t)p->nreg);
    p->reg_err = (int *)malloc(sizeof(int) * (size_t)p->nreg);
    p->buf = (orc_lbuf *)calloc((size_t)p->threads, sizeof(orc_lbuf));
    if (!p->node_pos || !p->node_mass || !p->quad || !p->acc_new || !p->children || !p->body_count ||
        !p->sorted || !p->region_of || !p->reg_bodies || !p->reg_start || !p->cnt || !p->top_idx || !p->reg_hi ||
        !p->reg_cells || !p->reg_thread || !p->reg_off || !p->reg_place || !p->reg_err || !p->buf) {
        orc_pipe_destroy(p);
        return NULL;
    }
    return p;
}

static long orc_lbuf_cell(orc_lbuf *b) {
    if (b->used == b->cap) {
        long cap = b->cap ? 2 * b->cap : 4096;
        int *row = (int *)realloc(b->row, sizeof(int) * 8 * (size_t)cap);
        if (!row) return -1;
        b->row = row;
        b->cap = cap;
    }
    int *r = b->row + 8 * b->used;
    for (int s = 0; s < 8; ++s) r[s] = ORC_EMPTY;
    return b->used++;
}

/* Inserts the k bodies `list` into a new subtree whose root cell has cube rq,
 * as orc_tree_build inserts below a cell (geometric semantics).  Local cells
 * are numbered from 0 (the root) in creation order, so a parent's number is
 * below its children's; slots hold bodies, -1 or n + local cell.  *cells
 * gets the number of cells, *depth the deepest body's cell count below rq. */
static int orc_build_region(const float *pos3, int n, const int *list, int k, orc_cube rq, orc_lbuf *b, long *off,
                            int *cells, int *depth_out) {
    const long base = b->used;
    if (orc_lbuf_cell(b) < 0) return ORC_ERR_ARG;
    int dmax = 0;
    for (int i = 0; i < k; ++i) {
        const int p = list[i];
        const float *P = pos3 + (long)p * 3;
        orc_cube q = rq;
        long node = 0;
        int depth = 0;
        int slot = orc_octant_geo(P, &q);
        int child = b->row[8 * (base + node) + slot];
        while (child >= n) {
            node = child - n;
            orc_descend_geo(P, &q);
            ++depth;
            slot = orc_octant_geo(P, &q);
            child = b->row[8 * (base + node) + slot];
        }
        if (child != ORC_EMPTY) { /* split until the two bodies part (build_tree.cl:92-147) */
            const int og = child;
            const float *O = pos3 + (long)og * 3;
            orc_cube oq = q;
            int c2;
            do {
                const long cell = orc_lbuf_cell(b);
                if (cell < 0) return ORC_ERR_ARG;
                const long local = cell - base;
                if (++depth > 4 * ORC_MAX_DEPTH) return ORC_ERR_DEPTH;
                orc_descend_geo(P, &q);
                orc_descend_geo(O, &oq);
                b->row[8 * (base + node) + slot] = n + (int)local;
                b->row[8 * cell + orc_octant_geo(O, &oq)] = og;
                node = local;
                slot = orc_octant_geo(P, &q);
                c2 = b->row[8 * cell + slot];
            } while (c2 >= 0);
        }
        b->row[8 * (base + node) + slot] = p;
        if (depth > dmax) dmax = depth;
    }
    *off = base;
    *cells = (int)(b->used - base);
    *depth_out = dmax;
    return ORC_OK;
}

/* Depth-first listing of the top cells in slot order: bodies that sit in a
 * top cell take the next place, a level-L region of two or more bodies
 * takes as many places as it holds (orc_sort's order). */
static void orc_top_places(orc_pipe *p, int l, long r, int *k) {
    const int L = p->levels;
    for (int s = 0; s < 8; ++s) {
        const long sub = 8 * r + s;
        const int c = p->cnt[orc_level_base(l + 1) + sub];
        if (c == 0) continue;
        if (c == 1) {
            const long first_region = sub << (3 * (L - l - 1));
            p->sorted[(*k)++] = p->reg_bodies[p->reg_start[first_region]];
        } else if (l + 1 < L) {
            orc_top_places(p, l + 1, sub, k);
        } else {
            p->reg_place[sub] = *k;
            *k += c;
        }
    }
}

static double orc_now(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

/* One step of the system in place: bbox, build, saturate (+ quadrupoles),
 * sort, the warp-voted walk (vote width 32, standard criterion, FMA
 * arithmetic) of every body in sorted order, then the Euler update of
 * pos3/vel3 with acc3 <- the new accelerations.  stage_s (optional, 6):
 * seconds of bbox, build, saturate, sort, force, integrate.  stats
 * (optional, 2): body and cell interactions.  Returns 0 or an ORC_ERR_*. */
int orc_pipe_step(void *vp, float *pos3, float *vel3, float *acc3, const float *mass, float theta, float eps,
                  float G, float dt, int quadrupole, int compensated, double *stage_s, long long *stats) {
    orc_pipe *p = (orc_pipe *)vp;
    if (!p) return ORC_ERR_ARG;
    const int n = p->n, L = p->levels, nreg = p->nreg;
    const int root = n + p->nodes;
    double t[7];
    t[0] = orc_now();

    /* bbox: exact min/max per axis through order-preserving keys */
    uint32_t klo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, khi[3] = {0, 0, 0};
#pragma omp parallel
    {
        uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0, 0, 0};
#pragma omp for schedule(static) nowait
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                const uint32_t v = orc_fkey(pos3[3 * (long)i + k]);
                lo[k] = v < lo[k] ? v : lo[k];
                hi[k] = v > hi[k] ? v : hi[k];
            }
#pragma omp critical
        for (int k = 0; k < 3; ++k) {
            klo[k] = lo[k] < klo[k] ? lo[k] : klo[k];
            khi[k] = hi[k] > khi[k] ? hi[k] : khi[k];
        }
    }
    float box[6];
    for (int k = 0; k < 3; ++k) {
        uint32_t a = (klo[k] & 0x80000000u) ? (klo[k] & 0x7fffffffu) : ~klo[k];
        uint32_t b = (khi[k] & 0x80000000u) ? (khi[k] & 0x7fffffffu) : ~khi[k];
        memcpy(&box[k], &a, 4);
        memcpy(&box[3 + k], &b, 4);
    }
    t[1] = orc_now();

    /* build: bodies into the node arrays, level-L regions, region counts */
    float rc[4];
    orc_root_cube(box, rc);
    const orc_cube rootq = {{rc[0], rc[1], rc[2]}, rc[3]};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const float *P = pos3 + 3 * (long)i;
        p->node_pos[3 * (long)i + 0] = P[0];
        p->node_pos[3 * (long)i + 1] = P[1];
        p->node_pos[3 * (long)i + 2] = P[2];
        p->node_mass[i] = mass[i];
        orc_cube q = rootq;
        int r = 0;
        for (int l = 0; l < L; ++l) {
            r = 8 * r + orc_octant_geo(P, &q);
            orc_descend_geo(P, &q);
        }
        p->region_of[i] = r;
    }
    int *cl = p->cnt + orc_level_base(L);
    memset(cl, 0, sizeof(int) * (size_t)nreg);
    for (int i = 0; i < n; ++i) ++cl[p->region_of[i]];
    p->reg_start[0] = 0;
    for (int r = 0; r < nreg; ++r) p->reg_start[r + 1] = p->reg_start[r] + cl[r];
    {
        int *fill = p->reg_hi; /* scratch: next free place per region */
        memcpy(fill, p->reg_start, sizeof(int) * (size_t)nreg);
        for (int i = 0; i < n; ++i) p->reg_bodies[fill[p->region_of[i]]++] = i;
    }
    for (int l = L - 1; l >= 0; --l) {
        int *up = p->cnt + orc_level_base(l), *dn = p->cnt + orc_level_base(l + 1);
        for (long r = 0; r < (1L << (3 * l)); ++r) {
            int s = 0;
            for (int c = 0; c < 8; ++c) s += dn[8 * r + c];
            up[r] = s;
        }
    }
    /* the level-L regions of two or more bodies, each built by one thread */
    for (int tt = 0; tt < p->threads; ++tt) p->buf[tt].used = 0;
    int depth_max = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : depth_max)
    for (int r = 0; r < nreg; ++r) {
        p->reg_cells[r] = 0;
        p->reg_err[r] = ORC_OK;
        const int k = cl[r];
        if (k < 2) continue;
#ifdef _OPENMP
        const int tid = omp_get_thread_num();
#else
        const int tid = 0;
#endif
        orc_cube q = rootq;
        for (int l = L - 1; l >= 0; --l) { /* the region's cube: descend by its path digits */
            const int o = (r >> (3 * l)) & 7;
            const float P[3] = {(o & 2) ? q.c[0] - q.r : q.c[0] + q.r, (o & 4) ? q.c[1] - q.r : q.c[1] + q.r,
                                (o & 1) ? q.c[2] - q.r : q.c[2] + q.r};
            orc_descend_geo(P, &q);
        }
        int d = 0;
        p->reg_thread[r] = tid;
        p->reg_err[r] = orc_build_region(pos3, n, p->reg_bodies + p->reg_start[r], k, q, &p->buf[tid], &p->reg_off[r],
                                         &p->reg_cells[r], &d);
        depth_max = d > depth_max ? d : depth_max;
    }
    for (int r = 0; r < nreg; ++r)
        if (p->reg_err[r] != ORC_OK) return p->reg_err[r];
    /* cell numbers: the root, the top cells level by level, then each
     * region's range (root of the range at its top): parents above children */
    int bottom = root;
    for (int l = 0; l < L; ++l) {
        const int *c = p->cnt + orc_level_base(l);
        int *ti = p->top_idx + orc_level_base(l);
        for (long r = 0; r < (1L << (3 * l)); ++r) ti[r] = l == 0 ? root : (c[r] >= 2 ? --bottom : -1);
    }
    p->top_lo = bottom;
    for (int r = 0; r < nreg; ++r) {
        if (p->reg_cells[r] == 0) {
            p->reg_hi[r] = -1;
            continue;
        }
        p->reg_hi[r] = bottom - 1;
        bottom -= p->reg_cells[r];
    }
    if (bottom <= n) return ORC_ERR_CELL_OVERFLOW;
    p->bottom = bottom;
    p->max_depth = L + depth_max;
    /* top cells' rows */
    for (int l = 0; l < L; ++l) {
        const int *ti = p->top_idx + orc_level_base(l);
        const int *cn = p->cnt + orc_level_base(l + 1);
        for (long r = 0; r < (1L << (3 * l)); ++r) {
            if (ti[r] < 0) continue;
            int *row = p->children + 8 * (long)ti[r];
            for (int s = 0; s < 8; ++s) {
                const long sub = 8 * r + s;
                const int c = cn[sub];
                if (c == 0) row[s] = ORC_EMPTY;
                else if (c == 1) row[s] = p->reg_bodies[p->reg_start[sub << (3 * (L - l - 1))]];
                else row[s] = l + 1 < L ? p->top_idx[orc_level_base(l + 1) + sub] : p->reg_hi[sub];
            }
        }
    }
    /* the regions' rows, renumbered: local cell j -> reg_hi - j */
#pragma omp parallel for schedule(dynamic, 4)
    for (int r = 0; r < nreg; ++r) {
        const int cells = p->reg_cells[r];
        if (!cells) continue;
        const int hi = p->reg_hi[r];
        const int *src = p->buf[p->reg_thread[r]].row + 8 * p->reg_off[r];
        for (int j = 0; j < cells; ++j) {
            int *row = p->children + 8 * (long)(hi - j);
            for (int s = 0; s < 8; ++s) {
                const int v = src[8 * j + s];
                row[s] = v >= n ? hi - (v - n) : v;
            }
        }
    }
    t[2] = orc_now();

    /* saturate (+ quadrupoles): the regions, then the top cells */
    int sat_err = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : sat_err)
    for (int r = 0; r < nreg; ++r) {
        const int cells = p->reg_cells[r];
        if (!cells) continue;
        const int hi = p->reg_hi[r], lo = hi - cells + 1;
        sat_err |= orc_saturate_range(0, n, lo, hi, p->node_pos, p->node_mass, p->children, p->body_count);
        if (quadrupole) orc_quadrupoles_range(n, lo, hi, p->node_pos, p->node_mass, p->children, p->quad);
    }
    if (sat_err) return ORC_ERR_ARG;
    if (orc_saturate_range(0, n, p->top_lo, root, p->node_pos, p->node_mass, p->children, p->body_count))
        return ORC_ERR_ARG;
    if (quadrupole) orc_quadrupoles_range(n, p->top_lo, root, p->node_pos, p->node_mass, p->children, p->quad);
    t[3] = orc_now();

    /* sort: places of the top cells' bodies and regions, then each region */
    int k = 0;
    orc_top_places(p, 0, 0, &k);
    if (k != n) return ORC_ERR_ARG;
    int sort_err = 0;
#pragma omp parallel for schedule(dynamic, 4) reduction(| : sort_err)
    for (int r = 0; r < nreg; ++r) {
        if (!p->reg_cells[r]) continue;
        if (orc_sort(p->children, n, p->reg_hi[r], p->sorted + p->reg_place[r]) != cl[r]) sort_err = 1;
    }
    if (sort_err) return ORC_ERR_ARG;
    t[4] = orc_now();

    /* force over every body in sorted order, then the Euler update */
    float dq[ORC_MAX_DEPTH];
    orc_bh_thresholds(ORC_CRIT_STANDARD, box, theta, eps, p->max_depth, dq);
    if (stats) stats[0] = stats[1] = 0;
    const int frc = orc_bh_force(p->node_pos, p->node_mass, p->children, n, p->nodes, dq, eps, G, ORC_ARITH_FMA,
                                 32, p->sorted, n, 1, compensated, quadrupole ? p->quad : NULL, stats, p->acc_new);
    if (frc) return frc;
    t[5] = orc_now();
    orc_integrate(ORC_EULER, 0, n, dt, p->acc_new, acc3, vel3, pos3, 3);
    t[6] = orc_now();
    if (stage_s)
        for (int s = 0; s < 6; ++s) stage_s[s] = t[s + 1] - t[s];
    return ORC_OK;
}

/* The last step's tree and order for tests: children rows of the node index
 * space (compacted by the saturation), sorted[n], {bottom, max_depth}. */
int orc_pipe_export(void *vp, int *children, int *sorted, int *info2) {
    orc_pipe *p = (orc_pipe *)vp;
    if (!p) return ORC_ERR_ARG;
    const long total = (long)p->n + p->nodes + 1;
    if (children) {
        for (long i = 0; i < total * 8; ++i) children[i] = ORC_EMPTY;
        memcpy(children + 8 * (long)p->bottom, p->children + 8 * (long)p->bottom,
               sizeof(int) * 8 * (size_t)(total - p->bottom));
    }
    if (sorted) memcpy(sorted, p->sorted, sizeof(int) * (size_t)p->n);
    if (info2) {
        info2[0] = p->bottom;
        info2[1] = p->max_depth;
    }
    return ORC_OK;
}

int orc_pipe_levels_of(void *vp) { return vp ? ((orc_pipe *)vp)->levels : -1; }
