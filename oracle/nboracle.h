/*
 * nboracle.h -- TEST INFRASTRUCTURE: declarations shared by the CPU oracle's
 * translation units (nboracle.c: the kernel-by-kernel restatement of the
 * reference; nbpipeline.c: the same kernels as one parallel step, the timed
 * CPU baseline).  Nothing in the product includes this header.
 */
#ifndef NBORACLE_H
#define NBORACLE_H

#include <stdint.h>
#include <string.h>

#define ORC_EMPTY (-1)
#define ORC_MAX_DEPTH 64

enum { ORC_OK = 0, ORC_ERR_CELL_OVERFLOW = 4, ORC_ERR_DEPTH = 5, ORC_ERR_ARG = 1 };
enum { ORC_SEM_REFERENCE = 0, ORC_SEM_GEOMETRIC = 1 };
enum { ORC_CRIT_REFERENCE = 0, ORC_CRIT_STANDARD = 1 };
enum { ORC_ARITH_REFERENCE = 0, ORC_ARITH_FMA = 1 };
enum { ORC_LEAPFROG = 1, ORC_EULER = 2, ORC_KDK = 3 };

/* Order-preserving key of a float: an unsigned compare on keys is the float
 * order with -0 < +0.  The GPU reduction uses the same total order, which
 * makes the exact bounding box bit-reproducible. */
static inline uint32_t orc_fkey(float f) {
    uint32_t b;
    memcpy(&b, &f, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

/* Geometric semantics: a cubic root around the box centre with half-width
 * 0.5*max extent (Burtscher), octant 4*(y<cy)+2*(x<cx)+(z<cz) (the
 * reference's numbering, kernels/build_tree.hcl:14-29), child centre =
 * centre -/+ r/2 per axis. */
typedef struct { float c[3]; float r; } orc_cube;

static inline int orc_octant_geo(const float p[3], const orc_cube *q) {
    return (p[1] < q->c[1] ? 4 : 0) + (p[0] < q->c[0] ? 2 : 0) + (p[2] < q->c[2] ? 1 : 0);
}
static inline void orc_descend_geo(const float p[3], orc_cube *q) {
    q->r *= 0.5f;
    for (int k = 0; k < 3; ++k) q->c[k] += (p[k] < q->c[k]) ? -q->r : q->r;
}

void orc_root_cube(const float box6[6], float out4[4]);
int orc_saturate_range(int compaction_bug, int n, int lo, int hi, float *node_pos, float *node_mass,
                       int *children, int *body_count);
void orc_quadrupoles_range(int n, int lo, int hi, const float *node_pos, const float *node_mass,
                           const int *children, float *quad);
int orc_sort(const int *children, int n, int root, int *sorted);
void orc_bh_thresholds(int criterion, const float box6[6], float theta, float eps, int max_depth, float *dq);
int orc_bh_force(const float *node_pos, const float *node_mass, const int *children, int n, int nodes,
                 const float *dq, float eps, float G, int arith, int vote_width, const int *order, int norder,
                 int skip_self, int compensated, const float *quad, long long *stats, float *acc3);
void orc_integrate(int method, int primed, int n, float dt, const float *acc_new3, float *accs3, float *vel3,
                   float *pos3, int pos_stride);

#endif
