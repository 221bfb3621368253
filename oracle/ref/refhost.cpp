/*
 * refhost.cpp -- TEST INFRASTRUCTURE (oracle). Never linked into the product.
 *
 * Headless stand-in for the reference's CMyApp OpenCL host: owns the buffer
 * set of CMyApp::InitParticles (src/MyApp.cpp:216-243), sizes it like
 * CMyApp::SetKernelConfig (src/MyApp.cpp:71-83) and launches the reference's
 * own kernels (compiled from the kernels/ .cl files through clshim.h) with the NDRange
 * shapes of CMyApp::Update (src/MyApp.cpp:583-630) on the coroutine runtime
 * in clrt.cpp.  Differences from the as-wired host, each one deliberate:
 *   - `method` of calculate_force_local is passed as a real NumericalMethod
 *     (the reference binds NumberOfBodies there, src/MyApp.cpp:319);
 *   - the boundary buffer can be written directly, so a stage-isolated tree
 *     can be built on the exact bounding box;
 *   - hybrid_reduce_root is not run: its output is never read (the host
 *     passes cl_p to parallel_reduce_root, src/MyApp.cpp:282).
 * Exposed as extern "C" for ctypes (tests only).
 */
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

struct cl_float4 { float x, y, z, w; };

extern "C" {
int clref_launch(size_t global, size_t local, const std::function<void()> *body);
void clref_set_round_cap(long cap);

/* the reference kernels (signatures of the kernels/ .cl files) */
void init(float *positions, float *mass, int *children, float *error, float *boundaries,
          int *bottom, int num_of_bodies, int num_of_nodes, unsigned max_children, int *body_depth);
void build_tree(float *positions, volatile float *mass, float *boundaries, volatile int *children,
                volatile int *max_depth, unsigned max_children, int num_of_bodies, int num_of_nodes,
                volatile int *bottom, volatile int *error, int *body_depth);
void saturate_tree(float *positions, volatile float *mass, volatile int *children, int num_of_bodies,
                   int num_of_nodes, volatile int *bottom, int *body_count);
void calculate_force_local(float *positions, float *mass, float *vels, float *accs, int *children,
                           float theta, float eps, int num_of_bodies, int num_of_nodes, float G,
                           float dt, int *max_depth, int *errors, float *boundaries, int method);
void update(float *v, float *p, float *m, float *a, float dt, float G, int method);
void update_local(float *v, float *p, float *m, float *a, float dt, float G, int num_of_bodies,
                  int method);
void update_collision_local(float *v, float *p, int num_of_bodies);
void copy_vertices(float *p, cl_float4 *v, unsigned num_of_bodies);
void parallel_reduce_root(float *local_extremities, float *extremity, float *scratch);
}

namespace {
struct RefSim {
    int n, wg, cus, nodes;
    unsigned max_children;
    std::vector<float> p, m, v, a, boundary, temp;
    std::vector<int> children, error, body_depth, body_count;
    int bottom = 0, max_depth = 0;
};

size_t round_up(size_t n, size_t wg) { return ((n + wg - 1) / wg) * wg; }
}  // namespace

extern "C" {

int ref_workgroup_size(void) {
#ifdef WORKGROUP_SIZE
    return WORKGROUP_SIZE;
#else
    return -1;
#endif
}

/* SetKernelConfig (src/MyApp.cpp:71-83) with warpsize 16 (src/MyApp.h:122). */
void *ref_create(int n, int cus) {
    RefSim *s = new RefSim();
    s->n = n;
    s->wg = ref_workgroup_size();
    s->cus = cus;
    int nodes = n * 2;
    if (nodes < 1024 * cus) nodes = 1024 * cus;
    while ((nodes & (16 - 1)) != 0) ++nodes;
    s->nodes = nodes;
    s->max_children = (unsigned)((nodes + n + 1) * 8);
    s->p.assign((size_t)(n + nodes + 1) * 3, 0.0f);
    s->m.assign((size_t)(n + nodes + 1), 0.0f);
    s->v.assign((size_t)n * 3, 0.0f);
    s->a.assign((size_t)n * 3, 0.0f);
    s->boundary.assign(8, 0.0f);
    s->temp.assign((size_t)s->wg * 8, 0.0f);
    s->children.assign(s->max_children, -1);
    s->error.assign((size_t)n, 0);
    s->body_depth.assign((size_t)n, 0);
    s->body_count.assign((size_t)(nodes + 1 + n), 0);
    return s;
}

void ref_destroy(void *h) { delete (RefSim *)h; }
int ref_num_nodes(void *h) { return ((RefSim *)h)->nodes; }
void ref_set_round_cap(long cap) { clref_set_round_cap(cap); }

void ref_set_bodies(void *h, const float *pos3, const float *vel3, const float *mass, const float *acc3) {
    RefSim *s = (RefSim *)h;
    memcpy(s->p.data(), pos3, sizeof(float) * 3 * s->n);
    memcpy(s->m.data(), mass, sizeof(float) * s->n);
    if (vel3) memcpy(s->v.data(), vel3, sizeof(float) * 3 * s->n);
    if (acc3) memcpy(s->a.data(), acc3, sizeof(float) * 3 * s->n);
}

void ref_set_boundary(void *h, const float *box6) { memcpy(((RefSim *)h)->boundary.data(), box6, 6 * sizeof(float)); }
void ref_set_max_depth(void *h, int d) { ((RefSim *)h)->max_depth = d; }

/* parallel_reduce_root as wired: first argument is cl_p (src/MyApp.cpp:282),
 * one work-group of WORKGROUP_SIZE (src/MyApp.cpp:586). */
int ref_bbox_as_wired(void *h) {
    RefSim *s = (RefSim *)h;
    std::vector<float> scratch((size_t)s->wg * 6, 0.0f);
    float *p = s->p.data(), *b = s->boundary.data(), *sc = scratch.data();
    std::function<void()> body = [=] { parallel_reduce_root(p, b, sc); };
    return clref_launch(s->wg, s->wg, &body);
}

int ref_init(void *h) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data(), *m = s->m.data(), *b = s->boundary.data();
    int *ch = s->children.data(), *err = s->error.data(), *bd = s->body_depth.data(), *bot = &s->bottom;
    int n = s->n, nodes = s->nodes;
    unsigned mc = s->max_children;
    std::function<void()> body = [=] { init(p, m, ch, (float *)err, b, bot, n, nodes, mc, bd); };
    return clref_launch(round_up(n, s->wg), s->wg, &body);
}

int ref_build_tree(void *h) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data(), *m = s->m.data(), *b = s->boundary.data();
    int *ch = s->children.data(), *err = s->error.data(), *bd = s->body_depth.data();
    int *bot = &s->bottom, *md = &s->max_depth;
    int n = s->n, nodes = s->nodes;
    unsigned mc = s->max_children;
    std::function<void()> body = [=] { build_tree(p, m, b, ch, md, mc, n, nodes, bot, err, bd); };
    return clref_launch(round_up(n, s->wg), s->wg, &body);
}

int ref_saturate_tree(void *h) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data(), *m = s->m.data();
    int *ch = s->children.data(), *bc = s->body_count.data(), *bot = &s->bottom;
    int n = s->n, nodes = s->nodes;
    std::function<void()> body = [=] { saturate_tree(p, m, ch, n, nodes, bot, bc); };
    return clref_launch(round_up(n, s->wg), s->wg, &body);
}

int ref_calculate_force(void *h, float theta, float eps, float G, float dt, int method) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data(), *m = s->m.data(), *v = s->v.data(), *a = s->a.data(), *b = s->boundary.data();
    int *ch = s->children.data(), *md = &s->max_depth, *err = s->error.data();
    int n = s->n, nodes = s->nodes;
    std::function<void()> body = [=] {
        calculate_force_local(p, m, v, a, ch, theta, eps, n, nodes, G, dt, md, err, b, method);
    };
    return clref_launch(round_up(n, s->wg), s->wg, &body);
}

/* update: global N, local NullRange (src/MyApp.cpp:602-604); the runtime
 * picks the largest divisor of N not above WORKGROUP_SIZE. */
int ref_update_global(void *h, float dt, float G, int method) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data(), *m = s->m.data(), *v = s->v.data(), *a = s->a.data();
    size_t local = 1;
    for (size_t l = (size_t)s->wg; l >= 1; --l)
        if (s->n % l == 0) { local = l; break; }
    std::function<void()> body = [=] { update(v, p, m, a, dt, G, method); };
    return clref_launch(s->n, local, &body);
}

int ref_update_local(void *h, float dt, float G, int method) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data(), *m = s->m.data(), *v = s->v.data(), *a = s->a.data();
    int n = s->n;
    std::function<void()> body = [=] { update_local(v, p, m, a, dt, G, n, method); };
    return clref_launch(round_up(n, s->wg), s->wg, &body);
}

int ref_collision(void *h) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data(), *v = s->v.data();
    int n = s->n;
    std::function<void()> body = [=] { update_collision_local(v, p, n); };
    return clref_launch(round_up(n, s->wg), s->wg, &body);
}

int ref_copy_vertices(void *h, float *out4) {
    RefSim *s = (RefSim *)h;
    float *p = s->p.data();
    unsigned n = (unsigned)s->n;
    cl_float4 *o = (cl_float4 *)out4;
    std::function<void()> body = [=] { copy_vertices(p, o, n); };
    return clref_launch(round_up(n, s->wg), s->wg, &body);
}

/* which: 0 positions[(N+nodes+1)*3], 1 mass[N+nodes+1], 2 children[max_children],
 * 3 body_count[N+nodes+1], 4 vel[3N], 5 acc[3N], 6 boundary[8], 7 error[N],
 * 8 body_depth[N], 9 bottom (int), 10 max_depth (int). Returns bytes copied. */
long ref_get(void *h, int which, void *dst) {
    RefSim *s = (RefSim *)h;
    const void *src = nullptr;
    size_t bytes = 0;
    switch (which) {
    case 0: src = s->p.data(); bytes = s->p.size() * 4; break;
    case 1: src = s->m.data(); bytes = s->m.size() * 4; break;
    case 2: src = s->children.data(); bytes = s->children.size() * 4; break;
    case 3: src = s->body_count.data(); bytes = s->body_count.size() * 4; break;
    case 4: src = s->v.data(); bytes = s->v.size() * 4; break;
    case 5: src = s->a.data(); bytes = s->a.size() * 4; break;
    case 6: src = s->boundary.data(); bytes = 8 * 4; break;
    case 7: src = s->error.data(); bytes = s->error.size() * 4; break;
    case 8: src = s->body_depth.data(); bytes = s->body_depth.size() * 4; break;
    case 9: src = &s->bottom; bytes = 4; break;
    case 10: src = &s->max_depth; bytes = 4; break;
    default: return -1;
    }
    if (dst) memcpy(dst, src, bytes);
    return (long)bytes;
}

}  // extern "C"
