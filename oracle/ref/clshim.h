/*
 * clshim.h -- TEST INFRASTRUCTURE (oracle). Never linked into the product.
 *
 * Force-included (g++ -include) when one of the reference's OpenCL C kernel
 * files (the kernels/ .cl files) is compiled as C++ for the CPU reference emulator in
 * oracle/_ref/.  It supplies the OpenCL C vocabulary those files use:
 * address-space qualifiers, float3/float4 value types with their operators,
 * the geometric built-ins, work-item queries, barriers and the atomics.
 *
 * Work-items run as cooperative coroutines (clrt.cpp).  Every barrier,
 * work_group_all and atomic access is a scheduling point, so a spin loop in
 * one work-item lets the others progress.
 *
 * Numerical choices (all inside the precision the OpenCL C 2.0 spec allows):
 *   - rsqrt(x) = 1/sqrt(x), both correctly rounded (spec: <= 2 ulp);
 *   - normalize(v) = v * (1/sqrt(dot(v,v))), and the zero vector maps to the
 *     zero vector (the spec's special case for normalize);
 *   - pow(x, y) uses the C library powf (exact for y == 1);
 *   - no FP contraction (the translation units are built -ffp-contract=off).
 *
 * __local: inside kernel bodies it becomes a function-scope static placed in
 * the "clref_local" section; the runtime swaps that section per work-group
 * so each group sees its own local memory.  For kernels that take __local
 * pointer parameters (boundary_reduce.cl) CLREF_LOCAL_PARAM makes it empty.
 */
#ifndef NBGB_ORACLE_CLSHIM_H
#define NBGB_ORACLE_CLSHIM_H

#include <stddef.h>

#define __kernel extern "C"
#define __global
#define __constant const
#define __private
#ifdef CLREF_LOCAL_PARAM
#define __local
#else
#define __local static __attribute__((section("clref_local")))
#endif

#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2
#define memory_order_relaxed 0
#define memory_order_acquire 2
#define memory_order_release 3
#define memory_order_acq_rel 4
#define memory_order_seq_cst 5
#define memory_scope_work_item 0
#define memory_scope_work_group 1
#define memory_scope_device 2
#define memory_scope_all_svm_devices 3

typedef float atomic_float;
typedef int atomic_int;
typedef unsigned int uint;

/* ---- runtime hooks (clrt.cpp) ---- */
extern "C" {
size_t clref_get_global_id(unsigned);
size_t clref_get_local_id(unsigned);
size_t clref_get_group_id(unsigned);
size_t clref_get_global_size(unsigned);
size_t clref_get_local_size(unsigned);
size_t clref_get_num_groups(unsigned);
void clref_barrier(void);
void clref_yield(void);
int clref_work_group_all(int);
}

static inline size_t get_global_id(unsigned d) { return clref_get_global_id(d); }
static inline size_t get_local_id(unsigned d) { return clref_get_local_id(d); }
static inline size_t get_group_id(unsigned d) { return clref_get_group_id(d); }
static inline size_t get_global_size(unsigned d) { return clref_get_global_size(d); }
static inline size_t get_local_size(unsigned d) { return clref_get_local_size(d); }
static inline size_t get_num_groups(unsigned d) { return clref_get_num_groups(d); }

static inline void barrier(int) { clref_barrier(); }
static inline int work_group_all(int p) { return clref_work_group_all(p ? 1 : 0); }

/* mem_fence: in calculate_forces.cl the fences sit at the points where a
 * 16-lane "warp" shares its traversal stack; CLREF_FENCE_IS_BARRIER turns them
 * into group barriers so the lanes advance in lockstep as on SIMT hardware
 * (only meaningful with WORKGROUP_SIZE == WARP_SIZE).  Elsewhere a fence is
 * a scheduling point only. */
#ifdef CLREF_FENCE_IS_BARRIER
static inline void mem_fence(int) { clref_barrier(); }
#else
static inline void mem_fence(int) { clref_yield(); }
#endif
static inline void atomic_work_item_fence(int, int, int) { clref_yield(); }

/* ---- atomics (single OS thread: plain read-modify-write + yield) ---- */
static inline int atomic_cmpxchg(volatile int *p, int cmp, int val) {
    clref_yield();
    int old = *p;
    if (old == cmp) *p = val;
    return old;
}
static inline int atom_dec(volatile int *p) { clref_yield(); int old = *p; *p = old - 1; return old; }
static inline int atom_inc(volatile int *p) { clref_yield(); int old = *p; *p = old + 1; return old; }
static inline int atom_max(volatile int *p, int v) { clref_yield(); int old = *p; if (v > old) *p = v; return old; }
static inline int atomic_dec(volatile int *p) { return atom_dec(p); }
static inline int atomic_max(volatile int *p, int v) { return atom_max(p, v); }
static inline float atomic_load_explicit(volatile float *p, int, int) { clref_yield(); return *p; }
static inline int atomic_load_explicit(volatile int *p, int, int) { clref_yield(); return *p; }
static inline void atomic_store_explicit(volatile float *p, float v, int, int) { clref_yield(); *p = v; }
static inline void atomic_store_explicit(volatile int *p, int v, int, int) { clref_yield(); *p = v; }

/* ---- vector types ---- */
struct float3 { float x, y, z; };
struct float4 { float x, y, z, w; };

static inline float3 operator+(float3 a, float3 b) { float3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline float3 operator-(float3 a, float3 b) { float3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline float3 operator*(float3 a, float s) { float3 r = {a.x * s, a.y * s, a.z * s}; return r; }
static inline float3 operator*(float s, float3 a) { float3 r = {s * a.x, s * a.y, s * a.z}; return r; }
static inline float3 operator/(float3 a, float s) { float3 r = {a.x / s, a.y / s, a.z / s}; return r; }
static inline float3 &operator+=(float3 &a, float3 b) { a = a + b; return a; }
static inline float3 &operator-=(float3 &a, float3 b) { a = a - b; return a; }
static inline float3 &operator*=(float3 &a, float s) { a = a * s; return a; }

/* ---- scalar / geometric built-ins ---- */
static inline float fabs(float x) { return __builtin_fabsf(x); }
static inline float fmax(float a, float b) { return __builtin_fmaxf(a, b); }
static inline float fmin(float a, float b) { return __builtin_fminf(a, b); }
static inline float sqrt(float x) { return __builtin_sqrtf(x); }
static inline float rsqrt(float x) { return 1.0f / __builtin_sqrtf(x); }
static inline float pow(float x, float y) { return __builtin_powf(x, y); }
/* OpenCL min/max on floats: fmin/fmax semantics for ordered inputs */
static inline float min(float a, float b) { return b < a ? b : a; }
static inline float max(float a, float b) { return a < b ? b : a; }
static inline int min(int a, int b) { return b < a ? b : a; }
static inline int max(int a, int b) { return a < b ? b : a; }
static inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float length(float3 a) { return __builtin_sqrtf(dot(a, a)); }
static inline float distance(float3 a, float3 b) { return length(a - b); }
static inline float3 normalize(float3 v) {
    float l2 = dot(v, v);
    if (l2 == 0.0f) return v;
    float inv = 1.0f / __builtin_sqrtf(l2);
    return v * inv;
}

/* printf appears only under DEBUG, which the emulator never defines. */

#endif
