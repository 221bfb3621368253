// k_diag.cu -- FP64 diagnostics and the debug export of the tree.
//
// FP64 appears on the GPU only here: the accuracy probe (a direct sum for a
// sample of bodies, against which a step's FP32 forces are measured) and the
// energy / momentum reductions.  None of it runs inside nb_step.
#include "nbgb_internal.cuh"

namespace nbgb {

// Reference-layout export (src/MyApp.cpp:219-235): children[8*(N+C+1)] with
// cell rows at their node index, node positions / masses / body counts.
__global__ void k_export_tree(DevSim s, int *children_full, float *pos_full, float *mass_full, int *count_full,
                              float *quad_full) {
    const int n = s.n, cap = s.cap, total = n + cap + 1;
    const int bottom = s.ctrl->bottom;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        int row[8];
        float4 pm;
        int cnt;
        if (k < n) {
            for (int j = 0; j < 8; ++j) row[j] = kEmpty;
            pm = s.body_cur[k];
            cnt = 0;
        } else if (k >= bottom) {
            const int c = k - n;
            for (int j = 0; j < 8; ++j) row[j] = s.child[c * 8 + j];
            pm = s.cell_pm[c];
            cnt = s.count[c];
        } else {
            for (int j = 0; j < 8; ++j) row[j] = kEmpty;
            pm = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            cnt = 0;
        }
        if (children_full)
            for (int j = 0; j < 8; ++j) children_full[(size_t)k * 8 + j] = row[j];
        if (pos_full) {
            pos_full[(size_t)k * 3] = pm.x;
            pos_full[(size_t)k * 3 + 1] = pm.y;
            pos_full[(size_t)k * 3 + 2] = pm.z;
        }
        if (mass_full) mass_full[k] = pm.w;
        if (count_full) count_full[k] = cnt;
        if (quad_full) {
            float q[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            if (k >= n && k >= bottom && s.cell_q) {
                const float4 a = s.cell_q[2 * (k - n)], b = s.cell_q[2 * (k - n) + 1];
                q[0] = a.x; q[1] = a.y; q[2] = a.z; q[3] = a.w; q[4] = b.x; q[5] = b.y;
            }
            for (int j = 0; j < 6; ++j) quad_full[(size_t)k * 6 + j] = q[j];
        }
    }
}

cudaError_t launch_export_tree(const DevSim &s, int *children_full, float *pos_full, float *mass_full,
                               int *count_full, float *quad_full, cudaStream_t st) {
    const int total = s.n + s.cap + 1;
    int blocks = (total + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    k_export_tree<<<blocks, 256, 0, st>>>(s, children_full, pos_full, mass_full, count_full, quad_full);
    return cudaGetLastError();
}

// One block per sample body: FP64 Plummer sum over all other bodies, block
// reduction, three doubles out.
__global__ void __launch_bounds__(256) k_force_probe(const float4 *__restrict__ body, int n,
                                                     const int *__restrict__ sample, double eps, double G,
                                                     double *out3) {
    const int i = sample[blockIdx.x];
    const float4 me = body[i];
    const double px = me.x, py = me.y, pz = me.z, e2 = eps * eps;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        if (j == i) continue;
        const float4 q = __ldg(&body[j]);
        const double dx = (double)q.x - px, dy = (double)q.y - py, dz = (double)q.z - pz;
        const double d2 = dx * dx + dy * dy + dz * dz + e2;
        const double r = 1.0 / sqrt(d2);
        const double F = (double)q.w * r * r * r;
        ax += dx * F;
        ay += dy * F;
        az += dz * F;
    }
    __shared__ double red[3][256];
    red[0][threadIdx.x] = ax;
    red[1][threadIdx.x] = ay;
    red[2][threadIdx.x] = az;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) out3[(size_t)blockIdx.x * 3 + k] = red[k][0] * G;
}

cudaError_t launch_force_probe(const float4 *body, int n, const int *sample, int ns, double eps, double G,
                               double *out3, cudaStream_t st) {
    if (ns <= 0) return cudaSuccess;
    k_force_probe<<<ns, 256, 0, st>>>(body, n, sample, eps, G, out3);
    return cudaGetLastError();
}

// Kinetic energy, momentum, angular momentum, total mass (FP64 atomics on a
// per-block reduction); optional FP64 pair potential (O(N^2)).
__global__ void __launch_bounds__(256) k_moments(const float4 *__restrict__ body, const float4 *__restrict__ vel, int n,
                                                 double *out) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = body[i];
        const float4 v = vel[i];
        const double m = p.w, vx = v.x, vy = v.y, vz = v.z, x = p.x, y = p.y, z = p.z;
        acc[0] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        acc[1] += m * vx;
        acc[2] += m * vy;
        acc[3] += m * vz;
        acc[4] += m * (y * vz - z * vy);
        acc[5] += m * (z * vx - x * vz);
        acc[6] += m * (x * vy - y * vx);
        acc[7] += m;
    }
    for (int k = 0; k < 8; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(&out[k], v);
    }
}

__global__ void __launch_bounds__(256) k_potential(const float4 *__restrict__ body, int n, double eps, double G,
                                                   double *out) {
    double pe = 0.0;
    const double e2 = eps * eps;
    for (int i = blockIdx.x; i < n; i += gridDim.x) {
        const float4 a = body[i];
        for (int j = i + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const float4 b = __ldg(&body[j]);
            const double dx = (double)b.x - a.x, dy = (double)b.y - a.y, dz = (double)b.z - a.z;
            pe -= G * (double)a.w * (double)b.w / sqrt(dx * dx + dy * dy + dz * dz + e2);
        }
    }
    for (int o = 16; o > 0; o >>= 1) pe += __shfl_xor_sync(0xffffffffu, pe, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&out[8], pe);
}

cudaError_t launch_diagnostics(const float4 *body, const float4 *vel, int n, int with_potential, double eps,
                               double G, double *out9, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out9, 0, 9 * sizeof(double), st);
    if (e != cudaSuccess) return e;
    int blocks = (n + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    if (blocks < 1) blocks = 1;
    k_moments<<<blocks, 256, 0, st>>>(body, vel, n, out9);
    if (with_potential) {
        int pb = n < 8192 ? (n > 0 ? n : 1) : 8192;
        k_potential<<<pb, 256, 0, st>>>(body, n, eps, G, out9);
    }
    return cudaGetLastError();
}

}  // namespace nbgb
