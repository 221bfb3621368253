// ic.cpp -- seeded initial conditions (CMyApp::InitBodyAttributes,
// src/MyApp.cpp:331-495), generated on the host so every consumer gets the
// same bytes.  The reference draws from an unseeded std::random_device; here
// each quantity has its own SplitMix64 stream derived from cfg->seed and the
// normals come from Box-Muller in double, rounded to float.
//
// SplitMix64 is a counter (its k-th output is a mix of seed + k * golden),
// and every mode draws a fixed number of uniforms per pair of bodies, so the
// bodies are generated in parallel chunks that start at even bodies, each
// chunk's stream jumped to its first uniform: the output is the same bytes
// as one sequential pass.  Sums over all bodies stay sequential.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

#include "../../include/nbgb.h"

namespace {

constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ULL;

struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    void skip(uint64_t k) { s += k * kGolden; }
    uint64_t next() {
        uint64_t z = (s += kGolden);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    // uniform in (0, 1]
    double uniform() { return ((next() >> 11) + 1) * (1.0 / 9007199254740992.0); }
};

struct Normal {
    SplitMix64 r;
    bool have = false;
    double spare = 0.0;
    // the stream positioned at uniform number `first` with no spare normal
    Normal(uint64_t seed, uint64_t first) : r(seed) { r.skip(first); }
    double next() {
        if (have) {
            have = false;
            return spare;
        }
        const double u1 = r.uniform(), u2 = r.uniform();
        const double rad = std::sqrt(-2.0 * std::log(u1));
        const double a = 6.283185307179586 * u2;
        spare = rad * std::sin(a);
        have = true;
        return rad * std::cos(a);
    }
};

constexpr uint64_t kPosStream = 0x706f736974696f6eULL;
constexpr uint64_t kMassStream = 0x6d61737365730000ULL;
constexpr uint64_t kVelStream = 0x76656c6f63697479ULL;

void normalize3(float &x, float &y, float &z) {
    const float l = std::sqrt(x * x + y * y + z * z);
    if (l > 0.0f) {
        x /= l;
        y /= l;
        z /= l;
    }
}

// fn(i0, i1) over [0, n) in chunks that start at even indices, on up to the
// host's hardware threads
template <class F>
void parallel_bodies(int n, F fn) {
    const int min_chunk = 1 << 15;
    int threads = (int)std::thread::hardware_concurrency();
    threads = std::max(1, std::min(threads, n / min_chunk));
    if (threads <= 1) {
        fn(0, n);
        return;
    }
    int chunk = (n + threads - 1) / threads;
    chunk += chunk & 1;
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const int i0 = t * chunk, i1 = std::min(n, i0 + chunk);
        if (i0 >= i1) break;
        pool.emplace_back(fn, i0, i1);
    }
    for (auto &th : pool) th.join();
}

}  // namespace

extern "C" nb_status nb_generate_ic(const nb_config *cfg, float *pos3, float *vel3, float *mass) {
    if (!cfg || cfg->num_of_bodies < 0) return NB_ERR_INVALID_ARGUMENT;
    const int n = cfg->num_of_bodies;
    const float R = cfg->starting_volume_radius;

    if (mass) {
        // one normal per body: two uniforms per pair of bodies
        if (cfg->mass_config == NB_MASS_EQUAL) {
            for (int i = 0; i < n; ++i) mass[i] = 1.0f / (float)n;
        } else if (cfg->mass_config == NB_MASS_LOGNORMAL) {
            std::vector<double> m(n);
            parallel_bodies(n, [&](int i0, int i1) {
                Normal nm(cfg->seed ^ kMassStream, (uint64_t)i0);
                for (int i = i0; i < i1; ++i) m[i] = std::exp((double)cfg->mass_lognormal_sigma * nm.next());
            });
            double tot = 0.0;
            for (int i = 0; i < n; ++i) tot += m[i];
            for (int i = 0; i < n; ++i) mass[i] = (float)(m[i] / tot);
        } else {  // |N(mean, deviation)| (src/MyApp.cpp:335-343)
            parallel_bodies(n, [&](int i0, int i1) {
                Normal nm(cfg->seed ^ kMassStream, (uint64_t)i0);
                for (int i = i0; i < i1; ++i)
                    mass[i] = (float)std::fabs((double)cfg->mass_mean + (double)cfg->mass_deviation * nm.next());
            });
        }
        // src/MyApp.cpp:345-355 draws indices in [0, M) until all M are
        // massive, i.e. bodies 0..M-1
        const int M = cfg->number_of_massive_objects < n ? cfg->number_of_massive_objects : n;
        for (int i = 0; i < M; ++i) mass[i] = cfg->massive_object_mass;
    }

    std::vector<float> tmp;
    float *P = pos3;
    if (!P && vel3) {
        tmp.resize((size_t)n * 3);
        P = tmp.data();
    }
    if (P) {
        const uint64_t pseed = cfg->seed ^ kPosStream;
        switch (cfg->pos_config) {
        case NB_SPHERE_POS: {  // Fibonacci sphere (src/MyApp.cpp:361-383)
            const float golden = 1.6180339887498948482f, two_pi = 6.2831853071795864769f;
            const float N = (float)n;
            parallel_bodies(n, [&](int i0, int i1) {
                for (int i = i0; i < i1; ++i) {
                    // the running float index (idx += 1) stops growing at 2^24
                    const float idx = (float)std::min(i, 1 << 24);
                    const float eps = 0.5f;
                    float ip;
                    const float x = std::modf(idx / golden, &ip);
                    const float y = (idx + eps) / (N - 1.0f + 2.0f * eps);
                    const float lat = 2.0f * two_pi * x;
                    const float lon = std::acos(1.0f - 2.0f * y);
                    P[3 * i] = R * std::sin(lat) * std::sin(lon);
                    P[3 * i + 1] = R * std::cos(lon);
                    P[3 * i + 2] = R * std::cos(lat) * std::sin(lon);
                }
            });
        } break;
        case NB_BALL_POS:  // three normals and a uniform per body: eight uniforms per pair
            parallel_bodies(n, [&](int i0, int i1) {
                Normal np(pseed, 4 * (uint64_t)i0);
                for (int i = i0; i < i1; ++i) {
                    double x = np.next(), y = np.next(), z = np.next();
                    const double l = std::sqrt(x * x + y * y + z * z);
                    const double r = (double)R * std::cbrt(np.r.uniform());
                    P[3 * i] = (float)(x / l * r);
                    P[3 * i + 1] = (float)(y / l * r);
                    P[3 * i + 2] = (float)(z / l * r);
                }
            });
            break;
        case NB_NORMAL_SIGMA_POS:  // three normals per body: six uniforms per pair
            parallel_bodies(n, [&](int i0, int i1) {
                Normal np(pseed, 3 * (uint64_t)i0);
                for (int i = i0; i < i1; ++i)
                    for (int k = 0; k < 3; ++k) P[3 * i + k] = (float)((double)cfg->pos_sigma[k] * np.next());
            });
            break;
        case NB_UNIFORM_POS:
        default:  // normal(0, R) per axis (src/MyApp.cpp:384-396)
            parallel_bodies(n, [&](int i0, int i1) {
                Normal np(pseed, 3 * (uint64_t)i0);
                for (int i = 3 * i0; i < 3 * i1; ++i) P[i] = (float)((double)R * np.next());
            });
            break;
        }
    }

    if (vel3) {
        const float mul = cfg->starting_speed_mul;
        double mtot = 0.0;  // total mass for NB_CIRCULAR_Z_VEL
        if (mass)
            for (int j = 0; j < n; ++j) mtot += mass[j];
        else
            mtot = 1.0;
        // NB_RANDOM_VEL draws three normals per body: six uniforms per pair
        parallel_bodies(n, [&](int i0, int i1) {
        Normal nv(cfg->seed ^ kVelStream, 3 * (uint64_t)i0);
        for (int i = i0; i < i1; ++i) {
            float px = P[3 * i], py = P[3 * i + 1], pz = P[3 * i + 2];
            float vx = 0.0f, vy = 0.0f, vz = 0.0f;
            switch (cfg->vel_config) {
            case NB_RANDOM_VEL: {  // normalize(N(0,0.1)^3) * mul (:423-436)
                vx = (float)(0.1 * nv.next());
                vy = (float)(0.1 * nv.next());
                vz = (float)(0.1 * nv.next());
                normalize3(vx, vy, vz);
                vx *= mul; vy *= mul; vz *= mul;
            } break;
            case NB_STARTING_OUT_VEL:
            case NB_STARTING_IN_VEL: {  // +-normalize(pos) * mul (:439-463)
                vx = px; vy = py; vz = pz;
                normalize3(vx, vy, vz);
                const float sgn = cfg->vel_config == NB_STARTING_OUT_VEL ? 1.0f : -1.0f;
                vx *= mul * sgn; vy *= mul * sgn; vz *= mul * sgn;
            } break;
            case NB_TANGENT_XZ_VEL: {  // cross(y, pos), or cross(x, pos) on the y = 0 plane (:475-486)
                if (std::fabs(py) < FLT_EPSILON) {
                    vx = 0.0f; vy = -pz; vz = py;
                } else {
                    vx = pz; vy = 0.0f; vz = -px;
                }
                vx *= mul; vy *= mul; vz *= mul;
            } break;
            case NB_CIRCULAR_Z_VEL: {
                const double r = std::sqrt((double)px * px + (double)py * py + (double)pz * pz);
                const double rc = std::sqrt((double)px * px + (double)py * py);
                if (rc > 0.0 && r > 0.0) {
                    const double x = r / (double)R;
                    const double menc = mtot * x * x * x;
                    const double speed = std::sqrt((double)cfg->gravitational_constant * menc / r) * mul;
                    vx = (float)(-py / rc * speed);
                    vy = (float)(px / rc * speed);
                    vz = 0.0f;
                }
            } break;
            case NB_FUNC_ZERO_VEL:
            default:  // glm::epsilon<float>() per component (:464-474)
                vx = vy = vz = FLT_EPSILON;
                break;
            }
            vel3[3 * i] = vx;
            vel3[3 * i + 1] = vy;
            vel3[3 * i + 2] = vz;
        }
        });
    }
    return NB_OK;
}
