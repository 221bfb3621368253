// nbgb.hpp -- C++ host layer over the C ABI (include/nbgb.h), mirroring the
// reference's host classes so a CMyApp-style caller keeps its vocabulary:
//   SimulationConfig / BarnesHutConfig / Simulation (src/SimulationConfig.h:46-133,
//   src/BarnesHutConfig.h:10-61) with the same getters and setters, and
//   NBodyApp with InitParticles / Update / ResetSimulation / CopyVertices
//   (CMyApp, src/MyApp.cpp:216-243, 550-656, 1017-1031).
// Header-only; link with libnbgb.so.  Errors surface as nb::Error exceptions
// on the C++ side only -- the C ABI below never throws.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "nbgb.h"

namespace nb {

enum NumericalMethod { LEAPFROG = NB_LEAPFROG, EULER = NB_EULER, KDK_LEAPFROG = NB_KDK_LEAPFROG };
enum PositionConfig { SPHERE_POS = NB_SPHERE_POS, UNIFORM_POS = NB_UNIFORM_POS, BALL_POS = NB_BALL_POS,
                      NORMAL_SIGMA_POS = NB_NORMAL_SIGMA_POS };
enum VelocityConfig { RANDOM_VEL = NB_RANDOM_VEL, STARTING_OUT_VEL = NB_STARTING_OUT_VEL,
                      STARTING_IN_VEL = NB_STARTING_IN_VEL, FUNC_ZERO_VEL = NB_FUNC_ZERO_VEL,
                      TANGENT_XZ_VEL = NB_TANGENT_XZ_VEL, CIRCULAR_Z_VEL = NB_CIRCULAR_Z_VEL };
enum AlgorithmConfig { BARNES_HUT = NB_BARNES_HUT, BRUTE_FORCE_GLOBAL = NB_BRUTE_FORCE_GLOBAL,
                       BRUTE_FORCE_LOCAL = NB_BRUTE_FORCE_LOCAL };

struct NormalDistribution {
    float mean;
    float deviation;
};

struct Error : std::runtime_error {
    nb_status status;
    Error(nb_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

inline void check(nb_status s, const char *what, const nb_sim *sim = nullptr) {
    if (s != NB_OK) {
        std::string m = std::string(what) + ": " + nb_status_string(s);
        if (sim) m += std::string(" (") + nb_last_error_message(sim) + ")";
        throw Error(s, m);
    }
}

// BarnesHutConfig (src/BarnesHutConfig.h:10-61)
class BarnesHutConfig {
public:
    int &GetMaxOctreeDepth() { return max_octree_depth; }
    float &GetTheta() { return theta; }
    float &GetEpsilon() { return epsilon; }
    void SetMaxOctreeDepth(int v) { max_octree_depth = v; }
    void SetTheta(float v) { theta = v; }
    void SetEpsilon(float v) { epsilon = v; }

private:
    int max_octree_depth = 32;
    float theta = 1.5f;
    float epsilon = 0.01f;
};

// SimulationConfig (src/SimulationConfig.h:46-105) plus this library's options
class SimulationConfig {
public:
    int &GetNumberOfBodies() { return c_.num_of_bodies; }
    float &GetGravitationalConstant() { return c_.gravitational_constant; }
    float &GetStartingSpeedMul() { return c_.starting_speed_mul; }
    float &GetStartingVolumeRadius() { return c_.starting_volume_radius; }
    int &GetNumberOfMassiveObjects() { return c_.number_of_massive_objects; }
    float &GetMassiveObjectMass() { return c_.massive_object_mass; }
    int &GetPositionConfig() { return c_.pos_config; }
    int &GetVelocityConfig() { return c_.vel_config; }
    NormalDistribution GetMassDistribution() const { return {c_.mass_mean, c_.mass_deviation}; }
    int &GetAlgorithmConfig() { return c_.algo_config; }
    BarnesHutConfig &GetBarnesHutConfig() { return bh_; }
    int &GetNumericalMethod() { return c_.numerical_method; }
    bool GetCollision() const { return c_.collision != 0; }

    void SetNumberOfBodies(int v) { c_.num_of_bodies = v; }
    void SetGravitationalConstant(float v) { c_.gravitational_constant = v; }
    void SetStartingSpeedMul(float v) { c_.starting_speed_mul = v; }
    void SetStartingVolumeRadius(float v) { c_.starting_volume_radius = v; }
    void SetNumberOfMassiveObjects(int v) { c_.number_of_massive_objects = v; }
    void SetMassiveObjectMass(float v) { c_.massive_object_mass = v; }
    void SetPositionConfig(PositionConfig v) { c_.pos_config = v; }
    void SetVelocityConfig(VelocityConfig v) { c_.vel_config = v; }
    void SetMassDistribution(const NormalDistribution &d) {
        c_.mass_mean = d.mean;
        c_.mass_deviation = d.deviation;
    }
    void SetAlgorithmConfig(AlgorithmConfig v) { c_.algo_config = v; }
    void SetBarnesHutConfig(BarnesHutConfig b) { bh_ = b; }
    void SetNumericalMethod(NumericalMethod v) { c_.numerical_method = v; }
    void SetCollision(bool v) { c_.collision = v ? 1 : 0; }

    // options of this library (defaults keep the reference's behaviour where one exists)
    nb_config &Extra() { return c_; }

    // the C struct handed to nb_create
    nb_config ToC() const {
        nb_config c = c_;
        BarnesHutConfig b = bh_;
        c.max_octree_depth = b.GetMaxOctreeDepth();
        c.theta = b.GetTheta();
        c.epsilon = b.GetEpsilon();
        return c;
    }

    SimulationConfig() { nb_config_default(&c_); }

private:
    nb_config c_{};
    BarnesHutConfig bh_;
};

// Simulation (src/SimulationConfig.h:107-133)
struct Simulation {
    SimulationConfig GetConfig() const { return config; }
    void SetConfig(const SimulationConfig &c) { config = c; }
    float &GetSimulationSpeedMul() { return simulationSpeedMul; }
    float &GetParticleSize() { return particleSize; }

private:
    SimulationConfig config;
    float simulationSpeedMul = 1.0f;
    float particleSize = 0.05f;
};

struct SUpdateInfo {  // src/MyApp.h:42-46
    float ElapsedTimeInSec = 0.0f;
    float DeltaTimeInSec = 0.0f;
};

// The per-step part of CMyApp, headless.
class NBodyApp {
public:
    NBodyApp() = default;
    ~NBodyApp() { Clean(); }
    NBodyApp(const NBodyApp &) = delete;
    NBodyApp &operator=(const NBodyApp &) = delete;

    Simulation &GetSimulation() { return sim_; }
    SimulationConfig &NextConfig() { return next_config_; }

    // InitParticles (src/MyApp.cpp:216-243): buffers + seeded initial conditions
    void InitParticles() {
        Clean();
        nb_config c = sim_.GetConfig().ToC();
        c.simulation_speed_mul = sim_.GetSimulationSpeedMul();
        c.particle_size = sim_.GetParticleSize();
        check(nb_create(&c, &handle_), "nb_create");
        check(nb_init_bodies(handle_), "nb_init_bodies", handle_);
    }

    // Update (src/MyApp.cpp:550-656): clamped frame dt, one step
    void Update(const SUpdateInfo &info) {
        if (!handle_) InitParticles();
        check(nb_update(handle_, info.DeltaTimeInSec), "nb_update", handle_);
        elapsed_ += info.DeltaTimeInSec;
    }

    // ResetSimulation (src/MyApp.cpp:1017-1031): apply the pending config
    void ResetSimulation() {
        sim_.SetConfig(next_config_);
        InitParticles();
    }

    // copy_vertices into a caller buffer of N float4 (device or host)
    void CopyVertices(float *dst4, bool dst_is_device) {
        check(nb_copy_vertices(handle_, dst4, dst_is_device ? 1 : 0), "nb_copy_vertices", handle_);
    }

    void GetState(std::vector<float> &pos3, std::vector<float> &vel3, std::vector<float> &mass) {
        const int n = sim_.GetConfig().ToC().num_of_bodies;
        pos3.resize(3 * (size_t)n);
        vel3.resize(3 * (size_t)n);
        mass.resize(n);
        check(nb_get_state(handle_, pos3.data(), vel3.data(), nullptr, mass.data()), "nb_get_state", handle_);
    }

    nb_sim *Handle() { return handle_; }

    void Clean() {
        if (handle_) nb_destroy(handle_);
        handle_ = nullptr;
    }

private:
    Simulation sim_;
    SimulationConfig next_config_;
    nb_sim *handle_ = nullptr;
    float elapsed_ = 0.0f;
};

// Many simulations stepped together (nb_batch_*); no counterpart in the
// reference, which runs one CMyApp per simulation.
class Batch {
public:
    explicit Batch(const std::vector<SimulationConfig> &configs) {
        std::vector<nb_config> c;
        for (const auto &sc : configs) c.push_back(sc.ToC());
        for (const auto &x : c) sizes_.push_back(x.num_of_bodies);
        check(nb_batch_create(c.data(), (int32_t)c.size(), &b_), "nb_batch_create");
    }
    ~Batch() {
        if (b_) nb_batch_destroy(b_);
    }
    Batch(const Batch &) = delete;
    Batch &operator=(const Batch &) = delete;

    size_t Size() const { return sizes_.size(); }
    void SetState(int k, const std::vector<float> &pos3, const std::vector<float> &vel3,
                  const std::vector<float> &mass) {
        step_check(nb_batch_set_state(b_, k, pos3.data(), vel3.empty() ? nullptr : vel3.data(), mass.data()),
                   "nb_batch_set_state");
    }
    void GetState(int k, std::vector<float> &pos3, std::vector<float> &vel3) {
        const size_t n = (size_t)sizes_.at(k);
        pos3.resize(3 * n);
        vel3.resize(3 * n);
        step_check(nb_batch_get_state(b_, k, pos3.data(), vel3.data(), nullptr, nullptr), "nb_batch_get_state");
    }
    int Autotune(const char *cache_path) {
        int32_t v = -1;
        step_check(nb_batch_autotune(b_, cache_path, &v), "nb_batch_autotune");
        return v;
    }
    void Step(float dt, int nsteps) { step_check(nb_batch_step(b_, dt, nsteps), "nb_batch_step"); }
    nb_status SystemStatus(int k) { return nb_batch_system_status(b_, k); }
    nb_batch *Handle() { return b_; }

private:
    void step_check(nb_status s, const char *what) {
        if (s != NB_OK) throw Error(s, std::string(what) + ": " + nb_batch_last_error_message(b_));
    }
    nb_batch *b_ = nullptr;
    std::vector<int> sizes_;
};

// Job server (nb_server_*): continuous batching of simulation jobs; events
// arrive on a library thread.
class Server {
public:
    using Callback = void (*)(void *user, int64_t job, int32_t event, int32_t value, const float *pos3,
                              const float *vel3, int32_t n);
    explicit Server(const nb_server_config *cfg = nullptr, Callback fn = nullptr, void *user = nullptr) {
        nb_server_config c;
        if (cfg) c = *cfg;
        else nb_server_config_default(&c);
        check(nb_server_create(&c, fn, user, &s_), "nb_server_create");
    }
    ~Server() {
        if (s_) nb_server_destroy(s_);
    }
    Server(const Server &) = delete;
    Server &operator=(const Server &) = delete;

    // initial conditions generated from the config when pos3 is empty
    int64_t Submit(const SimulationConfig &sc, int steps, float dt, const std::vector<float> &pos3 = {},
                   const std::vector<float> &vel3 = {}, const std::vector<float> &mass = {}) {
        nb_config c = sc.ToC();
        int64_t job = -1;
        const nb_status s =
            nb_server_submit(s_, &c, steps, dt, pos3.empty() ? nullptr : pos3.data(),
                             vel3.empty() ? nullptr : vel3.data(), mass.empty() ? nullptr : mass.data(), &job);
        if (s != NB_OK) throw Error(s, "nb_server_submit");
        return job;
    }
    nb_status Wait(int64_t job = -1, double timeout_s = -1.0) { return nb_server_wait(s_, job, timeout_s); }
    nb_server_stats Stats() {
        nb_server_stats st;
        nb_server_get_stats(s_, &st);
        return st;
    }
    nb_server *Handle() { return s_; }

private:
    nb_server *s_ = nullptr;
};

}  // namespace nb
