// gsim.hpp -- header-only C++ mirror of the reference's simulation classes over the C ABI
// of gsim.h.  A caller written against the reference
//
//     gsim::ParticleSystem system(device, count, type, size, minMass, maxMass, G, dt, speed, eps, theta, algo);
//     gsim::BarnesHutSimulation sim(device, &system);
//     sim.RunSimulations(100);
//     ...
//     system.SaveParticles(path);
//
// (src/Main.cpp:250-321) keeps its shape: the classes below take the same arguments
// (minus the Vulkan device), keep the same method names and throw gsim_gb300::Exception
// where the reference throws gsim::Exception (src/Debug/Exception.hpp:72).
//
//   ParticleSystem       src/Particles/ParticleSystem.hpp:11-212 (file and generator ctors,
//                        getters, GetParticles, SaveParticles)
//   DirectSimulation     src/Simulation/Direct/DirectSimulation.hpp:11-81
//   BarnesHutSimulation  src/Simulation/BarnesHut/BarnesHutSimulation.hpp:11-110
//
// The device state lives in one gs_sim owned by the simulation object; the particle
// system reads it back through that simulation once one is attached.
#pragma once

#include <stdint.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "gsim.h"

namespace gsim_gb300 {

class Exception : public std::runtime_error {
public:
    Exception(gs_status status, const std::string& msg) : std::runtime_error(msg), status_(status) {}
    gs_status GetStatus() const { return status_; }

private:
    gs_status status_;
};

inline void Check(gs_status s) {
    if (s != GS_OK) {
        const char* m = gs_last_error();
        throw Exception(s, (m && *m) ? m : gs_status_string(s));
    }
}

class ParticleSystem {
public:
    enum GenerateType {  // ParticleSystem::GenerateType (src/Particles/ParticleSystem.hpp:14-25)
        GENERATE_TYPE_RANDOM = GS_GEN_RANDOM,
        GENERATE_TYPE_GALAXY = GS_GEN_GALAXY,
        GENERATE_TYPE_GALAXY_COLLISION = GS_GEN_GALAXY_COLLISION,
        GENERATE_TYPE_SYMMETRICAL_GALAXY_COLLISION = GS_GEN_SYMMETRICAL_GALAXY_COLLISION,
    };
    enum SimulationAlgorithm {  // ParticleSystem::SimulationAlgorithm (:27-34)
        SIMULATION_ALGORITHM_DIRECT_SUM = GS_DIRECT_SUM,
        SIMULATION_ALGORITHM_BARNES_HUT = GS_BARNES_HUT,
    };
    struct Vec2 {
        float x, y;
    };
    struct Particle {  // src/Particles/Particle.hpp:55-62
        Vec2 pos;
        Vec2 vel;
        float mass;
    };

    ParticleSystem(const ParticleSystem&) = delete;
    ParticleSystem& operator=(const ParticleSystem&) = delete;

    // Load from a particle file ("x y vx vy m" records).
    ParticleSystem(const char* filePath, float G, float dt, float speed, float softening, float theta,
                   SimulationAlgorithm algorithm, int device = 0, uint32_t flags = 0)
        : algorithm_(algorithm) {
        InitParams(G, dt, speed, softening, theta, device, flags);
        uint64_t n = 0;
        Check(gs_read_particles(filePath, 0, &n, nullptr, nullptr, nullptr));
        Resize(n);
        Check(gs_read_particles(filePath, n, &n, pos_.data(), vel_.data(), mass_.data()));
    }

    // Generate with one of the four presets; the reference seeds from time(nullptr),
    // here the seed is explicit.
    ParticleSystem(size_t count, GenerateType type, float size, float minMass, float maxMass, float G, float dt,
                   float speed, float softening, float theta, SimulationAlgorithm algorithm, uint64_t seed = 1,
                   int device = 0, uint32_t flags = 0)
        : algorithm_(algorithm) {
        InitParams(G, dt, speed, softening, theta, device, flags);
        if (type == GENERATE_TYPE_SYMMETRICAL_GALAXY_COLLISION) count &= ~size_t(1);  // ParticleSystem.cpp:520-523
        if (!count) throw Exception(GS_ERR_INVALID_ARGUMENT, "The simulation must contain at least one particle!");
        Resize(count);
        Check(gs_generate(type, count, size, minMass, maxMass, G, seed, pos_.data(), vel_.data(), mass_.data()));
    }

    size_t GetParticleCount() const { return mass_.size(); }
    size_t GetAlignedParticleCount() const {
        const size_t a = (size_t)gs_required_alignment(algorithm_);
        return (GetParticleCount() + a - 1) / a * a;
    }
    float GetGravitationalConst() const { return params_.gravitational_const; }
    float GetSimulationTime() const { return params_.simulation_time; }
    float GetSimulationSpeed() const { return params_.simulation_speed; }
    float GetSofteningLen() const { return params_.softening_len; }
    float GetAccuracyParameter() const { return params_.accuracy_parameter; }
    SimulationAlgorithm GetAlgorithm() const { return algorithm_; }
    const gs_params& GetParams() const { return params_; }
    gs_params& GetParams() { return params_; }

    // Current state (first N particles); after the simulation ran, its latest output.
    void GetParticles(Particle* out) {
        Sync();
        for (size_t i = 0; i < mass_.size(); ++i)
            out[i] = Particle{{pos_[2 * i], pos_[2 * i + 1]}, {vel_[2 * i], vel_[2 * i + 1]}, mass_[i]};
    }
    void SaveParticles(const char* filePath) {
        Sync();
        Check(gs_write_particles(filePath, mass_.size(), pos_.data(), vel_.data(), mass_.data()));
    }

    // used by the simulation classes
    const float* Pos() const { return pos_.data(); }
    const float* Vel() const { return vel_.data(); }
    const float* Mass() const { return mass_.data(); }
    void Attach(gs_sim* sim) { sim_ = sim; }
    void Detach(gs_sim* sim) {
        if (sim_ == sim) {
            Sync();
            sim_ = nullptr;
        }
    }

private:
    void InitParams(float G, float dt, float speed, float softening, float theta, int device, uint32_t flags) {
        gs_params_init(&params_);
        params_.gravitational_const = G;
        params_.simulation_time = dt;
        params_.simulation_speed = speed;
        params_.softening_len = softening;
        params_.accuracy_parameter = theta;
        params_.algorithm = algorithm_;
        params_.device = device;
        params_.flags = flags;
    }
    void Resize(size_t n) {
        pos_.assign(2 * n, 0.0f);
        vel_.assign(2 * n, 0.0f);
        mass_.assign(n, 0.0f);
    }
    void Sync() {
        if (sim_) Check(gs_get_particles(sim_, pos_.data(), vel_.data(), mass_.data()));
    }

    SimulationAlgorithm algorithm_;
    gs_params params_{};
    std::vector<float> pos_, vel_, mass_;
    gs_sim* sim_ = nullptr;
};

namespace detail {
class SimulationBase {
public:
    SimulationBase(const SimulationBase&) = delete;
    SimulationBase& operator=(const SimulationBase&) = delete;

    // Wait for the previous batch, then submit `count` steps (RunSimulations).
    void RunSimulations(uint32_t count) { Check(gs_run(sim_, count)); }
    static size_t GetRequiredParticleAlignment() { return (size_t)gs_required_alignment(GS_DIRECT_SUM); }
    gs_sim* Handle() { return sim_; }

    ~SimulationBase() {
        if (sim_) {
            gs_sync(sim_, 0);  // the fence wait of the reference's destructor
            system_->Detach(sim_);
            gs_destroy(sim_);
        }
    }

protected:
    SimulationBase(ParticleSystem* system, int32_t algorithm) : system_(system) {
        gs_params p = system->GetParams();
        p.algorithm = algorithm;
        Check(gs_create(&p, system->GetParticleCount(), system->Pos(), system->Vel(), system->Mass(), &sim_));
        system->Attach(sim_);
    }

private:
    ParticleSystem* system_;
    gs_sim* sim_ = nullptr;
};
}  // namespace detail

class DirectSimulation : public detail::SimulationBase {
public:
    explicit DirectSimulation(ParticleSystem* system) : SimulationBase(system, GS_DIRECT_SUM) {}
};

class BarnesHutSimulation : public detail::SimulationBase {
public:
    explicit BarnesHutSimulation(ParticleSystem* system) : SimulationBase(system, GS_BARNES_HUT) {}
};

}  // namespace gsim_gb300
