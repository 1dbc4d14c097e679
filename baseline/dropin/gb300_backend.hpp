#pragma once
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <mpcd/api/simulation_parameters.hpp>
#include "common/backend.hpp"
#include "mpcd_gb.h"          // from the GB300 repository's include/

namespace mpcd::gb300 {

class GbBackend final : public Backend {
public:
    explicit GbBackend(SimulationParameters const& p) : Backend(p) {
        mpcd_gb_params c{};
        c.experiment = p.experiment == ExperimentType::channel ? 1 : 0;
        c.algorithm  = p.algorithm == MPCDAlgorithm::extended ? 1 : 0;
        c.collision_kernel = static_cast<int32_t>(p.collision_kernel);
        for (int d = 0; d < 3; ++d) { c.periodicity[d] = p.periodicity[d]; c.volume_size[d] = p.volume_size[d]; }
        c.N = p.N; c.n = p.n; c.device_id = p.device_id;
        c.delta_t = p.delta_t; c.temperature = p.temperature;
        c.thermal_velocity = p.thermal_velocity; c.drag = p.drag;
        std::ifstream("/dev/urandom", std::ios::binary).read(reinterpret_cast<char*>(&c.seed), sizeof c.seed);
        if (mpcd_gb_create(&c, &h_) != MPCD_GB_OK)
            throw std::runtime_error(mpcd_gb_last_error(nullptr));
    }
    ~GbBackend() override { mpcd_gb_destroy(h_); }

    void step(int n) override                    { check(mpcd_gb_step(h_, n)); }
    void stepAndAccumulateSample(int n) override { check(mpcd_gb_step_and_sample(h_, n)); }
    void getSampleMean(std::vector<float>& d, std::vector<float>& v) override {
        d.resize(mpcd_gb_num_cells(h_)); v.resize(3 * d.size());
        check(mpcd_gb_get_sample_mean(h_, d.data(), v.data()));
    }
    size_t getNParticles() override { return mpcd_gb_num_particles(h_); }
    void getParticlePositions(std::vector<float>& x) override {
        x.resize(3 * getNParticles()); check(mpcd_gb_get_positions(h_, x.data()));
    }
    void getParticleVelocities(std::vector<float>& v) override {
        v.resize(3 * getNParticles()); check(mpcd_gb_get_velocities(h_, v.data()));
    }
    void setParticlePositions(std::vector<float> const& x) override  { check(mpcd_gb_set_positions(h_, x.data())); }
    void setParticleVelocities(std::vector<float> const& v) override { check(mpcd_gb_set_velocities(h_, v.data())); }
    void setParticles(std::vector<float> const& x, std::vector<float> const& v) override {
        check(mpcd_gb_set_particles(h_, x.data(), v.data()));
    }

private:
    void check(int32_t rc) { if (rc != MPCD_GB_OK) throw std::runtime_error(mpcd_gb_last_error(h_)); }
    mpcd_gb_handle* h_ = nullptr;
};

}  // namespace mpcd::gb300
