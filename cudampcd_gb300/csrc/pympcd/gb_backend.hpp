// mpcd::Backend implemented over the C ABI of libmpcd_gb.so (include/mpcd_gb.h).
#pragma once

#include <cstdint>
#include <vector>

#include "backend.hpp"
#include "mpcd_gb.h"

namespace mpcd::gb300 {

class GbBackend final : public Backend {
public:
    explicit GbBackend(SimulationParameters const& p);
    ~GbBackend() override;
    GbBackend(GbBackend const&) = delete;
    GbBackend& operator=(GbBackend const&) = delete;

    void step(int n_steps) override;
    void stepAndAccumulateSample(int n_steps) override;
    void getSampleMean(std::vector<float>& mean_density, std::vector<float>& mean_velocity) override;
    size_t getNParticles() override;
    void getParticlePositions(std::vector<float>& positions) override;
    void getParticleVelocities(std::vector<float>& velocities) override;
    void setParticlePositions(std::vector<float> const& positions) override;
    void setParticleVelocities(std::vector<float> const& velocities) override;
    void setParticles(std::vector<float> const& positions, std::vector<float> const& velocities) override;

    mpcd_gb_handle* handle() const { return handle_; }

private:
    void check(int32_t rc) const;
    mpcd_gb_handle* handle_ = nullptr;
};

}  // namespace mpcd::gb300
