// The reference's bridge class (include/mpcd/api/simulation_handle.hpp:14-45):
// owns one Backend chosen by name.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "backend.hpp"

namespace mpcd {

// Backend factory (reference: src/libmpcd/common/backend_factory.hpp:15-27).
// "cuda" selects the GB300 backend; any other name throws "Unsupported backend type".
std::unique_ptr<Backend> create_backend(SimulationParameters const& params, std::string const& backend_type);

namespace api {

class SimulationHandle {
public:
    SimulationHandle(SimulationParameters const&, std::string backend_type);
    ~SimulationHandle();

    SimulationHandle(SimulationHandle&&) noexcept;
    SimulationHandle& operator=(SimulationHandle&&) noexcept;
    SimulationHandle(const SimulationHandle&) = delete;
    SimulationHandle& operator=(const SimulationHandle&) = delete;

    SimulationParameters const& getParameters() const;

    void step(int n_steps);
    void stepAndAccumulateSample(int n_steps);
    void getSampleMean(std::vector<float>& mean_density, std::vector<float>& mean_velocity);

    void getParticlePositions(std::vector<float>& positions) const;
    void getParticleVelocities(std::vector<float>& velocities) const;
    void setParticlePositions(std::vector<float> const& positions);
    void setParticleVelocities(std::vector<float> const& velocities);
    void setParticles(std::vector<float> const& positions, std::vector<float> const& velocities);

    size_t getNParticles() const;

private:
    std::unique_ptr<Backend> backend_;
};

}  // namespace api
}  // namespace mpcd
