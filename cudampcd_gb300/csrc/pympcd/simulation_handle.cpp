#include "simulation_handle.hpp"

#include <stdexcept>

#include "gb_backend.hpp"

namespace mpcd {

std::unique_ptr<Backend> create_backend(SimulationParameters const& params, std::string const& backend_type)
{
    if (backend_type == "cuda") return std::make_unique<gb300::GbBackend>(params);
    throw std::runtime_error("Unsupported backend type");
}

namespace api {

SimulationHandle::SimulationHandle(SimulationParameters const& params, std::string backend_type)
    : backend_(create_backend(params, backend_type))
{
}

SimulationHandle::~SimulationHandle() = default;
SimulationHandle::SimulationHandle(SimulationHandle&&) noexcept = default;
SimulationHandle& SimulationHandle::operator=(SimulationHandle&&) noexcept = default;

SimulationParameters const& SimulationHandle::getParameters() const { return backend_->getParameters(); }

void SimulationHandle::step(int n_steps) { backend_->step(n_steps); }

void SimulationHandle::stepAndAccumulateSample(int n_steps) { backend_->stepAndAccumulateSample(n_steps); }

void SimulationHandle::getSampleMean(std::vector<float>& mean_density, std::vector<float>& mean_velocity)
{
    backend_->getSampleMean(mean_density, mean_velocity);
}

void SimulationHandle::getParticlePositions(std::vector<float>& positions) const
{
    backend_->getParticlePositions(positions);
}

void SimulationHandle::getParticleVelocities(std::vector<float>& velocities) const
{
    backend_->getParticleVelocities(velocities);
}

void SimulationHandle::setParticlePositions(std::vector<float> const& positions)
{
    backend_->setParticlePositions(positions);
}

void SimulationHandle::setParticleVelocities(std::vector<float> const& velocities)
{
    backend_->setParticleVelocities(velocities);
}

void SimulationHandle::setParticles(std::vector<float> const& positions, std::vector<float> const& velocities)
{
    backend_->setParticles(positions, velocities);
}

size_t SimulationHandle::getNParticles() const { return backend_->getNParticles(); }

}  // namespace api
}  // namespace mpcd
