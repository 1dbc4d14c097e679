#include "gb_backend.hpp"

#include <fstream>
#include <stdexcept>
#include <string>

namespace mpcd::gb300 {

namespace {
uint64_t urandom_seed()
{
    uint64_t s = 0;
    std::ifstream f("/dev/urandom", std::ios::binary);
    if (!f || !f.read(reinterpret_cast<char*>(&s), sizeof s))
        throw std::runtime_error("cannot read /dev/urandom for a seed");
    return s;
}
}  // namespace

GbBackend::GbBackend(SimulationParameters const& p) : Backend(p)
{
    mpcd_gb_params c{};
    c.experiment = p.experiment == ExperimentType::channel ? 1 : 0;
    c.algorithm = p.algorithm == MPCDAlgorithm::extended ? 1 : 0;
    c.collision_kernel = static_cast<int32_t>(p.collision_kernel);
    for (int d = 0; d < 3; ++d) {
        c.periodicity[d] = p.periodicity[d];
        c.volume_size[d] = p.volume_size[d];
    }
    c.N = p.N;
    c.n = p.n;
    c.device_id = p.device_id;
    c.delta_t = p.delta_t;
    c.temperature = p.temperature;
    c.thermal_velocity = p.thermal_velocity;
    c.drag = p.drag;
    c.seed = p.seed_set ? p.seed : urandom_seed();
    const int32_t rc = mpcd_gb_create(&c, &handle_);
    if (rc != MPCD_GB_OK) throw std::runtime_error(std::string("GB300 backend: ") + mpcd_gb_last_error(nullptr));
    parameters.seed = c.seed;
    parameters.seed_set = true;
    parameters.N = static_cast<unsigned int>(mpcd_gb_num_particles(handle_));
}

GbBackend::~GbBackend() { mpcd_gb_destroy(handle_); }

void GbBackend::check(int32_t rc) const
{
    if (rc != MPCD_GB_OK) throw std::runtime_error(std::string("GB300 backend: ") + mpcd_gb_last_error(handle_));
}

void GbBackend::step(int n_steps) { check(mpcd_gb_step(handle_, n_steps)); }

void GbBackend::stepAndAccumulateSample(int n_steps) { check(mpcd_gb_step_and_sample(handle_, n_steps)); }

void GbBackend::getSampleMean(std::vector<float>& mean_density, std::vector<float>& mean_velocity)
{
    const size_t C = mpcd_gb_num_cells(handle_);
    mean_density.resize(C);
    mean_velocity.resize(3 * C);
    check(mpcd_gb_get_sample_mean(handle_, mean_density.data(), mean_velocity.data()));
}

size_t GbBackend::getNParticles() { return mpcd_gb_num_particles(handle_); }

void GbBackend::getParticlePositions(std::vector<float>& positions)
{
    positions.resize(3 * getNParticles());
    check(mpcd_gb_get_positions(handle_, positions.data()));
}

void GbBackend::getParticleVelocities(std::vector<float>& velocities)
{
    velocities.resize(3 * getNParticles());
    check(mpcd_gb_get_velocities(handle_, velocities.data()));
}

void GbBackend::setParticlePositions(std::vector<float> const& positions)
{
    if (positions.size() != 3 * getNParticles()) throw std::runtime_error("positions must hold 3N floats");
    check(mpcd_gb_set_positions(handle_, positions.data()));
}

void GbBackend::setParticleVelocities(std::vector<float> const& velocities)
{
    if (velocities.size() != 3 * getNParticles()) throw std::runtime_error("velocities must hold 3N floats");
    check(mpcd_gb_set_velocities(handle_, velocities.data()));
}

void GbBackend::setParticles(std::vector<float> const& positions, std::vector<float> const& velocities)
{
    if (positions.size() != 3 * getNParticles() || velocities.size() != 3 * getNParticles())
        throw std::runtime_error("positions and velocities must hold 3N floats each");
    check(mpcd_gb_set_particles(handle_, positions.data(), velocities.data()));
}

}  // namespace mpcd::gb300
