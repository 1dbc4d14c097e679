// Simulation parameters, declared field for field as the reference's
// mpcd::SimulationParameters (include/mpcd/api/simulation_parameters.hpp:53-102)
// so that code written against the reference API compiles unchanged; one field
// is added: the Philox seed of the GB300 backend.
#pragma once

#include <array>
#include <cstdint>
#include <string>

namespace mpcd {

enum class ExperimentType {
    standard,  // periodic box, walls where periodicity is 0
    channel,   // cylindrical channel along x
};

enum class MPCDAlgorithm {
    srd,       // stochastic rotation dynamics
    extended,  // extended MPC (stochastic gate, subgroup thermalisation)
};

enum class CollisionKernel {
    trivial,
    sorting,
    optimized,  // all three select the same fused GB300 kernel
};

struct SimulationParameters {
    ExperimentType experiment = ExperimentType::standard;
    MPCDAlgorithm algorithm = MPCDAlgorithm::srd;
    CollisionKernel collision_kernel = CollisionKernel::optimized;

    std::array<int, 3> periodicity = {1, 1, 1};
    std::array<float, 3> volume_size = {10.0f, 10.0f, 10.0f};

    unsigned int N = 0, n = 10, device_id = 0;

    float delta_t = 0.01f, temperature = 1.0f, thermal_velocity = 1.0f, drag = 0.0f;

    unsigned int equilibration_steps = 0, steps = 0, sample_every = 0, average_samples = 0;
    bool sample_fluid = false;
    bool write_backup = false, read_backup = false;
    std::string output_directory, load_directory;

    // Philox key of the GB300 backend; when seed_set is false the backend draws
    // one from /dev/urandom, as the reference seeds its generators.
    uint64_t seed = 0;
    bool seed_set = false;
};

}  // namespace mpcd
