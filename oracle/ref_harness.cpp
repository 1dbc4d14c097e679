// Reference harness -- TEST INFRASTRUCTURE ONLY.
//
// Compiled by oracle/build_oracle.py together with the reference's own CPU
// sources, where they lie in the azantop/cudaMPCD tree
// (src/libmpcd/cpu_backend/simulation_functions.cpp, cpu_backend.cpp), into
// oracle/_ref/libmpcd_ref.so.  It exposes a C interface so that tests can run
// the reference CPU path with a seeded Xoshiro128+ stream and compare it with
// the C restatement in oracle/oracle.c.  Nothing in the product uses it.
//
// The reference CPUBackend keeps its RNG and particles private and seeds the
// RNG from /dev/urandom; to drive it deterministically this harness reaches the
// two members through pointers-to-member formed in explicit template
// instantiations (where access checking does not apply).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "cpu_backend/cpu_backend.hpp"
#include "cpu_backend/simulation_functions.hpp"

using namespace mpcd;

namespace {
template <typename Tag, typename Tag::type M>
struct Reach {
    friend typename Tag::type member(Tag) { return M; }
};
struct RandomTag {
    typedef Xoshiro128Plus cpu::CPUBackend::*type;
    friend type member(RandomTag);
};
struct ParticlesTag {
    typedef std::vector<Particle> cpu::CPUBackend::*type;
    friend type member(ParticlesTag);
};
template struct Reach<RandomTag, &cpu::CPUBackend::random>;
template struct Reach<ParticlesTag, &cpu::CPUBackend::particles>;

Xoshiro128Plus& rng_of(void* h) { return static_cast<cpu::CPUBackend*>(h)->*member(RandomTag{}); }
std::vector<Particle>& particles_of(void* h) { return static_cast<cpu::CPUBackend*>(h)->*member(ParticlesTag{}); }
}  // namespace

namespace {
SimulationParameters make_params(const int32_t L[3], const int32_t periodic[3], int32_t experiment,
                                 int32_t algorithm, float dt, float drag, float thermal_velocity,
                                 uint32_t n_density, uint32_t N)
{
    SimulationParameters p;
    for (int a = 0; a < 3; ++a) {
        p.volume_size[a] = static_cast<float>(L[a]);
        p.periodicity[a] = periodic[a];
    }
    p.experiment = experiment ? ExperimentType::channel : ExperimentType::standard;
    p.algorithm = algorithm ? MPCDAlgorithm::extended : MPCDAlgorithm::srd;
    p.delta_t = dt;
    p.drag = drag;
    p.thermal_velocity = thermal_velocity;
    p.temperature = thermal_velocity * thermal_velocity;
    p.n = n_density;
    p.N = N;
    return p;
}

void load(std::vector<Particle>& particles, const float* pos, const float* vel)
{
    for (size_t i = 0; i < particles.size(); ++i) {
        particles[i] = Particle{};
        particles[i].position = Vector(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        particles[i].velocity = Vector(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
    }
}

void store(const std::vector<Particle>& particles, float* pos, float* vel, uint32_t* cell)
{
    for (size_t i = 0; i < particles.size(); ++i) {
        pos[3 * i] = particles[i].position.x;
        pos[3 * i + 1] = particles[i].position.y;
        pos[3 * i + 2] = particles[i].position.z;
        vel[3 * i] = particles[i].velocity.x;
        vel[3 * i + 1] = particles[i].velocity.y;
        vel[3 * i + 2] = particles[i].velocity.z;
        if (cell) cell[i] = particles[i].cell_idx;
    }
}
}  // namespace

extern "C" {

void ref_xoshiro_sequence(uint64_t a, uint64_t b, int32_t kind, size_t n, void* out)
{
    Xoshiro128Plus r;
    r.seed(a, b);
    for (size_t i = 0; i < n; ++i) {
        switch (kind) {
        case 0: static_cast<uint32_t*>(out)[i] = r(); break;
        case 1: static_cast<float*>(out)[i] = r.genUniformFloat(); break;
        case 2: static_cast<float*>(out)[i] = r.gaussianf(); break;
        default: {
            Vector v = r.genUnitVector();
            float* o = static_cast<float*>(out) + 3 * i;
            o[0] = v.x; o[1] = v.y; o[2] = v.z;
        }
        }
    }
}

// cpu::distribute_particles with a seeded stream.
void ref_distribute(const int32_t L[3], const int32_t periodic[3], int32_t experiment, float thermal_velocity,
                    uint32_t N, uint64_t a, uint64_t b, float* pos, float* vel, uint32_t* cell)
{
    SimulationParameters p = make_params(L, periodic, experiment, 0, 0.01f, 0.0f, thermal_velocity, 1, N);
    cpu::VolumeContainer<MPCCell> cells({p.volume_size[0], p.volume_size[1], p.volume_size[2]});
    std::vector<Particle> particles(N);
    Xoshiro128Plus r;
    r.seed(a, b);
    cpu::distribute_particles(particles, cells, p, r);
    store(particles, pos, vel, cell);
}

// cpu::translate_particles; counter must be zeroed by the caller, table holds C*cap entries.
void ref_translate(const int32_t L[3], const int32_t periodic[3], int32_t experiment, float dt,
                   const float shift[3], uint32_t N, float* pos, float* vel, uint32_t* counter,
                   uint32_t* table, uint32_t cap, uint32_t* cell)
{
    cpu::VolumeContainer<MPCCell> cells({static_cast<float>(L[0]), static_cast<float>(L[1]), static_cast<float>(L[2])});
    std::vector<Particle> particles(N);
    load(particles, pos, vel);
    std::vector<uint32_t> cnt(counter, counter + cells.size());
    std::vector<uint32_t> tab(cells.size() * cap, 0u);
    Xoshiro128Plus r;
    r.seed(1, 2);
    cpu::translate_particles(particles, cells, r, Vector(shift[0], shift[1], shift[2]),
                             Vector(cells.getEdges()), IntVector(periodic[0], periodic[1], periodic[2]), dt,
                             experiment ? ExperimentType::channel : ExperimentType::standard, cnt, tab);
    store(particles, pos, vel, cell);
    std::copy(cnt.begin(), cnt.end(), counter);
    std::copy(tab.begin(), tab.end(), table);
}

// cpu::srd_collision / cpu::extended_collision with a Xoshiro128+ seeded (a, b).
void ref_collision(int32_t algorithm, const int32_t L[3], const int32_t periodic[3], float dt, float drag,
                   float thermal_velocity, uint32_t n_density, const float shift[3], uint32_t N, float* pos,
                   float* vel, const uint32_t* counter, const uint32_t* table, uint32_t cap, uint64_t a,
                   uint64_t b, uint32_t* cell)
{
    cpu::VolumeContainer<MPCCell> cells({static_cast<float>(L[0]), static_cast<float>(L[1]), static_cast<float>(L[2])});
    std::vector<Particle> particles(N);
    load(particles, pos, vel);
    std::vector<uint32_t> cnt(counter, counter + cells.size());
    std::vector<uint32_t> tab(table, table + cells.size() * cap);
    Xoshiro128Plus r;
    r.seed(a, b);
    auto fn = algorithm ? cpu::extended_collision : cpu::srd_collision;
    fn(particles, cells, r, Vector(shift[0], shift[1], shift[2]), Vector(cells.getEdges()),
       IntVector(periodic[0], periodic[1], periodic[2]), dt, drag, thermal_velocity, n_density, cnt, tab);
    store(particles, pos, vel, cell);
}

// Whole reference CPUBackend driven with a seeded stream.
void* ref_backend_create(const int32_t L[3], const int32_t periodic[3], int32_t experiment, int32_t algorithm,
                         float dt, float drag, float thermal_velocity, uint32_t n_density, uint32_t N)
{
    try {
        SimulationParameters p =
            make_params(L, periodic, experiment, algorithm, dt, drag, thermal_velocity, n_density, N);
        return new cpu::CPUBackend(p);
    } catch (...) {
        return nullptr;
    }
}

void ref_backend_destroy(void* h) { delete static_cast<cpu::CPUBackend*>(h); }

void ref_backend_seed(void* h, uint64_t a, uint64_t b) { rng_of(h).seed(a, b); }

void ref_backend_set(void* h, const float* pos, const float* vel)
{
    load(particles_of(h), pos, vel);
}

void ref_backend_get(void* h, float* pos, float* vel)
{
    store(particles_of(h), pos, vel, nullptr);
}

void ref_backend_step(void* h, int32_t n) { static_cast<cpu::CPUBackend*>(h)->step(n); }

void ref_backend_step_and_sample(void* h, int32_t n) { static_cast<cpu::CPUBackend*>(h)->stepAndAccumulateSample(n); }

void ref_backend_sample_mean(void* h, float* density, float* velocity)
{
    std::vector<float> d, v;
    static_cast<cpu::CPUBackend*>(h)->getSampleMean(d, v);
    std::copy(d.begin(), d.end(), density);
    std::copy(v.begin(), v.end(), velocity);
}

}  // extern "C"
