// Python module _pympcd of cudampcd_gb300: the same classes, properties and
// methods as the reference binding (src/bindings/bindings.cpp:49-178), served
// by the GB300 backend.  Additions: Params.seed, Simulation.set_particle_* and
// Simulation.num_particles.
#include <cmath>
#include <cstddef>
#include <stdexcept>
#include <vector>

#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include "simulation_handle.hpp"

namespace py = pybind11;

using mpcd::CollisionKernel;
using mpcd::ExperimentType;
using mpcd::MPCDAlgorithm;
using mpcd::SimulationParameters;
using mpcd::api::SimulationHandle;

namespace {

// Hand a vector to numpy without a copy; the capsule owns it.
py::array_t<float> to_numpy(std::vector<float>&& v, std::vector<py::ssize_t> shape, std::vector<py::ssize_t> strides)
{
    auto* owned = new std::vector<float>(std::move(v));
    py::capsule owner(owned, [](void* p) { delete static_cast<std::vector<float>*>(p); });
    return py::array_t<float>(shape, strides, owned->data(), owner);
}

py::array_t<float> vectors_to_numpy(std::vector<float>&& v)
{
    const py::ssize_t n = static_cast<py::ssize_t>(v.size() / 3);
    return to_numpy(std::move(v), {n, 3}, {3 * (py::ssize_t)sizeof(float), (py::ssize_t)sizeof(float)});
}

std::vector<float> from_numpy(py::array_t<float, py::array::c_style | py::array::forcecast> a)
{
    return std::vector<float>(a.data(), a.data() + a.size());
}

unsigned fluid_count(SimulationParameters const& p)
{
    return static_cast<unsigned>(p.n * (p.volume_size[0] - 2 * (1 - p.periodicity[0])) *
                                 (p.volume_size[1] - 2 * (1 - p.periodicity[1])) *
                                 (p.volume_size[2] - 2 * (1 - p.periodicity[2])));
}

}  // namespace

PYBIND11_MODULE(_pympcd, m)
{
    m.doc() = "Multi-particle collision dynamics on one GB300 GPU (drop-in for pympcd).";

    py::class_<SimulationHandle>(m, "Simulation", "Handle of one simulation and its backend")
        .def(py::init<SimulationParameters const&, std::string>(), py::arg("params"), py::arg("backend") = "cuda")
        .def("step", &SimulationHandle::step, py::arg("n_steps"), py::call_guard<py::gil_scoped_release>(),
             "Perform n_steps simulation steps.")
        .def("step_and_sample", &SimulationHandle::stepAndAccumulateSample, py::arg("n_steps"),
             py::call_guard<py::gil_scoped_release>(), "Perform n_steps steps and accumulate the lab-grid sample.")
        .def(
            "get_mean_fields",
            [](SimulationHandle& self) {
                std::vector<float> density, velocity;
                {
                    py::gil_scoped_release release;
                    self.getSampleMean(density, velocity);
                }
                auto const& p = self.getParameters();
                const py::ssize_t x = (py::ssize_t)p.volume_size[0], y = (py::ssize_t)p.volume_size[1],
                                  z = (py::ssize_t)p.volume_size[2], sf = (py::ssize_t)sizeof(float);
                // Same shape and strides as the reference binding (bindings.cpp:62-72),
                // including its y stride of Ly (exact for Lx == Ly).
                std::vector<py::ssize_t> shape = {x, y, z}, strides = {sf, y * sf, x * y * sf};
                auto d = to_numpy(std::move(density), shape, strides);
                for (auto& s : strides) s *= 3;
                strides.push_back(sf);
                shape.push_back(3);
                auto v = to_numpy(std::move(velocity), shape, strides);
                return py::make_tuple(d, v);
            },
            "Mean density and velocity fields (voxel arrays) of the accumulated sample.")
        .def(
            "get_particle_positions",
            [](SimulationHandle const& self) {
                std::vector<float> out;
                {
                    py::gil_scoped_release release;
                    self.getParticlePositions(out);
                }
                return vectors_to_numpy(std::move(out));
            },
            "Particle positions, (N, 3) float32, by particle id (a fixed order).")
        .def(
            "get_particle_velocities",
            [](SimulationHandle const& self) {
                std::vector<float> out;
                {
                    py::gil_scoped_release release;
                    self.getParticleVelocities(out);
                }
                return vectors_to_numpy(std::move(out));
            },
            "Particle velocities, (N, 3) float32, by particle id.")
        .def(
            "set_particle_positions",
            [](SimulationHandle& self, py::array_t<float, py::array::c_style | py::array::forcecast> a) {
                self.setParticlePositions(from_numpy(a));
            },
            "Replace all positions ((N, 3), order of get_particle_positions).")
        .def(
            "set_particle_velocities",
            [](SimulationHandle& self, py::array_t<float, py::array::c_style | py::array::forcecast> a) {
                self.setParticleVelocities(from_numpy(a));
            },
            "Replace all velocities ((N, 3), order of get_particle_positions).")
        .def(
            "set_particles",
            [](SimulationHandle& self, py::array_t<float, py::array::c_style | py::array::forcecast> x,
               py::array_t<float, py::array::c_style | py::array::forcecast> v) {
                self.setParticles(from_numpy(x), from_numpy(v));
            },
            "Replace all positions and velocities.")
        .def_property_readonly("num_particles", &SimulationHandle::getNParticles);

    py::class_<SimulationParameters>(m, "Params", "Simulation parameters")
        .def(py::init<>())
        .def_readwrite("device_id", &SimulationParameters::device_id)
        .def_readwrite("delta_t", &SimulationParameters::delta_t)
        .def_readwrite("N", &SimulationParameters::N)
        .def_readwrite("drag", &SimulationParameters::drag)
        .def_readwrite("equilibration_steps", &SimulationParameters::equilibration_steps)
        .def_readwrite("steps", &SimulationParameters::steps)
        .def_readwrite("sample_rate", &SimulationParameters::sample_every)
        .def_readwrite("average_samples", &SimulationParameters::average_samples)
        .def_property(
            "temperature", [](SimulationParameters const& p) { return p.temperature; },
            [](SimulationParameters& p, double t) {
                p.temperature = (float)t;
                p.thermal_velocity = std::sqrt((float)t);
            })
        .def_property(
            "volume_size",
            [](SimulationParameters const& p) {
                return py::make_tuple(p.volume_size[0], p.volume_size[1], p.volume_size[2]);
            },
            [](SimulationParameters& p, py::sequence t) {
                if (py::len(t) != 3) throw std::runtime_error("Expected 3 elements");
                for (int i = 0; i < 3; ++i) {
                    p.volume_size[i] = t[i].cast<float>();
                    if (p.periodicity[i] == 0) p.volume_size[i] += 2;   // wall layer
                }
                p.N = fluid_count(p);
            })
        .def_property(
            "n", [](SimulationParameters const& p) { return p.n; },
            [](SimulationParameters& p, int n) {
                p.n = n;
                p.N = (unsigned)(p.n * p.volume_size[0] * p.volume_size[1] * p.volume_size[2]);
            })
        .def_property(
            "periodicity",
            [](SimulationParameters const& p) {
                return py::make_tuple(p.periodicity[0], p.periodicity[1], p.periodicity[2]);
            },
            [](SimulationParameters& p, py::sequence t) {
                if (py::len(t) != 3) throw std::runtime_error("Expected 3 elements");
                for (int i = 0; i < 3; ++i) {
                    p.periodicity[i] = t[i].cast<int>();
                    if (p.periodicity[i] == 0 && p.volume_size[i] != 0) p.volume_size[i] += 2;
                }
                p.N = fluid_count(p);
            })
        .def_property(
            "experiment",
            [](SimulationParameters const& p) {
                return p.experiment == ExperimentType::standard ? "standard" : "channel";
            },
            [](SimulationParameters& p, std::string const& e) {
                p.experiment = e == "standard" ? ExperimentType::standard : ExperimentType::channel;
            })
        .def_property(
            "algorithm",
            [](SimulationParameters const& p) { return p.algorithm == MPCDAlgorithm::srd ? "srd" : "extended"; },
            [](SimulationParameters& p, std::string const& a) {
                p.algorithm = a == "srd" ? MPCDAlgorithm::srd : MPCDAlgorithm::extended;
            })
        .def_property(
            "collision_kernel",
            [](SimulationParameters const& p) -> std::string {
                switch (p.collision_kernel) {
                case CollisionKernel::trivial: return "trivial";
                case CollisionKernel::sorting: return "sorting";
                default: return "optimized";
                }
            },
            [](SimulationParameters& p, std::string const& k) {
                if (k == "trivial") p.collision_kernel = CollisionKernel::trivial;
                else if (k == "sorting") p.collision_kernel = CollisionKernel::sorting;
                else p.collision_kernel = CollisionKernel::optimized;
            })
        .def_property(
            "seed", [](SimulationParameters const& p) -> py::object {
                if (!p.seed_set) return py::none();
                return py::int_(p.seed);
            },
            [](SimulationParameters& p, py::object s) {
                if (s.is_none()) {
                    p.seed_set = false;
                } else {
                    p.seed = s.cast<uint64_t>();
                    p.seed_set = true;
                }
            });

    m.attr("__version__") = "1.0.0";
}
