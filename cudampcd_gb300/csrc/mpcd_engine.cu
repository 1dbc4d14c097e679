// Host engine of the GB300 MPCD step and the C ABI of include/mpcd_gb.h.
//
// One handle = one simulation on one GPU (or a batched ensemble of independent
// boxes advanced by the same launches): its device buffers, one CUDA stream,
// the step counter that keys every Philox draw, and the sampling state machine
// of the reference (cuda_backend_impl.cu:182-218).  No call synchronises
// except the getters, the sample read-out and the error check at the end of
// step()/step_and_sample().
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mpcd_gb.h"
#include "mpcd_kernels.h"

namespace mpcd_gb {
namespace {

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

// ---------------------------------------------------------------- host Philox (same draw model as the device)
void philox_host(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = (uint32_t)p1;
        c[2] = n2;
        c[3] = (uint32_t)p0;
    }
}

void shift_host(const BoxDesc& b, uint64_t step, float out[3])
{
    uint32_t c[4] = {0u, (uint32_t)step, 1u | ((uint32_t)(step >> 32) << 8), 0u};
    philox_host(c, b.seed_lo, b.seed_hi);
    for (int i = 0; i < 3; ++i) out[i] = (float)(c[i] >> 8) * 0x1p-24f - 0.5f;
}

// Device allocations the library has made in this process (mpcd_gb_device_allocations).
std::atomic<unsigned long long> g_device_allocations{0};

struct DeviceBuffer {
    void* p = nullptr;
    size_t bytes = 0;
    ~DeviceBuffer() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    cudaError_t alloc(size_t n)
    {
        release();
        if (n == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, n);
        g_device_allocations.fetch_add(1, std::memory_order_relaxed);
        if (e == cudaSuccess) bytes = n;
        else p = nullptr;
        return e;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

class Error : public std::exception {
public:
    Error(int code, std::string msg) : code_(code), msg_(std::move(msg)) {}
    const char* what() const noexcept override { return msg_.c_str(); }
    int code() const { return code_; }

private:
    int code_;
    std::string msg_;
};

void check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error(e == cudaErrorMemoryAllocation ? MPCD_GB_ENOMEM : MPCD_GB_ECUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
    }
}

}  // namespace

class Engine {
public:
    // R boxes (R = 1: a plain simulation); every box has its own geometry,
    // density, drag, temperature, time step and seed, all share the algorithm.
    Engine(const mpcd_gb_params* ps, int R) : params_(ps[0]), box_params_(ps, ps + R)
    {
        validate();
        build_boxes();   // host-side sizes and limits, before any CUDA call
        check(cudaSetDevice((int)params_.device_id), "cudaSetDevice");
        check(cudaStreamCreateWithFlags(&own_stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        stream_ = own_stream_;
        if (box_params_.size() > 1) {   // ensembles: the batch classes' side streams
            for (int i = 0; i < 2; ++i) {
                check(cudaStreamCreateWithFlags(&branches_.side[i], cudaStreamNonBlocking), "cudaStreamCreate");
                check(cudaEventCreateWithFlags(&branches_.join[i], cudaEventDisableTiming), "cudaEventCreate");
            }
            check(cudaEventCreateWithFlags(&branches_.fork, cudaEventDisableTiming), "cudaEventCreate");
        }
        cudaDeviceProp prop;
        check(cudaGetDeviceProperties(&prop, (int)params_.device_id), "cudaGetDeviceProperties");
        sms_ = prop.multiProcessorCount;
        allocate();
        configure();
        initialise();
    }

    ~Engine()
    {
        for (auto& g : graph_) g.reset();
        if (own_stream_) {
            cudaStreamSynchronize(own_stream_);
            cudaStreamDestroy(own_stream_);
        }
        for (int i = 0; i < 2; ++i) {
            if (branches_.side[i]) {
                cudaStreamSynchronize(branches_.side[i]);
                cudaStreamDestroy(branches_.side[i]);
            }
            if (branches_.join[i]) cudaEventDestroy(branches_.join[i]);
        }
        if (branches_.fork) cudaEventDestroy(branches_.fork);
    }

    // ------------------------------------------------------------ reference Backend interface
    void step(int n, bool sample)
    {
        if (n < 0) throw Error(MPCD_GB_EINVAL, "negative step count");
        for (int i = 0; i < n;) {
            const bool snapshot = sample && !sampling_;
            if (graphs_ && !snapshot && !use_table_ && step_ % kGraphSteps == 0 && n - i >= kGraphSteps) {
                const int done = replay_graph(sample, (n - i) / kGraphSteps);
                i += done;
                if (sample) sample_counter_ += (uint64_t)done;
                continue;
            }
            ++i;
            const uint64_t k = step_;
            // a sampled run-kernel step folds the previous step's sample itself; the
            // first sample after a restart (snapshot) and other kernels fold their own now
            const bool folded = launch_one_step(sample, sample && !snapshot);
            if (sample) {
                if (!folded)
                    check(launch_sample_finalize(sample_buffer(k), acc_.as<SampleAcc>(), cells_, snapshot ? 1 : 0,
                                                 sms_ * 8, stream_),
                          "sample finalize");
                if (snapshot) {
                    sampling_ = true;
                    sample_counter_ = 0;
                } else {
                    ++sample_counter_;
                }
            }
        }
        // the last step's sample (its buffer is clear if that step folded it already)
        if (sample && n > 0)
            check(launch_sample_finalize(sample_buffer(step_ - 1), acc_.as<SampleAcc>(), cells_, 0, sms_ * 8, stream_),
                  "sample finalize");
        check_device_errors();
    }

    // The lab-grid sums of step k: two buffers by step parity, so that a sampled step
    // can fold the previous step's while it fills its own.
    float4* sample_buffer(uint64_t k) const { return samp_.as<float4>() + (k & 1) * cells_; }

    // Mean fields of the FP64 sums (kept in storage order), gathered into the
    // reference order on the device: 16 bytes per cell cross to the host.
    void sample_mean(float* density, float* velocity)
    {
        if (!mean_.p) check(mean_.alloc(sizeof(float) * 4 * cells_), "alloc mean fields");
        float* d_density = mean_.as<float>();
        float* d_velocity = d_density + cells_;
        // cpu_backend.cpp:218 / cuda_backend_impl.cu:210: divide by the counter, S-1 for S samples
        const double inverse = 1.0 / (double)sample_counter_;
        for (const BoxDesc& b : boxes_)   // lab cells of every box, each in reference order
            check(launch_mean_fields(acc_.as<SampleAcc>(), b, inverse, d_density, d_velocity, stream_), "mean fields");
        check(cudaMemcpyAsync(density, d_density, sizeof(float) * cells_, cudaMemcpyDeviceToHost, stream_),
              "sample read");
        check(cudaMemcpyAsync(velocity, d_velocity, sizeof(float) * 3 * cells_, cudaMemcpyDeviceToHost, stream_),
              "sample read");
        check(cudaStreamSynchronize(stream_), "sample read");
        sampling_ = false;
    }

    void get(float* pos, float* vel)
    {
        materialise();
        if (pos)
            check(cudaMemcpyAsync(pos, dense_pos_.p, sizeof(float) * 3 * N_, cudaMemcpyDeviceToHost, stream_),
                  "positions read");
        if (vel)
            check(cudaMemcpyAsync(vel, dense_vel_.p, sizeof(float) * 3 * N_, cudaMemcpyDeviceToHost, stream_),
                  "velocities read");
        check(cudaStreamSynchronize(stream_), "particle read");
    }

    void set(const float* pos, const float* vel)
    {
        if (!pos || !vel) materialise();
        if (pos)
            check(cudaMemcpyAsync(dense_pos_.p, pos, sizeof(float) * 3 * N_, cudaMemcpyHostToDevice, stream_),
                  "positions write");
        if (vel)
            check(cudaMemcpyAsync(dense_vel_.p, vel, sizeof(float) * 3 * N_, cudaMemcpyHostToDevice, stream_),
                  "velocities write");
        scatter_dense();
        check(cudaStreamSynchronize(stream_), "particle write");
        check_device_errors();
    }

    void dump(uint32_t* cell, uint32_t* slot, uint32_t* id, uint32_t* counts)
    {
        DeviceBuffer dc, ds, di;
        check(dc.alloc(sizeof(uint32_t) * N_), "dump alloc");
        check(ds.alloc(sizeof(uint32_t) * N_), "dump alloc");
        check(di.alloc(sizeof(uint32_t) * N_), "dump alloc");
        layout(dc.as<uint32_t>(), ds.as<uint32_t>(), nullptr, di.as<uint32_t>());
        std::vector<uint32_t> hc(N_), hs(N_), hi(N_);
        check(cudaMemcpyAsync(hc.data(), dc.p, sizeof(uint32_t) * N_, cudaMemcpyDeviceToHost, stream_), "dump");
        check(cudaMemcpyAsync(hs.data(), ds.p, sizeof(uint32_t) * N_, cudaMemcpyDeviceToHost, stream_), "dump");
        check(cudaMemcpyAsync(hi.data(), di.p, sizeof(uint32_t) * N_, cudaMemcpyDeviceToHost, stream_), "dump");
        check(cudaStreamSynchronize(stream_), "dump");
        sort_overflow_tail(hc.data(), hs.data(), hi.data());
        if (cell) std::copy(hc.begin(), hc.end(), cell);
        if (slot) std::copy(hs.begin(), hs.end(), slot);
        if (id) std::copy(hi.begin(), hi.end(), id);
        if (counts) {
            std::vector<uint32_t> raw(cells_);
            check(cudaMemcpyAsync(raw.data(), count_[step_ % 3].p, sizeof(uint32_t) * cells_, cudaMemcpyDeviceToHost,
                                  stream_),
                  "dump");
            check(cudaStreamSynchronize(stream_), "dump");
            for (const BoxDesc& b : boxes_)
                for (uint32_t s = 0; s < b.C; ++s) {
                    const uint32_t Lz = (uint32_t)b.L[2], Lx = (uint32_t)b.L[0];
                    const uint32_t z = s % Lz, col = s / Lz, x = col % Lx, y = col / Lx;
                    counts[b.cell_base + x + Lx * (y + (uint32_t)b.L[1] * z)] = raw[b.cell_base + s];
                }
        }
        check(cudaStreamSynchronize(stream_), "dump");
    }

    // ------------------------------------------------------------ device-pointer I/O, drag
    void set_device(const float* d_pos, const float* d_vel)
    {
        if (!d_pos || !d_vel) materialise();
        if (d_pos)
            check(cudaMemcpyAsync(dense_pos_.p, d_pos, sizeof(float) * 3 * N_, cudaMemcpyDeviceToDevice, stream_),
                  "positions write");
        if (d_vel)
            check(cudaMemcpyAsync(dense_vel_.p, d_vel, sizeof(float) * 3 * N_, cudaMemcpyDeviceToDevice, stream_),
                  "velocities write");
        scatter_dense();
        check_device_errors();
    }

    void get_device(float* d_pos, float* d_vel)
    {
        materialise();
        if (d_pos)
            check(cudaMemcpyAsync(d_pos, dense_pos_.p, sizeof(float) * 3 * N_, cudaMemcpyDeviceToDevice, stream_),
                  "positions read");
        if (d_vel)
            check(cudaMemcpyAsync(d_vel, dense_vel_.p, sizeof(float) * 3 * N_, cudaMemcpyDeviceToDevice, stream_),
                  "velocities read");
        check(cudaStreamSynchronize(stream_), "particle read");
    }

    // Continue from the current particle state with the step counter (the key
    // of every Philox draw) set to k.
    void set_step(uint64_t k)
    {
        if (k >= (1ull << 40)) throw Error(MPCD_GB_EINVAL, "step index beyond 2^40");
        materialise();
        step_ = k;
        scatter_dense();
        check_device_errors();
        sampling_ = false;
    }

    // Wall pressure estimator: restart zeroes the impulse sums and measures every
    // step from now on; out = {bottom, top} pressure and the steps measured.
    void wall_pressure(bool restart, double out[3])
    {
        if (boxes_.size() != 1 || !boxes_[0].wall_z)
            throw Error(MPCD_GB_ESTATE, "the wall pressure needs a single box with walls in z");
        const size_t off = offsetof(DeviceState, wall_impulse);
        if (restart) {
            check(cudaMemsetAsync(static_cast<char*>(state_.p) + off, 0, 2 * sizeof(double), stream_), "pressure");
            if (!pressure_) {
                pressure_ = true;
                for (auto& g : graph_) g.reset();   // the graphs bake the flag into their launches
            }
            pressure_step0_ = step_;
        }
        double imp[2] = {0, 0};
        check(cudaMemcpyAsync(imp, static_cast<char*>(state_.p) + off, sizeof imp, cudaMemcpyDeviceToHost, stream_),
              "pressure");
        check(cudaStreamSynchronize(stream_), "pressure");
        const BoxDesc& b = boxes_[0];
        const double steps = (double)(step_ - pressure_step0_);
        const double norm = steps > 0 ? 1.0 / ((double)b.L[0] * b.L[1] * steps * b.dt) : 0.0;
        out[0] = imp[0] * norm;
        out[1] = imp[1] * norm;
        out[2] = steps;
    }

    // ------------------------------------------------------------ snapshots
    //
    // File layout (little-endian): "MPCDGBS1", u32 version = 1, u32 boxes, u64 step,
    // u64 N, per box {i32 experiment, i32 algorithm, i32 periodicity[3], f32
    // volume_size[3], u32 n, f32 delta_t, f32 temperature, f32 thermal_velocity,
    // f32 drag, u64 seed}, f32 positions[3N], f32 velocities[3N] (post-step state by
    // particle id), u64 FNV-1a of all preceding bytes.
    struct SnapshotBox {
        int32_t experiment, algorithm, periodicity[3];
        float volume_size[3];
        uint32_t n;
        float delta_t, temperature, thermal_velocity, drag;
        uint64_t seed;
    };

    static uint64_t fnv1a(uint64_t h, const void* data, size_t bytes)
    {
        const unsigned char* c = static_cast<const unsigned char*>(data);
        for (size_t i = 0; i < bytes; ++i) h = (h ^ c[i]) * 0x100000001B3ull;
        return h;
    }

    void save_snapshot(const char* path)
    {
        if (!path) throw Error(MPCD_GB_EINVAL, "null path");
        std::vector<float> pos(3 * N_), vel(3 * N_);
        get(pos.data(), vel.data());
        std::FILE* f = std::fopen(path, "wb");
        if (!f) throw Error(MPCD_GB_EINVAL, std::string("cannot open ") + path + " for writing");
        uint64_t h = 0xCBF29CE484222325ull;
        bool ok = true;
        auto put = [&](const void* d, size_t bytes) {
            h = fnv1a(h, d, bytes);
            ok = ok && std::fwrite(d, 1, bytes, f) == bytes;
        };
        const uint32_t version = 1, boxes = (uint32_t)box_params_.size();
        const uint64_t step = step_, n = N_;
        put("MPCDGBS1", 8);
        put(&version, 4);
        put(&boxes, 4);
        put(&step, 8);
        put(&n, 8);
        for (const mpcd_gb_params& p : box_params_) {
            SnapshotBox b{};
            b.experiment = p.experiment;
            b.algorithm = p.algorithm;
            for (int d = 0; d < 3; ++d) {
                b.periodicity[d] = p.periodicity[d];
                b.volume_size[d] = p.volume_size[d];
            }
            b.n = p.n;
            b.delta_t = p.delta_t;
            b.temperature = p.temperature;
            b.thermal_velocity = p.thermal_velocity;
            b.drag = p.drag;
            b.seed = p.seed;
            put(&b, sizeof b);
        }
        put(pos.data(), sizeof(float) * pos.size());
        put(vel.data(), sizeof(float) * vel.size());
        ok = ok && std::fwrite(&h, 1, 8, f) == 8;
        ok = (std::fclose(f) == 0) && ok;
        if (!ok) throw Error(MPCD_GB_EINVAL, std::string("write to ") + path + " failed");
    }

    void load_snapshot(const char* path)
    {
        if (!path) throw Error(MPCD_GB_EINVAL, "null path");
        std::FILE* f = std::fopen(path, "rb");
        if (!f) throw Error(MPCD_GB_EINVAL, std::string("cannot open ") + path);
        uint64_t h = 0xCBF29CE484222325ull;
        bool ok = true;
        auto get_bytes = [&](void* d, size_t bytes) {
            ok = ok && std::fread(d, 1, bytes, f) == bytes;
            if (ok) h = fnv1a(h, d, bytes);
        };
        char magic[8] = {};
        uint32_t version = 0, boxes = 0;
        uint64_t step = 0, n = 0, stored = 0;
        get_bytes(magic, 8);
        get_bytes(&version, 4);
        get_bytes(&boxes, 4);
        get_bytes(&step, 8);
        get_bytes(&n, 8);
        auto fail = [&](const char* why) {
            std::fclose(f);
            throw Error(MPCD_GB_EINVAL, std::string("snapshot ") + path + ": " + why);
        };
        if (!ok || std::memcmp(magic, "MPCDGBS1", 8) != 0 || version != 1) fail("not a version-1 snapshot");
        if (boxes != box_params_.size() || n != N_) fail("box count or particle count differs from the handle");
        for (const mpcd_gb_params& p : box_params_) {
            SnapshotBox b{};
            get_bytes(&b, sizeof b);
            bool same = ok && b.experiment == p.experiment && b.algorithm == p.algorithm && b.n == p.n &&
                        b.delta_t == p.delta_t && b.thermal_velocity == p.thermal_velocity && b.drag == p.drag &&
                        b.seed == p.seed;
            for (int d = 0; d < 3; ++d)
                same = same && b.periodicity[d] == p.periodicity[d] && b.volume_size[d] == p.volume_size[d];
            if (!same) fail("box parameters or seed differ from the handle's");
        }
        std::vector<float> pos(3 * N_), vel(3 * N_);
        get_bytes(pos.data(), sizeof(float) * pos.size());
        get_bytes(vel.data(), sizeof(float) * vel.size());
        const uint64_t computed = h;
        ok = ok && std::fread(&stored, 1, 8, f) == 8;
        if (!ok) fail("truncated");
        if (stored != computed) fail("checksum mismatch");
        std::fclose(f);
        if (step >= (1ull << 40)) throw Error(MPCD_GB_EINVAL, "snapshot step index beyond 2^40");
        step_ = step;
        check(cudaMemcpyAsync(dense_pos_.p, pos.data(), sizeof(float) * 3 * N_, cudaMemcpyHostToDevice, stream_),
              "snapshot positions");
        check(cudaMemcpyAsync(dense_vel_.p, vel.data(), sizeof(float) * 3 * N_, cudaMemcpyHostToDevice, stream_),
              "snapshot velocities");
        scatter_dense();
        check(cudaStreamSynchronize(stream_), "snapshot");
        check_device_errors();
        sampling_ = false;
        adj_valid_ = false;
    }

    // Body force of every box from the next step on.
    void set_drag(float drag)
    {
        if (!std::isfinite(drag)) throw Error(MPCD_GB_EINVAL, "drag must be finite");
        if (step_ > 0) materialise();   // a later replay of the last step must still use its drag
        for (size_t r = 0; r < boxes_.size(); ++r) {
            box_params_[r].drag = drag;
            boxes_[r].drag_dt = drag * boxes_[r].dt;
        }
        params_.drag = drag;
        check(cudaStreamSynchronize(stream_), "set drag");
        check(cudaMemcpy(boxes_d_.p, boxes_.data(), sizeof(BoxDesc) * boxes_.size(), cudaMemcpyHostToDevice),
              "upload boxes");
        for (auto& g : graph_) g.reset();
    }

    // ------------------------------------------------------------ adjoint of the sampled profile
    //
    // Forward: from the current state, `steps` sampled steps; the dense state is
    // checkpointed every `every` steps.  Backward: per segment, last first,
    // restore its checkpoint, recompute its steps recording the tape (the draws
    // are replayed from the Philox counters, the recomputation is bit-identical),
    // then run the reverse sweep over them.
    void profile_forward(int steps, int every, float* d_profile)
    {
        if (boxes_.size() != 1 || params_.algorithm != 0)
            throw Error(MPCD_GB_ESTATE, "the profile adjoint needs a single-box SRD handle");
        if (steps < 1 || every < 1) throw Error(MPCD_GB_EINVAL, "steps and checkpoint interval must be positive");
        if (!d_profile) throw Error(MPCD_GB_EINVAL, "null profile buffer");
        if (use_table_) throw Error(MPCD_GB_ESTATE, "injected draws pending");
        const int nseg = (steps + every - 1) / every;
        const size_t per = sizeof(float) * 6 * N_;
        if (ckpt_.bytes < per * nseg) check(ckpt_.alloc(per * nseg), "alloc checkpoints");
        adj_valid_ = false;
        adj_s0_ = step_;
        adj_steps_ = steps;
        adj_every_ = every;
        sampling_ = false;
        for (int j = 0; j < nseg; ++j) {
            materialise();
            char* c = static_cast<char*>(ckpt_.p) + per * j;
            check(cudaMemcpyAsync(c, dense_pos_.p, per / 2, cudaMemcpyDeviceToDevice, stream_), "checkpoint");
            check(cudaMemcpyAsync(c + per / 2, dense_vel_.p, per / 2, cudaMemcpyDeviceToDevice, stream_),
                  "checkpoint");
            step(std::min(every, steps - j * every), true);
        }
        check(launch_profile(acc_.as<SampleAcc>(), boxes_[0], (uint64_t)steps, d_profile, stream_), "profile");
        check(cudaStreamSynchronize(stream_), "profile");
        adj_valid_ = true;
    }

    void profile_backward(const float* d_dU, float* d_dv0, double* ddrag)
    {
        if (!adj_valid_) throw Error(MPCD_GB_ESTATE, "no profile forward to differentiate");
        if (!d_dU || !d_dv0 || !ddrag) throw Error(MPCD_GB_EINVAL, "null argument");
        const BoxDesc& b = boxes_[0];
        alloc_tape();
        check(cudaMemsetAsync(lam_.p, 0, lam_.bytes, stream_), "adjoint");
        check(cudaMemsetAsync(gsum_.p, 0, gsum_.bytes, stream_), "adjoint");
        const int nseg = (adj_steps_ + adj_every_ - 1) / adj_every_;
        for (int j = nseg - 1; j >= 0; --j) {
            const int k = record_segment(j);
            for (int i = k - 1; i >= 0; --i) {
                const uint64_t t = adj_s0_ + (uint64_t)j * adj_every_ + i;
                check(launch_adjoint_step(b, t, (uint64_t)adj_steps_, lam_.as<float>(),
                                          tkey_.as<uint32_t>() + (size_t)i * N_, tlab_.as<uint32_t>() + (size_t)i * N_,
                                          tncell_.as<uint32_t>() + (size_t)i * cells_,
                                          tcnt_.as<uint32_t>() + (size_t)i * cells_, d_dU, cellsum_.as<float4>(),
                                          gsum_.as<double>(), sms_ * 8, stream_),
                      "adjoint step");
            }
        }
        check(launch_adjoint_finish((uint32_t)N_, lam_.as<float>(), tb0_.as<uint32_t>(), d_dv0, sms_ * 8, stream_),
              "adjoint");
        double g = 0;
        check(cudaMemcpyAsync(&g, gsum_.p, sizeof g, cudaMemcpyDeviceToHost, stream_), "adjoint");
        check(cudaStreamSynchronize(stream_), "adjoint");
        check_device_errors();
        *ddrag = g * (double)b.dt;
        sampling_ = false;
    }

    // Test hook: the tape of every step of the last profile forward (host arrays
    // of steps * N, steps * N, steps * C, steps * C and N entries).
    void profile_tape(uint32_t* key, uint32_t* lab, uint32_t* ncell, uint32_t* lab_count, uint32_t* bounce0)
    {
        if (!adj_valid_) throw Error(MPCD_GB_ESTATE, "no profile forward recorded");
        alloc_tape();
        const int nseg = (adj_steps_ + adj_every_ - 1) / adj_every_;
        for (int j = 0; j < nseg; ++j) {
            const int k = record_segment(j);
            const size_t t0 = (size_t)j * adj_every_;
            auto down = [&](uint32_t* dst, const DeviceBuffer& src, size_t per) {
                if (dst)
                    check(cudaMemcpyAsync(dst + t0 * per, src.p, sizeof(uint32_t) * per * k, cudaMemcpyDeviceToHost,
                                          stream_),
                          "tape read");
            };
            down(key, tkey_, N_);
            down(lab, tlab_, N_);
            down(ncell, tncell_, cells_);
            down(lab_count, tcnt_, cells_);
            if (j == 0 && bounce0)
                check(cudaMemcpyAsync(bounce0, tb0_.p, sizeof(uint32_t) * N_, cudaMemcpyDeviceToHost, stream_),
                      "tape read");
            check(cudaStreamSynchronize(stream_), "tape read");
        }
        check_device_errors();
        sampling_ = false;
    }

    // Cell offsets of the current layout into a caller's device buffer; the
    // scan's scratch is the library's static per-device array, nothing is allocated.
    void cell_offsets_noalloc(uint32_t* d_offsets, uint64_t n_offsets)
    {
        char msg[160];
        if (cells_ > MPCD_GB_NOALLOC_MAX_CELLS) {
            std::snprintf(msg, sizeof msg, "cell offsets: %llu cells exceed the limit of %llu of the static scan scratch",
                          (unsigned long long)cells_, (unsigned long long)MPCD_GB_NOALLOC_MAX_CELLS);
            throw Error(MPCD_GB_EINVAL, msg);
        }
        if (!d_offsets) throw Error(MPCD_GB_EINVAL, "cell offsets: null output buffer");
        if (n_offsets < cells_ + 1) {
            std::snprintf(msg, sizeof msg, "cell offsets: buffer of %llu entries, %llu needed",
                          (unsigned long long)n_offsets, (unsigned long long)(cells_ + 1));
            throw Error(MPCD_GB_EINVAL, msg);
        }
        StepArgs a = args(step_);
        check(launch_cell_offsets_static(a, count_[step_ % 3].as<uint32_t>(), cells_, d_offsets,
                                         (int)params_.device_id, stream_),
              "cell offsets");
    }

    // The overflow list is filled in arrival order; order its part of a dump (the
    // last layout_tail_ entries) by (cell, id) so that a dump is deterministic.
    void sort_overflow_tail(uint32_t* cell, uint32_t* slot, uint32_t* id)
    {
        const uint64_t m = layout_tail_;
        if (m < 2) return;
        const uint64_t base = N_ - m;
        std::vector<uint64_t> order(m);
        for (uint64_t i = 0; i < m; ++i) order[i] = i;
        std::sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) {
            const uint32_t ca = cell[base + a], cb = cell[base + b];
            return ca != cb ? ca < cb : id[base + a] < id[base + b];
        });
        auto permute = [&](uint32_t* v) {
            if (!v) return;
            std::vector<uint32_t> t(m);
            for (uint64_t i = 0; i < m; ++i) t[i] = v[base + order[i]];
            std::copy(t.begin(), t.end(), v + base);
        };
        permute(cell);
        permute(slot);
        permute(id);
    }

    // ------------------------------------------------------------ hooks
    void inject_shift(uint64_t step, const float s[3])
    {
        int slot = -1;
        for (int i = 0; i < kMaxInjectedShifts; ++i)
            if (inject_valid_[i] && inject_step_[i] == step) slot = i;
        for (int i = 0; i < kMaxInjectedShifts && slot < 0; ++i)
            if (!inject_valid_[i] || inject_step_[i] < step_) slot = i;
        if (slot < 0) throw Error(MPCD_GB_ESTATE, "too many pending injected shifts");
        inject_valid_[slot] = 1;
        inject_step_[slot] = step;
        for (int d = 0; d < 3; ++d) inject_shift_[slot][d] = s[d];
        sync_injections();
    }

    void get_shift(uint64_t step, float out[3]) const
    {
        for (int i = 0; i < kMaxInjectedShifts; ++i)
            if (inject_valid_[i] && inject_step_[i] == step) {
                for (int d = 0; d < 3; ++d) out[d] = inject_shift_[i][d];
                return;
            }
        shift_host(boxes_[0], step, out);
    }

    void inject_draws(uint32_t gmax, uint32_t pmax, const uint32_t* ghost_count, const float* ghost_pos,
                      const float* ghost_vel, const float* axis, const float* gate_u, const float* gauss)
    {
        if (!ghost_count || !axis) {
            use_table_ = false;
            return;
        }
        if (boxes_.size() != 1) throw Error(MPCD_GB_ESTATE, "injected draws need a single-box handle");
        const size_t C = boxes_[0].C;
        check(t_count_.alloc(sizeof(uint32_t) * C), "draws alloc");
        check(t_gpos_.alloc(sizeof(float) * C * gmax * 3 + 16), "draws alloc");
        check(t_gvel_.alloc(sizeof(float) * C * gmax * 3 + 16), "draws alloc");
        check(t_axis_.alloc(sizeof(float) * C * 3), "draws alloc");
        check(t_gate_.alloc(sizeof(float) * C), "draws alloc");
        check(t_gauss_.alloc(sizeof(float) * C * pmax + 16), "draws alloc");
        auto up = [&](DeviceBuffer& d, const void* h, size_t n) {
            if (h && n) check(cudaMemcpyAsync(d.p, h, n, cudaMemcpyHostToDevice, stream_), "draws upload");
            else check(cudaMemsetAsync(d.p, 0, d.bytes, stream_), "draws upload");
        };
        up(t_count_, ghost_count, sizeof(uint32_t) * C);
        up(t_gpos_, ghost_pos, sizeof(float) * C * gmax * 3);
        up(t_gvel_, ghost_vel, sizeof(float) * C * gmax * 3);
        up(t_axis_, axis, sizeof(float) * C * 3);
        up(t_gate_, gate_u, sizeof(float) * C);
        up(t_gauss_, gauss, sizeof(float) * C * pmax);
        tables_ = DrawTables{t_count_.as<uint32_t>(), t_gpos_.as<float>(), t_gvel_.as<float>(), t_axis_.as<float>(),
                             t_gate_.as<float>(), t_gauss_.as<float>(), gmax, pmax};
        check(cudaStreamSynchronize(stream_), "draws upload");
        use_table_ = true;
    }

    void counters(uint64_t out[2])
    {
        DeviceState st;
        check(cudaMemcpyAsync(&st, state_.p, sizeof st, cudaMemcpyDeviceToHost, stream_), "counters");
        check(cudaStreamSynchronize(stream_), "counters");
        out[0] = st.overflow_total;
        out[1] = st.error_flags;
    }

    void set_stream(void* s) { stream_ = s ? static_cast<cudaStream_t>(s) : own_stream_; }
    void synchronize() { check(cudaStreamSynchronize(stream_), "synchronize"); }

    void time_steps(int n, float* total_ms, float* kernel_ms)
    {
        cudaEvent_t e0, e1;
        check(cudaEventCreate(&e0), "event");
        check(cudaEventCreate(&e1), "event");
        std::vector<cudaEvent_t> ks(2 * (size_t)n);
        for (auto& e : ks) check(cudaEventCreate(&e), "event");
        check(cudaEventRecord(e0, stream_), "event");
        for (int i = 0; i < n; ++i) launch_one_step(false, false, ks[2 * i], ks[2 * i + 1]);
        check(cudaEventRecord(e1, stream_), "event");
        check(cudaEventSynchronize(e1), "event");
        float t = 0, k = 0;
        check(cudaEventElapsedTime(&t, e0, e1), "event");
        for (int i = 0; i < n; ++i) {
            float dt = 0;
            check(cudaEventElapsedTime(&dt, ks[2 * i], ks[2 * i + 1]), "event");
            k += dt;
        }
        for (auto& e : ks) cudaEventDestroy(e);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (total_ms) *total_ms = t;
        if (kernel_ms) *kernel_ms = k;
        check_device_errors();
    }

    size_t num_particles() const { return N_; }
    size_t num_cells() const { return cells_; }
    uint64_t step_index() const { return step_; }
    int num_boxes() const { return (int)boxes_.size(); }

    void box_range(int r, uint64_t out[4]) const
    {
        if (r < 0 || r >= (int)boxes_.size()) throw Error(MPCD_GB_EINVAL, "box index out of range");
        const BoxDesc& b = boxes_[(size_t)r];
        out[0] = b.dense_base;
        out[1] = b.N;
        out[2] = b.cell_base;
        out[3] = b.C;
    }

    // Time `steps` real steps of every admissible (buffer, fill factor) pair --
    // each box then takes its own tile size -- and keep the fastest; the steps
    // advance the simulation like any others.
    void autotune(int steps, uint32_t out[2])
    {
        if (steps < 1) throw Error(MPCD_GB_EINVAL, "autotune needs at least one step per candidate");
        uint32_t n_max = 0;
        for (const BoxDesc& b : boxes_) n_max = std::max(n_max, b.n);
        cudaEvent_t e0, e1;
        check(cudaEventCreate(&e0), "event");
        check(cudaEventCreate(&e1), "event");
        float best = -1.0f;
        double best_fill = fill_;
        uint32_t best_pbuf = pbuf_;
        std::vector<std::vector<uint32_t>> tried;   // tilings already timed (per-box tile cells + buffer)
        // buffers: 1408 keeps 4 SRD CTAs per SM with 128-cell tiles, 1344 extended ones
        for (uint32_t pbuf : {1024u, 1280u, 1344u, 1408u, 1536u, 2048u}) {
            if (pbuf < 5 * n_max) continue;
            for (double fill : {1.0, 1.15, 1.3, 1.6, 2.0, 3.0}) {
                std::vector<uint32_t> key{pbuf};
                for (const BoxDesc& b : boxes_) key.push_back(tile_for(b.n, fill, pbuf));
                if (std::find(tried.begin(), tried.end(), key) != tried.end()) continue;
                tried.push_back(key);
                retile(fill, pbuf);
                launch_one_step(false);   // first launch of a configuration: not timed
                check(cudaEventRecord(e0, stream_), "event");
                for (int i = 0; i < steps; ++i) launch_one_step(false);
                check(cudaEventRecord(e1, stream_), "event");
                check(cudaEventSynchronize(e1), "event");
                float ms = 0;
                check(cudaEventElapsedTime(&ms, e0, e1), "event");
                check_device_errors();
                if (best < 0 || ms < best) {
                    best = ms;
                    best_fill = fill;
                    best_pbuf = pbuf;
                }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        retile(best_fill, best_pbuf);
        out[0] = max_tile_cells_;
        out[1] = best_pbuf;
    }

private:
    unsigned parity() const { return (unsigned)(step_ & 1); }

    void validate()
    {
        if (box_params_.empty()) throw Error(MPCD_GB_EINVAL, "an ensemble needs at least one box");
        for (const mpcd_gb_params& p : box_params_) {
            validate_one(p);
            if (p.algorithm != params_.algorithm) throw Error(MPCD_GB_EINVAL, "all boxes must use the same algorithm");
            if (p.device_id != params_.device_id) throw Error(MPCD_GB_EINVAL, "all boxes must use the same device");
        }
    }

    static void validate_one(const mpcd_gb_params& p)
    {
        for (int d = 0; d < 3; ++d) {
            const float L = p.volume_size[d];
            if (!(L >= 1.0f) || L != std::floor(L) || L > 65536.0f)
                throw Error(MPCD_GB_EINVAL, "volume_size must hold positive integers");
            if (p.periodicity[d] != 0 && p.periodicity[d] != 1)
                throw Error(MPCD_GB_EINVAL, "periodicity must be 0 or 1");
            if (!p.periodicity[d] && L < 3.0f) throw Error(MPCD_GB_EINVAL, "a walled axis needs at least 3 layers");
        }
        if (p.n < 1) throw Error(MPCD_GB_EINVAL, "n must be at least 1");
        if (p.algorithm != 0 && p.algorithm != 1) throw Error(MPCD_GB_EINVAL, "algorithm must be srd or extended");
        if (p.experiment != 0 && p.experiment != 1) throw Error(MPCD_GB_EINVAL, "experiment must be standard or channel");
        if (!(p.delta_t > 0.0f) || !std::isfinite(p.delta_t)) throw Error(MPCD_GB_EINVAL, "delta_t must be positive");
        if (!std::isfinite(p.thermal_velocity) || p.thermal_velocity < 0.0f)
            throw Error(MPCD_GB_EINVAL, "thermal_velocity must be finite and non-negative");
        if (!std::isfinite(p.drag)) throw Error(MPCD_GB_EINVAL, "drag must be finite");
    }

    static BoxDesc make_box(const mpcd_gb_params& p)
    {
        BoxDesc b{};
        uint64_t Nf = p.n;
        for (int d = 0; d < 3; ++d) {
            b.L[d] = (int32_t)p.volume_size[d];
            b.Lf[d] = p.volume_size[d];
            b.L15[d] = 1.5f * b.Lf[d];
            b.L2x[d] = 2.0f * b.Lf[d];
            b.L3x[d] = 3.0f * b.Lf[d];
            b.Lh[d] = b.Lf[d] * 0.5f;
            b.periodic[d] = p.periodicity[d];
            Nf *= (uint64_t)(b.L[d] - 2 * (1 - b.periodic[d]));
        }
        b.wall_z = !p.periodicity[2];
        b.channel = p.experiment == 1;
        b.dt = p.delta_t;
        b.drag_dt = p.drag * p.delta_t;
        b.tv = p.thermal_velocity;
        b.R2 = (b.Lf[2] - 2) * (b.Lf[2] - 2) * 0.25f;
        // simulation_functions.cpp:118-119: sinf / cosf of 120 degrees in float
        b.sin_a = sinf((float)((M_PI * 120) / 180));
        b.cos_a = cosf((float)((M_PI * 120) / 180));
        b.n = p.n;
        b.cap = 4 * p.n;
        // bucket depth: n + 4 sqrt(n) + 2 (a Poisson(n) cell exceeds it in about 1 of
        // 10^4..10^5 cells), at most the reference's 4n
        b.depth = std::min(b.cap, p.n + (uint32_t)std::ceil(4.0 * std::sqrt((double)p.n)) + 2u);
        if (const char* e = std::getenv("MPCD_GB_BUCKET_DEPTH")) {   // test hook: force spills
            const uint32_t v = (uint32_t)std::strtoul(e, nullptr, 10);
            if (v >= 1) b.depth = std::min(b.cap, v);
        }
        const uint64_t C = (uint64_t)b.L[0] * b.L[1] * b.L[2];
        if (C >= (1ull << 31)) throw Error(MPCD_GB_EINVAL, "too many cells");
        if (Nf >= (1ull << 32) - 1) throw Error(MPCD_GB_EINVAL, "too many particles");
        b.C = (uint32_t)C;
        b.N = (uint32_t)Nf;
        b.div_z = ((1ull << 48) + (uint64_t)b.L[2] - 1) / (uint64_t)b.L[2];
        b.div_x = ((1ull << 48) + (uint64_t)b.L[0] - 1) / (uint64_t)b.L[0];
        b.seed_lo = (uint32_t)p.seed;
        b.seed_hi = (uint32_t)(p.seed >> 32);
        return b;
    }

    void build_boxes()
    {
        boxes_.clear();
        uint64_t cells = 0, slots = 0, particles = 0, walls = 0;
        uint32_t n_max = 0;
        for (const mpcd_gb_params& p : box_params_) {
            BoxDesc b = make_box(p);
            if (cells + b.C >= (1ull << 31)) throw Error(MPCD_GB_EINVAL, "too many cells in the ensemble");
            b.cell_base = (uint32_t)cells;
            b.slot_base = slots;
            b.dense_base = particles;
            b.wall_base = walls;
            // run-kernel batches of about 80-96 particles: 16 cells up to n = 6, 8 up to 12, else 4
            b.run_batch = b.n <= 6 ? 16u : (b.n <= 12 ? 8u : 4u);
            if (const char* e = std::getenv("MPCD_GB_RUN_BATCH")) {   // tuning sweeps
                const uint32_t v = (uint32_t)std::strtoul(e, nullptr, 10);
                if (v == 4 || v == 8 || v == 16) b.run_batch = v;
            }
            if (b.wall_z) walls += 2ull * (uint64_t)b.L[0] * (uint64_t)b.L[1];
            cells += b.C;
            slots += (uint64_t)b.C * b.depth;
            particles += b.N;
            n_max = std::max(n_max, b.n);
            boxes_.push_back(b);
        }
        if (particles >= (1ull << 32) - 1) throw Error(MPCD_GB_EINVAL, "too many particles in the ensemble");
        N_ = particles;
        cells_ = cells;
        walls_ = walls;
        n_max_ = n_max;
        total_slots_ = slots;
        ov_cap_ = (uint32_t)std::max<uint64_t>(1u << 16, std::min<uint64_t>(N_, 1u << 22));
        // extension area: the colliding sets of the cells past their depth (at most N
        // particles in all; at least one cell's 4n)
        uint32_t cap_max = 0;
        for (const BoxDesc& b : boxes_) cap_max = std::max(cap_max, b.cap);
        ext_cap_ = (uint32_t)std::max<uint64_t>(cap_max, std::min<uint64_t>(N_, 1u << 22));
        if (total_slots_ + ext_cap_ + ov_cap_ >= (1ull << 32))
            throw Error(MPCD_GB_EINVAL, "bucket slots exceed the 32-bit slot space of one handle");
        // tiles: per box a power-of-two number of cells (a group of 256 / cells
        // threads per cell) holding up to pbuf particles on average; the buffer
        // holds one cell with all its ghosts (cap + n = 5n) at least.  The
        // default buffer keeps 4 CTAs per SM: 1408 particles with SRD's 128-cell
        // tiles (at 1536 their 58 KB of shared memory allows only 3), 1344 with the
        // extended collision's 64-cell tiles (38 B per particle); the autotuner
        // confirmed both as the fastest buffers at n = 5, 10 and 20.
        const uint32_t pbuf_default = params_.algorithm == 1 ? 1344u : 1408u;
        uint32_t pbuf = 5 * n_max <= pbuf_default ? pbuf_default : std::max(1536u, 5 * n_max);
        if (pbuf > 2048) throw Error(MPCD_GB_EINVAL, "n above 409: one cell and its ghosts must fit a tile");
        // tuning overrides (used by the tuning sweeps)
        if (const char* e = std::getenv("MPCD_GB_PBUF")) {
            const uint32_t v = (uint32_t)std::strtoul(e, nullptr, 10);
            if (v >= 5 * n_max && v <= 2048) pbuf = v;
        }
        if (const char* e = std::getenv("MPCD_GB_TILE_CELLS")) {
            const uint32_t v = (uint32_t)std::strtoul(e, nullptr, 10);
            if (v >= 8 && v <= tile_cells_max() && (v & (v - 1)) == 0) forced_tile_cells_ = v;
        }
        set_tiles(1.0, pbuf);
        float table[13][3];
        const int steps = 4;
        for (int select = 0; select <= 12; ++select) {   // simulation_functions.cpp:272-290
            const int phi_i = select % steps + 1, theta_i = select / steps + 1;
            float theta, phi;
            if ((theta_i % 2) && (phi_i % 2))
                theta = theta_i == 1 ? 0.95531661812450927816f : (float)M_PI - 0.95531661812450927816f;
            else
                theta = theta_i * ((float)M_PI / steps);
            phi = phi_i * ((float)M_PI / steps);
            table[select][0] = sinf(theta) * cosf(phi);
            table[select][1] = sinf(theta) * sinf(phi);
            table[select][2] = cosf(theta);
        }
        std::memcpy(ext_axis_, table, sizeof table);
    }

    // extended: at least 4 threads per cell (its fixed 4-lane reductions); the
    // offset scan covers 128 cells
    uint32_t tile_cells_max() const { return params_.algorithm == 1 ? 64u : 128u; }

    // Tile of a box of density n: the largest power of two (8 .. tile_cells_max)
    // whose expected particles, tc * n * fill, fit the buffer.  Sparse boxes of an
    // ensemble so take larger tiles than dense ones.
    uint32_t tile_for(uint32_t n, double fill, uint32_t pbuf) const
    {
        if (forced_tile_cells_) return forced_tile_cells_;
        uint32_t tc = tile_cells_max();
        while (tc > 8 && tc * n * fill > pbuf) tc >>= 1;
        return tc;
    }

    // Work decomposition only: buckets are per cell, so tiles can change between steps.
    void set_tiles(double fill, uint32_t pbuf)
    {
        uint64_t tiles = 0;
        max_tile_cells_ = 0;
        tile_info_.clear();
        for (size_t r = 0; r < boxes_.size(); ++r) {
            BoxDesc& b = boxes_[r];
            const uint32_t tc = tile_for(b.n, fill, pbuf);
            b.tile_cells = tc;
            b.tile_base = (uint32_t)tiles;
            b.tiles = (b.C + tc - 1) / tc;
            tiles += b.tiles;
            max_tile_cells_ = std::max(max_tile_cells_, tc);
            for (uint32_t t = 0; t < b.tiles; ++t)
                tile_info_.push_back({b.cell_base + t * tc, std::min(tc, b.C - t * tc) | (tc << 16), (uint32_t)r, 0u});
        }
        tiles_ = tiles;
        // runs of up to 32 cells of one box (srd_run_kernel): {first cell, cells | box << 6},
        // listed by batch class (16, 8, then 4 cells per batch; one launch per class)
        run_info_.clear();
        for (int cls = 0; cls < 3; ++cls) {
            run_class_[cls] = (uint32_t)run_info_.size();
            const uint32_t batch = 16u >> cls;
            for (size_t r = 0; r < boxes_.size(); ++r) {
                const BoxDesc& b = boxes_[r];
                if (b.run_batch != batch) continue;
                for (uint32_t c = 0; c < b.C; c += 32)
                    run_info_.push_back(make_uint2(b.cell_base + c, std::min(32u, b.C - c) | ((uint32_t)r << 6)));
            }
        }
        run_class_[3] = (uint32_t)run_info_.size();
        pbuf_ = pbuf;
        fill_ = fill;
        for (auto& g : graph_) g.reset();   // graphs bake the tiling into their launches
    }

    void retile(double fill, uint32_t pbuf)
    {
        check(cudaStreamSynchronize(stream_), "retile");
        set_tiles(fill, pbuf);
        upload_tiling();
        configure();
    }

    // Box descriptors and the tile table to the device (the stream is idle).
    void upload_tiling()
    {
        check(cudaMemcpy(boxes_d_.p, boxes_.data(), sizeof(BoxDesc) * boxes_.size(), cudaMemcpyHostToDevice),
              "upload boxes");
        const size_t bytes = sizeof(TileEntry) * tile_info_.size();
        if (tile_info_d_.bytes < bytes) check(tile_info_d_.alloc(bytes), "alloc tile table");
        check(cudaMemcpy(tile_info_d_.p, tile_info_.data(), bytes, cudaMemcpyHostToDevice), "upload tile table");
        const size_t rbytes = sizeof(uint2) * run_info_.size();
        if (run_info_d_.bytes < rbytes) check(run_info_d_.alloc(rbytes), "alloc run table");
        check(cudaMemcpy(run_info_d_.p, run_info_.data(), rbytes, cudaMemcpyHostToDevice), "upload run table");
    }

    void allocate()
    {
        check(boxes_d_.alloc(sizeof(BoxDesc) * boxes_.size()), "alloc boxes");
        upload_tiling();
        for (int k = 0; k < 2; ++k) {
            check(slots_[k].alloc(sizeof(Slot) * (total_slots_ + ext_cap_)), "alloc buckets");
            check(ov_pos_[k].alloc(sizeof(float4) * ov_cap_), "alloc overflow list");
            check(ov_vel_[k].alloc(sizeof(float4) * ov_cap_), "alloc overflow list");
            check(ov_next_[k].alloc(sizeof(uint32_t) * ov_cap_), "alloc overflow chains");
            check(ov_head_[k].alloc(sizeof(uint32_t) * cells_), "alloc overflow chains");
        }
        for (int k = 0; k < 3; ++k) {
            check(count_[k].alloc(sizeof(uint32_t) * cells_), "alloc counts");
            check(cudaMemset(count_[k].p, 0, count_[k].bytes), "clear counts");
        }
        if (walls_) check(ghosts_.alloc(sizeof(GhostSum) * walls_), "alloc wall ghosts");
        if (boxes_.size() > 1) check(box_shifts_.alloc(sizeof(float4) * 2 * boxes_.size()), "alloc box shifts");
        check(state_.alloc(sizeof(DeviceState)), "alloc state");
        check(cudaMemset(state_.p, 0, sizeof(DeviceState)), "clear state");
        check(samp_.alloc(sizeof(float4) * cells_ * 2), "alloc sample");   // two parities
        check(cudaMemset(samp_.p, 0, samp_.bytes), "clear sample");
        check(acc_.alloc(sizeof(SampleAcc) * cells_), "alloc sample sums");
        check(cudaMemset(acc_.p, 0, acc_.bytes), "clear sample sums");
        check(dense_pos_.alloc(sizeof(float) * 3 * N_ + 16), "alloc dense positions");
        check(dense_vel_.alloc(sizeof(float) * 3 * N_ + 16), "alloc dense velocities");
        check(offsets_.alloc(sizeof(uint32_t) * (cells_ + 1)), "alloc offsets");
        check(scan_status_.alloc(sizeof(unsigned long long) * scan_status_words(cells_)), "alloc scan status");
        check(scan_counter_.alloc(sizeof(unsigned int)), "alloc scan counter");
        check(partial_.alloc(sizeof(double) * 3 * kReduceBlocks * boxes_.size()), "alloc partial sums");
    }

    void configure()
    {
        int per_sm = 0;
        check(configure_step(params_.algorithm, pbuf_, max_tile_cells_, &per_sm), "configure step kernel");
        if (per_sm < 1) throw Error(MPCD_GB_ECUDA, "step kernel does not fit on an SM");
        grid_ = (int)std::min<uint64_t>(tiles_, (uint64_t)sms_ * per_sm);
    }

    void initialise()
    {
        check(launch_init(boxes_d_.as<BoxDesc>(), (int)boxes_.size(), dense_pos_.as<float>(), dense_vel_.as<float>(),
                          N_, sms_ * 16, stream_),
              "init");
        // zero net momentum in every box (the reference does not remove it)
        for (size_t r = 0; r < boxes_.size(); ++r) {
            const BoxDesc& b = boxes_[r];
            check(launch_momentum_partial(dense_vel_.as<float>(), b.dense_base, b.dense_base + b.N,
                                          partial_.as<double>() + 3 * kReduceBlocks * r, kReduceBlocks, stream_),
                  "momentum");
        }
        std::vector<double> part(3 * kReduceBlocks * boxes_.size());
        check(cudaMemcpyAsync(part.data(), partial_.p, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, stream_),
              "momentum");
        check(cudaStreamSynchronize(stream_), "momentum");
        for (size_t r = 0; r < boxes_.size(); ++r) {
            const BoxDesc& b = boxes_[r];
            double m[3] = {0, 0, 0};
            for (int i = 0; i < kReduceBlocks; ++i)
                for (int d = 0; d < 3; ++d) m[d] += part[3 * kReduceBlocks * r + 3 * i + d];
            if (b.N)
                check(launch_subtract(dense_vel_.as<float>(), b.dense_base, b.dense_base + b.N, (float)(m[0] / b.N),
                                      (float)(m[1] / b.N), (float)(m[2] / b.N), sms_ * 16, stream_),
                      "momentum");
        }
        scatter_dense();
        check(cudaStreamSynchronize(stream_), "initialise");
        check_device_errors();
    }

    // Arguments of the launch that completes step k: buckets by parity k & 1,
    // counts and overflow fill by k % 3 (the inputs of step k survive step k,
    // so that a replay can recompute its collision).
    StepArgs args(uint64_t k, bool replay = false) const
    {
        StepArgs a{};
        a.box0 = boxes_[0];
        a.boxes = boxes_d_.as<BoxDesc>();
        a.nboxes = (int)boxes_.size();
        a.boxes_tile_cells = max_tile_cells_;
        a.num_tiles = (uint32_t)tiles_;
        a.tile_info = tile_info_d_.as<TileEntry>();
        a.run_info = boxes_.size() > 1 ? run_info_d_.as<uint2>() : nullptr;
        a.num_runs = (uint32_t)run_info_.size();
        for (int c = 0; c < 4; ++c) a.run_class[c] = run_class_[c];
        a.boxes_n_max = n_max_;
        a.total_walls = walls_;
        a.ghosts = ghosts_.as<GhostSum>();
        a.box_shifts = boxes_.size() > 1 ? box_shifts_.as<float4>() : nullptr;
        a.total_slots = total_slots_;
        a.ext_cap = ext_cap_;
        a.step = k;
        const unsigned p = (unsigned)(k & 1), q = p ^ 1u;
        a.in_slots = slots_[p].as<Slot>();
        a.in_count = count_[k % 3].as<uint32_t>();
        a.out_slots = slots_[q].as<Slot>();
        a.out_count = count_[(k + 1) % 3].as<uint32_t>();
        a.zero_count = count_[(k + 2) % 3].as<uint32_t>();
        a.ov_in_pos = ov_pos_[p].as<float4>();
        a.ov_in_vel = ov_vel_[p].as<float4>();
        a.ov_out_pos = ov_pos_[q].as<float4>();
        a.ov_out_vel = ov_vel_[q].as<float4>();
        a.ov_cap = ov_cap_;
        a.ov_in_slot = (uint32_t)(k % 3);
        a.ov_out_slot = (uint32_t)((k + 1) % 3);
        a.ov_zero_slot = (uint32_t)((k + 2) % 3);
        a.ov_head_in = ov_head_[p].as<uint32_t>();
        a.ov_head_out = ov_head_[q].as<uint32_t>();
        a.ov_next_in = ov_next_[p].as<uint32_t>();
        a.ov_next_out = ov_next_[q].as<uint32_t>();
        a.state = state_.as<DeviceState>();
        a.samp = sample_buffer(k);
        a.acc = acc_.as<SampleAcc>();
        a.fold_samp = nullptr;
        std::memcpy(a.ext_axis, ext_axis_, sizeof ext_axis_);
        a.draws = tables_;
        a.replay = replay ? 1 : 0;
        a.dense_pos = dense_pos_.as<float>();
        a.dense_vel = dense_vel_.as<float>();
        a.pressure = pressure_ && !replay ? 1 : 0;
        return a;
    }

    // ------------------------------------------------------------ step graphs
    //
    // kGraphSteps consecutive steps (buffer parity repeats every 2 steps, the
    // count rotation every 3) captured once per variant (with or without
    // sampling) and replayed from any step that is a multiple of kGraphSteps:
    // every kernel of the graph reads its absolute step from state->step_base,
    // and the graph's last node advances it.
    static constexpr int kGraphSteps = 6;

    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        ~StepGraph() { reset(); }
        void reset()
        {
            if (exec) cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
    };

    unsigned long long* step_base_ptr() const
    {
        return reinterpret_cast<unsigned long long*>(static_cast<char*>(state_.p) + offsetof(DeviceState, step_base));
    }

    cudaGraphExec_t step_graph(bool sample)
    {
        StepGraph& g = graph_[sample ? 1 : 0];
        if (g.exec) return g.exec;
        cudaStream_t cs = own_stream_;
        check(cudaStreamSynchronize(cs), "graph capture");
        check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "graph capture");
        cudaError_t err = cudaSuccess;
        for (int i = 0; i < kGraphSteps && err == cudaSuccess; ++i) {
            StepArgs a = args((uint64_t)i);   // buffers of step i == those of any step = i mod 6
            a.step_base = step_base_ptr();
            a.sample = sample ? 1 : 0;
            use_run_kernel_ghosts(a, false);
            if (sample && a.run_kernel) a.fold_samp = sample_buffer((uint64_t)i + 1);   // the other parity: step i-1's
            err = select_overflow(a, (uint64_t)i, cs);
            if (err == cudaSuccess) err = launch_step(a, params_.algorithm, false, pbuf_, grid_, cs, &branches_);
            if (err == cudaSuccess && sample && !a.fold_samp)
                err = launch_sample_finalize(a.samp, acc_.as<SampleAcc>(), cells_, 0, sms_ * 8, cs);
        }
        if (err == cudaSuccess) err = launch_advance(state_.as<DeviceState>(), kGraphSteps, cs);
        cudaGraph_t graph = nullptr;
        const cudaError_t end = cudaStreamEndCapture(cs, &graph);
        if (err == cudaSuccess) err = end;
        if (err == cudaSuccess) err = cudaGraphInstantiate(&g.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (err != cudaSuccess) g.reset();
        check(err, "step graph");
        return g.exec;
    }

    // reps replays of the step graph from step step_ (a multiple of kGraphSteps);
    // returns the steps run.
    int replay_graph(bool sample, int reps)
    {
        cudaGraphExec_t g = step_graph(sample);
        graph_base_host_ = step_;
        check(cudaMemcpyAsync(step_base_ptr(), &graph_base_host_, sizeof graph_base_host_, cudaMemcpyHostToDevice,
                              stream_),
              "graph step base");
        for (int r = 0; r < reps; ++r) check(cudaGraphLaunch(g, stream_), "graph launch");
        const int done = reps * kGraphSteps;
        step_ += (uint64_t)done;
        last_step_table_ = false;
        dense_valid_ = false;
        return done;
    }

    // The reference's choice of the particles that collide in overflowing cells,
    // made on the inputs of step k before its kernel runs.
    cudaError_t select_overflow(const StepArgs& a, uint64_t k, cudaStream_t st)
    {
        const unsigned p = (unsigned)(k & 1);
        return launch_overflow_select(a, slots_[p].as<Slot>(), ov_pos_[p].as<float4>(), ov_vel_[p].as<float4>(),
                                      ov_head_[p].as<uint32_t>(),
                                      a.run_kernel && (a.total_walls || a.box_shifts) ? sms_ * 8 : sms_, st);
    }

    // The wall-ghost array of srd_run_kernel for a step that it runs (its prologue
    // draws the ghosts), else none.
    void use_run_kernel_ghosts(StepArgs& a, bool table) const
    {
        a.run_kernel = run_kernel_takes(a, params_.algorithm, table) ? 1 : 0;
    }

    // One step: the overflow selection, then the step kernel (bracketed by the
    // events `before` and `after` when given, which time the step kernel alone).
    // fold: a sampled step may fold the previous step's sample (the other parity's
    // buffer) into the FP64 sums itself; returns whether it did (run kernel only).
    bool launch_one_step(bool sample, bool fold = false, cudaEvent_t before = nullptr, cudaEvent_t after = nullptr)
    {
        StepArgs a = args(step_);
        a.sample = sample ? 1 : 0;
        use_run_kernel_ghosts(a, use_table_);
        if (sample && fold && a.run_kernel) a.fold_samp = sample_buffer(step_ + 1);
        check(select_overflow(a, step_, stream_), "overflow selection");
        if (before) check(cudaEventRecord(before, stream_), "event");
        check(launch_step(a, params_.algorithm, use_table_, pbuf_, grid_, stream_, &branches_), "step kernel");
        if (after) check(cudaEventRecord(after, stream_), "event");
        last_step_table_ = use_table_;   // a replay of this step must consume the same draws
        use_table_ = false;
        ++step_;
        dense_valid_ = false;
        return a.fold_samp != nullptr;
    }

    // The post-step state, by particle id, in dense_pos_ / dense_vel_: recompute
    // the collision of the last step from its inputs (same draws, same
    // arithmetic, bit-identical) unless the dense arrays already hold it.
    void materialise()
    {
        if (!dense_valid_) {
            if (step_ == 0) throw Error(MPCD_GB_ESTATE, "no state to read");
            StepArgs a = args(step_ - 1, true);
            check(launch_step(a, params_.algorithm, last_step_table_, pbuf_, grid_, stream_), "replay");
            check(cudaStreamSynchronize(stream_), "replay");
            check_device_errors();
            dense_valid_ = true;
        }
    }

    void alloc_tape()
    {
        const size_t K = (size_t)adj_every_;
        auto need = [&](DeviceBuffer& d, size_t bytes, const char* what) {
            if (d.bytes < bytes) check(d.alloc(bytes), what);
        };
        need(tkey_, sizeof(uint32_t) * N_ * K, "alloc tape");
        need(tlab_, sizeof(uint32_t) * N_ * K, "alloc tape");
        need(tncell_, sizeof(uint32_t) * cells_ * K, "alloc tape");
        need(tcnt_, sizeof(uint32_t) * cells_ * K, "alloc tape");
        need(tb0_, sizeof(uint32_t) * N_, "alloc tape");
        need(lam_, sizeof(float) * 3 * N_, "alloc adjoint");
        need(cellsum_, sizeof(float4) * cells_ * 2, "alloc adjoint");   // cell sums, then axes and sampling terms
        need(gsum_, sizeof(double), "alloc adjoint");
    }

    // Restore checkpoint j and recompute its steps with the tape recorded
    // (slot i of the tape = step s0 + j * every + i); returns the steps run.
    int record_segment(int j)
    {
        const int k = std::min(adj_every_, adj_steps_ - j * adj_every_);
        const size_t per = sizeof(float) * 6 * N_;
        const char* c = static_cast<const char*>(ckpt_.p) + per * j;
        check(cudaMemcpyAsync(dense_pos_.p, c, per / 2, cudaMemcpyDeviceToDevice, stream_), "restore");
        check(cudaMemcpyAsync(dense_vel_.p, c + per / 2, per / 2, cudaMemcpyDeviceToDevice, stream_), "restore");
        step_ = adj_s0_ + (uint64_t)j * adj_every_;
        scatter_dense(tb0_.as<uint32_t>());
        for (int i = 0; i < k; ++i) {
            StepArgs a = args(step_);
            a.sample = 1;
            a.tape_key = tkey_.as<uint32_t>() + (size_t)i * N_;
            a.tape_lab = tlab_.as<uint32_t>() + (size_t)i * N_;
            a.tape_ncell = tncell_.as<uint32_t>() + (size_t)i * cells_;
            use_run_kernel_ghosts(a, false);   // the run kernel records the tape of single-box SRD steps
            check(select_overflow(a, step_, stream_), "overflow selection");
            check(launch_step(a, params_.algorithm, false, pbuf_, grid_, stream_), "tape step");
            check(launch_sample_finalize(a.samp, acc_.as<SampleAcc>(), cells_, 1, sms_ * 8, stream_,
                                         tcnt_.as<uint32_t>() + (size_t)i * cells_),
                  "tape sample");
            ++step_;
        }
        last_step_table_ = false;
        dense_valid_ = false;
        return k;
    }

    // Dense post-step arrays (dense_pos_, dense_vel_) -> buckets of step step_:
    // the scatter plays the epilogue of step step_ - 1 (tape_b0: bounce bits of its streaming).
    void scatter_dense(uint32_t* tape_b0 = nullptr)
    {
        const uint64_t k = step_;
        for (uint64_t j = k; j < k + 2; ++j) {
            check(cudaMemsetAsync(count_[j % 3].p, 0, count_[j % 3].bytes, stream_), "clear counts");
            check(cudaMemsetAsync((char*)state_.p + offsetof(DeviceState, ov_count) + sizeof(unsigned int) * (j % 3),
                                  0, sizeof(unsigned int), stream_),
                  "clear overflow list");
        }
        check(cudaMemsetAsync((char*)state_.p + offsetof(DeviceState, ext_count) + sizeof(unsigned int) * (k & 1), 0,
                              sizeof(unsigned int), stream_),
              "clear extension");
        StepArgs a = args(k - 1);   // out_* = buckets, counts and overflow list of step k
        a.tape_lab = tape_b0;
        check(launch_scatter(a, dense_pos_.as<float>(), dense_vel_.as<float>(), N_, sms_ * 8, stream_),
              "scatter");
        dense_valid_ = true;
    }

    void layout(uint32_t* cell, uint32_t* slot, uint32_t* prev, uint32_t* id)
    {
        const unsigned p = parity();
        StepArgs a = args(step_);
        check(select_overflow(a, step_, stream_), "overflow selection");   // the step's own selection repeats nothing
        check(launch_layout(a, count_[step_ % 3].as<uint32_t>(), slots_[p].as<Slot>(),
                            offsets_.as<uint32_t>(), cells_, N_, scan_status_.as<unsigned long long>(),
                            scan_counter_.as<unsigned int>(), ov_pos_[p].as<float4>(), ov_vel_[p].as<float4>(),
                            (unsigned)(step_ % 3), cell, slot, prev, id, sms_ * 8, stream_),
              "layout");
        uint32_t total = 0, tail = 0;
        check(cudaMemcpyAsync(&total, offsets_.as<uint32_t>() + cells_, sizeof total, cudaMemcpyDeviceToHost, stream_),
              "layout");
        check(cudaMemcpyAsync(&tail, scan_counter_.as<unsigned int>(), sizeof tail, cudaMemcpyDeviceToHost, stream_),
              "layout");
        check(cudaStreamSynchronize(stream_), "layout");
        check_device_errors();
        layout_tail_ = tail;
        expect_count((uint64_t)total + tail);
    }

    void expect_count(uint64_t have)
    {
        if (have != N_) {
            char msg[160];
            std::snprintf(msg, sizeof msg, "particle count mismatch: %llu stored, %llu expected",
                          (unsigned long long)have, (unsigned long long)N_);
            throw Error(MPCD_GB_EDEVICE, msg);
        }
    }

    void sync_injections()
    {
        DeviceState st;
        check(cudaMemcpyAsync(&st, state_.p, sizeof st, cudaMemcpyDeviceToHost, stream_), "inject");
        check(cudaStreamSynchronize(stream_), "inject");
        for (int i = 0; i < kMaxInjectedShifts; ++i) {
            st.inject_valid[i] = inject_valid_[i];
            st.inject_step[i] = inject_step_[i];
            for (int d = 0; d < 3; ++d) st.inject_shift[i][d] = inject_shift_[i][d];
        }
        check(cudaMemcpyAsync(state_.p, &st, sizeof st, cudaMemcpyHostToDevice, stream_), "inject");
        check(cudaStreamSynchronize(stream_), "inject");
    }

    void check_device_errors()
    {
        check(cudaGetLastError(), "launch");
        unsigned int flags = 0;
        check(cudaMemcpyAsync(&flags, (char*)state_.p + offsetof(DeviceState, error_flags), sizeof flags,
                              cudaMemcpyDeviceToHost, stream_),
              "error flags");
        check(cudaStreamSynchronize(stream_), "step");
        if (flags & kErrOverflowListFull) throw Error(MPCD_GB_EDEVICE, "cell overflow list exhausted");
        if (flags & kErrWaitTimeout) throw Error(MPCD_GB_EDEVICE, "device wait timed out");
        if (flags & kErrKeyMismatch) throw Error(MPCD_GB_EDEVICE, "particle found in the wrong cell bucket");
        if (flags & kErrExtensionFull) throw Error(MPCD_GB_EDEVICE, "cell bucket extension exhausted");
    }

    static constexpr int kReduceBlocks = 1024;

    StepGraph graph_[2];                    // [sampling]
    bool graphs_ = std::getenv("MPCD_GB_GRAPHS") == nullptr || std::getenv("MPCD_GB_GRAPHS")[0] != '0';
    unsigned long long graph_base_host_ = 0;
    mpcd_gb_params params_;                 // box 0 (algorithm and device of every box)
    std::vector<mpcd_gb_params> box_params_;
    cudaStream_t own_stream_ = nullptr, stream_ = nullptr;
    RunBranches branches_;   // ensembles: side streams of the batch classes
    int sms_ = 0, grid_ = 0;
    std::vector<BoxDesc> boxes_;
    uint64_t N_ = 0, cells_ = 0, tiles_ = 0, total_slots_ = 0, walls_ = 0;
    uint32_t ov_cap_ = 0, ext_cap_ = 0, pbuf_ = 0;
    uint64_t layout_tail_ = 0;   // overflow-list particles of the last layout
    uint32_t max_tile_cells_ = 0, forced_tile_cells_ = 0;   // largest tile of any box; a tile size forced for all
    double fill_ = 1.0;                                      // expected particles per tile = pbuf / fill
    float ext_axis_[13][3];
    uint64_t step_ = 0;
    bool sampling_ = false;
    uint64_t sample_counter_ = 0;
    DeviceBuffer mean_;   // mean fields of a read (4 floats per cell)
    bool use_table_ = false;
    bool last_step_table_ = false;
    bool dense_valid_ = false;   // dense_pos_ / dense_vel_ hold the state after step step_ - 1
    DrawTables tables_{};
    int inject_valid_[kMaxInjectedShifts] = {0, 0, 0, 0};
    uint64_t inject_step_[kMaxInjectedShifts] = {0, 0, 0, 0};
    float inject_shift_[kMaxInjectedShifts][3] = {};
    std::vector<TileEntry> tile_info_;   // tile table of the current tiling
    DeviceBuffer tile_info_d_;
    std::vector<uint2> run_info_;        // run table of srd_run_kernel
    uint32_t run_class_[4] = {0, 0, 0, 0};
    DeviceBuffer run_info_d_;
    uint32_t n_max_ = 0;
    DeviceBuffer ov_head_[2], ov_next_[2];   // overflow chains: heads by cell, links by entry (by step parity)
    DeviceBuffer boxes_d_, slots_[2], ghosts_, box_shifts_, count_[3], ov_pos_[2], ov_vel_[2], state_, samp_, acc_, dense_pos_,
        dense_vel_, offsets_, scan_status_, scan_counter_, partial_;
    DeviceBuffer t_count_, t_gpos_, t_gvel_, t_axis_, t_gate_, t_gauss_;
    // adjoint: checkpoints, tape of one segment, adjoint state
    DeviceBuffer ckpt_, tkey_, tlab_, tncell_, tcnt_, tb0_, lam_, cellsum_, gsum_;
    bool adj_valid_ = false;
    bool pressure_ = false;
    uint64_t pressure_step0_ = 0;
    uint64_t adj_s0_ = 0;
    int adj_steps_ = 0, adj_every_ = 1;
};

}  // namespace mpcd_gb

// ==================================================================== C ABI

struct mpcd_gb_handle {
    mpcd_gb::Engine* engine = nullptr;
    std::string error;
};

namespace {
thread_local std::string g_create_error;

template <class F>
int32_t guarded(mpcd_gb_handle* h, F&& f)
{
    if (!h || !h->engine) return MPCD_GB_EINVAL;
    try {
        h->error.clear();
        f(*h->engine);
        return MPCD_GB_OK;
    } catch (const mpcd_gb::Error& e) {
        h->error = e.what();
        return e.code();
    } catch (const std::bad_alloc&) {
        h->error = "host allocation failed";
        return MPCD_GB_ENOMEM;
    } catch (const std::exception& e) {
        h->error = e.what();
        return MPCD_GB_EINVAL;
    }
}
}  // namespace

extern "C" {

int32_t mpcd_gb_abi_version(void) { return MPCD_GB_ABI_VERSION; }

int32_t mpcd_gb_create(const mpcd_gb_params* params, mpcd_gb_handle** out)
{
    return mpcd_gb_ensemble_create(params, 1, out);
}

int32_t mpcd_gb_ensemble_create(const mpcd_gb_params* params, int32_t R, mpcd_gb_handle** out)
{
    g_create_error.clear();
    if (!params || !out || R < 1) {
        g_create_error = R < 1 ? "an ensemble needs at least one box" : "null argument";
        if (out) *out = nullptr;
        return MPCD_GB_EINVAL;
    }
    *out = nullptr;
    auto* h = new (std::nothrow) mpcd_gb_handle;
    if (!h) return MPCD_GB_ENOMEM;
    try {
        h->engine = new mpcd_gb::Engine(params, R);
    } catch (const mpcd_gb::Error& e) {
        g_create_error = e.what();
        delete h;
        return e.code();
    } catch (const std::exception& e) {
        g_create_error = e.what();
        delete h;
        return MPCD_GB_ENOMEM;
    }
    *out = h;
    return MPCD_GB_OK;
}

void mpcd_gb_destroy(mpcd_gb_handle* h)
{
    if (!h) return;
    delete h->engine;
    delete h;
}

const char* mpcd_gb_last_error(const mpcd_gb_handle* h)
{
    return h ? h->error.c_str() : g_create_error.c_str();
}

int32_t mpcd_gb_step(mpcd_gb_handle* h, int32_t n)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.step(n, false); });
}

int32_t mpcd_gb_step_and_sample(mpcd_gb_handle* h, int32_t n)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.step(n, true); });
}

int32_t mpcd_gb_get_sample_mean(mpcd_gb_handle* h, float* density, float* velocity)
{
    if (!density || !velocity) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.sample_mean(density, velocity); });
}

size_t mpcd_gb_num_particles(const mpcd_gb_handle* h) { return h && h->engine ? h->engine->num_particles() : 0; }

size_t mpcd_gb_num_cells(const mpcd_gb_handle* h) { return h && h->engine ? h->engine->num_cells() : 0; }

int32_t mpcd_gb_get_positions(mpcd_gb_handle* h, float* out)
{
    if (!out) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.get(out, nullptr); });
}

int32_t mpcd_gb_get_velocities(mpcd_gb_handle* h, float* out)
{
    if (!out) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.get(nullptr, out); });
}

int32_t mpcd_gb_set_positions(mpcd_gb_handle* h, const float* in)
{
    if (!in) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.set(in, nullptr); });
}

int32_t mpcd_gb_set_velocities(mpcd_gb_handle* h, const float* in)
{
    if (!in) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.set(nullptr, in); });
}

int32_t mpcd_gb_set_particles(mpcd_gb_handle* h, const float* positions, const float* velocities)
{
    if (!positions || !velocities) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.set(positions, velocities); });
}

int32_t mpcd_gb_set_stream(mpcd_gb_handle* h, void* stream)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.set_stream(stream); });
}

int32_t mpcd_gb_synchronize(mpcd_gb_handle* h)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.synchronize(); });
}

int32_t mpcd_gb_time_steps(mpcd_gb_handle* h, int32_t n_steps, float* total_ms, float* kernel_ms)
{
    if (n_steps < 0) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.time_steps(n_steps, total_ms, kernel_ms); });
}

uint64_t mpcd_gb_step_index(const mpcd_gb_handle* h) { return h && h->engine ? h->engine->step_index() : 0; }

int32_t mpcd_gb_inject_shift(mpcd_gb_handle* h, uint64_t step, const float shift[3])
{
    if (!shift) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.inject_shift(step, shift); });
}

int32_t mpcd_gb_get_shift(mpcd_gb_handle* h, uint64_t step, float shift[3])
{
    if (!shift) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.get_shift(step, shift); });
}

int32_t mpcd_gb_dump_layout(mpcd_gb_handle* h, uint32_t* cell, uint32_t* slot, uint32_t* id, uint32_t* counts)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.dump(cell, slot, id, counts); });
}

int32_t mpcd_gb_inject_draws(mpcd_gb_handle* h, uint32_t gmax, uint32_t pmax, const uint32_t* ghost_count,
                             const float* ghost_pos, const float* ghost_vel, const float* axis, const float* gate_u,
                             const float* gauss)
{
    return guarded(h, [&](mpcd_gb::Engine& e) {
        e.inject_draws(gmax, pmax, ghost_count, ghost_pos, ghost_vel, axis, gate_u, gauss);
    });
}

int32_t mpcd_gb_counters(mpcd_gb_handle* h, uint64_t out[2])
{
    if (!out) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.counters(out); });
}

int32_t mpcd_gb_set_particles_device(mpcd_gb_handle* h, const float* d_positions, const float* d_velocities)
{
    if (!d_positions && !d_velocities) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.set_device(d_positions, d_velocities); });
}

int32_t mpcd_gb_get_particles_device(mpcd_gb_handle* h, float* d_positions, float* d_velocities)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.get_device(d_positions, d_velocities); });
}

int32_t mpcd_gb_set_step(mpcd_gb_handle* h, uint64_t step)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.set_step(step); });
}

int32_t mpcd_gb_wall_pressure(mpcd_gb_handle* h, int32_t restart, double out[3])
{
    if (!out) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.wall_pressure(restart != 0, out); });
}

int32_t mpcd_gb_save_snapshot(mpcd_gb_handle* h, const char* path)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.save_snapshot(path); });
}

int32_t mpcd_gb_load_snapshot(mpcd_gb_handle* h, const char* path)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.load_snapshot(path); });
}

int32_t mpcd_gb_set_drag(mpcd_gb_handle* h, float drag)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.set_drag(drag); });
}

int32_t mpcd_gb_profile_forward(mpcd_gb_handle* h, int32_t steps, int32_t checkpoint_every, float* d_profile)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.profile_forward(steps, checkpoint_every, d_profile); });
}

int32_t mpcd_gb_profile_backward(mpcd_gb_handle* h, const float* d_grad_profile, float* d_grad_velocities,
                                 double* grad_drag)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.profile_backward(d_grad_profile, d_grad_velocities, grad_drag); });
}

int32_t mpcd_gb_profile_tape(mpcd_gb_handle* h, uint32_t* key, uint32_t* lab, uint32_t* ncell, uint32_t* lab_count,
                             uint32_t* bounce0)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.profile_tape(key, lab, ncell, lab_count, bounce0); });
}

int32_t mpcd_gb_num_boxes(const mpcd_gb_handle* h) { return h && h->engine ? h->engine->num_boxes() : 0; }

int32_t mpcd_gb_box_range(mpcd_gb_handle* h, int32_t r, uint64_t out[4])
{
    if (!out) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.box_range(r, out); });
}

int32_t mpcd_gb_autotune(mpcd_gb_handle* h, int32_t steps_per_candidate, uint32_t out[2])
{
    if (!out) return MPCD_GB_EINVAL;
    return guarded(h, [&](mpcd_gb::Engine& e) { e.autotune(steps_per_candidate, out); });
}

uint64_t mpcd_gb_device_allocations(void) { return mpcd_gb::g_device_allocations.load(); }

int32_t mpcd_gb_cell_offsets_noalloc(mpcd_gb_handle* h, uint32_t* d_offsets, uint64_t n_offsets)
{
    return guarded(h, [&](mpcd_gb::Engine& e) { e.cell_offsets_noalloc(d_offsets, n_offsets); });
}

}  // extern "C"
