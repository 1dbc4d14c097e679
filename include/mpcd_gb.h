/*
 * mpcd_gb.h -- C ABI of the GB300 MPCD time step (libmpcd_gb.so).
 *
 * This is the drop-in boundary for the MPCD step of azantop/cudaMPCD.  The
 * reference reaches its CUDA path through the abstract C++ class
 * mpcd::Backend (src/libmpcd/common/backend.hpp:11-31), created by
 * mpcd::create_backend(params, "cuda") (src/libmpcd/common/backend_factory.hpp:15-27)
 * for mpcd::api::SimulationHandle (src/libmpcd/api/simulator_handle.cpp:9).
 * Every Backend member maps onto one function below; a Backend subclass that
 * forwards to them is all the reference tree needs.
 *
 * Conventions
 *   - plain pointers and sizes; host buffers unless a name says "device";
 *   - every function returns 0 on success and a negative MPCD_GB_E* code on
 *     failure; mpcd_gb_last_error() then describes the failure (the reference
 *     throws std::runtime_error, src/libmpcd/cuda_backend/gpu_error_check.hpp:10-39);
 *   - a handle owns one CUDA stream and all device memory of one simulation;
 *     calls on one handle must not overlap (the reference is single-threaded);
 *   - positions and velocities are (N, 3) float32, xyz interleaved, indexed
 *     by particle id: the order fixed when the handle is created, unchanged by
 *     steps (the reference returns its internal array order, which its CUDA
 *     backend permutes every 100 steps, cuda_backend_impl.cu:127-128).
 */
#ifndef MPCD_GB_H
#define MPCD_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MPCD_GB_ABI_VERSION 1

enum {
    MPCD_GB_OK = 0,
    MPCD_GB_EINVAL = -1,    /* bad argument or parameter */
    MPCD_GB_ECUDA = -2,     /* CUDA runtime error */
    MPCD_GB_ENOMEM = -3,    /* device allocation failed */
    MPCD_GB_EDEVICE = -4,   /* device-side check failed (overflow list full, wait timeout, ...) */
    MPCD_GB_ESTATE = -5     /* call not valid in the current state */
};

/* Mirrors mpcd::SimulationParameters (include/mpcd/api/simulation_parameters.hpp:70-102)
 * for the fields the step reads, plus a Philox seed (the reference seeds from
 * /dev/urandom and has no seed field). */
typedef struct mpcd_gb_params {
    int32_t experiment;        /* 0 standard, 1 channel (ExperimentType) */
    int32_t algorithm;         /* 0 srd, 1 extended (MPCDAlgorithm) */
    int32_t collision_kernel;  /* accepted for compatibility (CollisionKernel); one fused kernel serves all */
    int32_t periodicity[3];
    float volume_size[3];      /* container size incl. wall layers, integral */
    uint32_t N;                /* ignored: N = n * fluid volume (see mpcd_gb_num_particles) */
    uint32_t n;                /* particles per cell */
    uint32_t device_id;
    float delta_t;
    float temperature;
    float thermal_velocity;
    float drag;
    uint64_t seed;             /* Philox key */
} mpcd_gb_params;

typedef struct mpcd_gb_handle mpcd_gb_handle;

/* ABI version of the loaded library (== MPCD_GB_ABI_VERSION). */
int32_t mpcd_gb_abi_version(void);

/* Replaces CudaBackend::CudaBackend (src/libmpcd/cuda_backend/cuda_backend.cu:7) /
 * BackendContext::BackendContext (src/libmpcd/cuda_backend/backend_context.cu:17-127):
 * allocate, distribute particles uniformly in the fluid volume with
 * Maxwell-Boltzmann velocities (net momentum removed). */
int32_t mpcd_gb_create(const mpcd_gb_params *params, mpcd_gb_handle **out);

/* Replaces CudaBackend::~CudaBackend (src/libmpcd/cuda_backend/cuda_backend_impl.cu:20-22). */
void mpcd_gb_destroy(mpcd_gb_handle *h);

/* Failure description of the last call on h (h may be NULL for mpcd_gb_create failures). */
const char *mpcd_gb_last_error(const mpcd_gb_handle *h);

/* Replaces Backend::step (backend.hpp:15; cuda_backend_impl.cu:111-131). */
int32_t mpcd_gb_step(mpcd_gb_handle *h, int32_t n_steps);

/* Replaces Backend::stepAndAccumulateSample (backend.hpp:17; cuda_backend_impl.cu:182-204). */
int32_t mpcd_gb_step_and_sample(mpcd_gb_handle *h, int32_t n_steps);

/* Replaces Backend::getSampleMean (backend.hpp:18; cuda_backend_impl.cu:206-218).
 * density: C floats, velocity: 3C floats (xyz interleaved), cell order x + Lx*(y + Ly*z).
 * Divides by the sample counter, S-1 for S sampled steps, as the reference does. */
int32_t mpcd_gb_get_sample_mean(mpcd_gb_handle *h, float *density, float *velocity);

/* Replaces Backend::getNParticles (backend.hpp:20). */
size_t mpcd_gb_num_particles(const mpcd_gb_handle *h);

/* Number of cells C = Lx*Ly*Lz (container). */
size_t mpcd_gb_num_cells(const mpcd_gb_handle *h);

/* Replace Backend::getParticlePositions / getParticleVelocities (backend.hpp:21-22). out: 3N floats. */
int32_t mpcd_gb_get_positions(mpcd_gb_handle *h, float *out);
int32_t mpcd_gb_get_velocities(mpcd_gb_handle *h, float *out);

/* Replace Backend::setParticlePositions / setParticleVelocities / setParticles (backend.hpp:23-25).
 * in: 3N floats indexed by particle id.  (The reference's CUDA setters index
 * the particle array with the float index, cuda_backend_impl.cu:157-180.) */
int32_t mpcd_gb_set_positions(mpcd_gb_handle *h, const float *in);
int32_t mpcd_gb_set_velocities(mpcd_gb_handle *h, const float *in);
int32_t mpcd_gb_set_particles(mpcd_gb_handle *h, const float *positions, const float *velocities);

/* ---- stream and timing (used by bench.py; no reference counterpart) ---- */

/* Run the handle's work on an existing stream (cudaStream_t passed as void*); NULL = own stream. */
int32_t mpcd_gb_set_stream(mpcd_gb_handle *h, void *stream);
/* Block until the handle's stream is idle. */
int32_t mpcd_gb_synchronize(mpcd_gb_handle *h);
/* Run n_steps steps between two CUDA events recorded on the handle's stream; returns
 * the elapsed device time and the elapsed time of the step kernel launches alone. */
int32_t mpcd_gb_time_steps(mpcd_gb_handle *h, int32_t n_steps, float *total_ms, float *kernel_ms);

/* ---- test hooks (no reference counterpart; used by the parity tests) ---- */

/* Current step index (the Philox step counter). */
uint64_t mpcd_gb_step_index(const mpcd_gb_handle *h);

/* Use `shift` as the grid shift of step `step` instead of the Philox draw
 * (the reference draws it on the host, cuda_backend_impl.cu:85-87).  Up to 4 pending. */
int32_t mpcd_gb_inject_shift(mpcd_gb_handle *h, uint64_t step, const float shift[3]);

/* The grid shift the handle uses for `step`. */
int32_t mpcd_gb_get_shift(mpcd_gb_handle *h, uint64_t step, float shift[3]);

/* Layout of the current cell buckets -- the counting sort by cell -- one entry
 * per particle in layout order: cells in storage order (z fastest, then x, then
 * y), within a cell its colliding particles (up to 4n) by ascending particle id
 * (the stable sort of the id-ordered particle array by cell), then the particles
 * past a cell's 4n, which skip the collision, ordered by (cell, id).  cell =
 * reference cell index x + Lx*(y + Ly*z) the particle is keyed to, id = particle
 * id, slot = where the handle stores it: a bucket slot, an extension slot
 * (bucket slots + offset) or an overflow-list entry (bucket and extension slots +
 * entry); within a cell, slots are numbered in id order.  counts: C entries
 * (reference cell order), the number of particles each cell received, overflow
 * included (the reference's uniform_counter).  Runs the next step's overflow
 * selection (which that step then finds done).  Any pointer may be NULL. */
int32_t mpcd_gb_dump_layout(mpcd_gb_handle *h, uint32_t *cell, uint32_t *slot, uint32_t *id, uint32_t *counts);

/* Injected draws for the next step (the oracle's recorded tables, reference
 * cell order): ghost_count[C], ghost_pos[C*gmax*3], ghost_vel[C*gmax*3],
 * axis[C*3], gate_u[C], gauss[C*pmax].  The next mpcd_gb_step consumes them;
 * pass NULL tables to return to Philox draws. */
int32_t mpcd_gb_inject_draws(mpcd_gb_handle *h, uint32_t gmax, uint32_t pmax, const uint32_t *ghost_count,
                             const float *ghost_pos, const float *ghost_vel, const float *axis,
                             const float *gate_u, const float *gauss);

/* Device-side counters: [0] particles that found their cell's bucket full (all time;
 * buckets are min(4n, n + ceil(4 sqrt(n)) + 2) deep, so this counts more than the
 * reference's overflow past 4n),
 * [1] error flags (bit 0 overflow list full, bit 1 wait timeout, bit 2 key mismatch,
 * bit 3 bucket extension full). */
int32_t mpcd_gb_counters(mpcd_gb_handle *h, uint64_t out[2]);

/* ---- snapshots: checkpoint and resume (the reference's writeBackupFile is a TODO,
 *      src/libmpcd/cuda_backend/cuda_backend_impl.cu:77-79) ---- */

/* Write the handle's state to `path`.  The file holds the step index, every box's
 * parameters and Philox seed, and the post-step positions and velocities by particle id,
 * with a checksum.  The layout is in mpcd_engine.cu.  Sample sums are not saved. */
int32_t mpcd_gb_save_snapshot(mpcd_gb_handle *h, const char *path);
/* Load a snapshot into a handle created with the same boxes (geometry, n, dt, T,
 * drag, seed, algorithm; MPCD_GB_EINVAL otherwise).  Stepping on continues the
 * saved trajectory bit for bit. */
int32_t mpcd_gb_load_snapshot(mpcd_gb_handle *h, const char *path);

/* ---- batched ensemble (no counterpart in the reference) ---- */

/* R independent boxes advanced together: one step-kernel launch per step walks a
 * table of boxes (per-box geometry, n, drag, temperature, time step and Philox seed;
 * every box must use the same algorithm and device).  Box r evolves exactly as a
 * single-box handle created from params[r] does.  On an ensemble handle:
 * mpcd_gb_num_particles / mpcd_gb_num_cells are totals; the getters, setters and
 * mpcd_gb_get_sample_mean concatenate the boxes in order (particles of box r at
 * [first_particle, +num_particles), cells of box r at [first_cell, +num_cells) in
 * that box's own x + Lx*(y + Ly*z) order); mpcd_gb_inject_shift applies to box 0 and
 * mpcd_gb_inject_draws needs R = 1.  mpcd_gb_create(p, h) is the R = 1 case. */
int32_t mpcd_gb_ensemble_create(const mpcd_gb_params *params, int32_t R, mpcd_gb_handle **out);
/* Number of boxes of the handle. */
int32_t mpcd_gb_num_boxes(const mpcd_gb_handle *h);
/* out = {first_particle, num_particles, first_cell, num_cells} of box r. */
int32_t mpcd_gb_box_range(mpcd_gb_handle *h, int32_t r, uint64_t out[4]);
/* Choose the particle buffer of the step kernel and the tiles of every box (per box
 * the largest power of two, 8..128 cells, whose expected particles times a fill
 * factor fit the buffer) by timing steps_per_candidate real steps of every
 * admissible (buffer, fill factor) pair; the steps advance the simulation.
 * out = {largest tile of any box (cells), buffer (particles)}. */
int32_t mpcd_gb_autotune(mpcd_gb_handle *h, int32_t steps_per_candidate, uint32_t out[2]);

/* ---- device-pointer I/O and the differentiable channel (no counterpart in the reference) ---- */

/* As mpcd_gb_set_particles / the getters, with device buffers of 3N floats (either may be
 * NULL to keep or skip that array). */
int32_t mpcd_gb_set_particles_device(mpcd_gb_handle *h, const float *d_positions, const float *d_velocities);
int32_t mpcd_gb_get_particles_device(mpcd_gb_handle *h, float *d_positions, float *d_velocities);

/* Continue from the current particle state with the step counter -- the key of every
 * Philox draw -- set to `step` (< 2^40).  Two runs that start from the same state at the
 * same step draw the same random numbers (common random numbers). */
int32_t mpcd_gb_set_step(mpcd_gb_handle *h, uint64_t step);

/* Wall pressure estimator (the reference has none).  It measures the momentum per unit
 * area and time that the fluid gives each z wall, along the wall's outward normal:
 *   - 2|v_z| for every bounce-back;
 *   - the z momentum that the wall's ghost particles take up in the collisions of the
 *     wall-layer cells (minus the real particles' change).
 * In equilibrium this is the fluid's pressure; for SRD, an ideal gas, it is n T.
 * restart != 0 zeroes the sums and measures from the next step on.  Every call returns
 * out = {bottom wall, top wall, steps measured}.  Single box with walls in z. */
int32_t mpcd_gb_wall_pressure(mpcd_gb_handle *h, int32_t restart, double out[3]);

/* Body force (SimulationParameters::drag) of every box from the next step on. */
int32_t mpcd_gb_set_drag(mpcd_gb_handle *h, float drag);

/* Sampled x-velocity profile of a single-box SRD handle, and its adjoint.
 * Forward: from the current state, run `steps` steps sampling each one, checkpoint the
 * particle state every `checkpoint_every` steps, and write
 *   U[z] = (1 / (steps Lx Ly)) sum_t sum_{x,y} mean v_x of lab cell (x, y, z) at step t
 * (d_profile: device float[Lz], Lz of the container).  The sample sums of the handle
 * are overwritten.
 * Backward: given d_grad_profile = dL/dU (device float[Lz]), write dL/dV0 (device
 * float[3N], V0 = the velocities at the start of the forward, by particle id) and
 * dL/d(drag) (host double).  Collision cells, grid shifts, rotation axes, ghost counts
 * and wall bounces are held fixed at those of the forward trajectory: each checkpoint
 * segment is recomputed (its draws replayed from the Philox counters) and then swept
 * in reverse.  Afterwards the handle's particle state is that of an intermediate step;
 * set the particles again before stepping on. */
int32_t mpcd_gb_profile_forward(mpcd_gb_handle *h, int32_t steps, int32_t checkpoint_every, float *d_profile);
int32_t mpcd_gb_profile_backward(mpcd_gb_handle *h, const float *d_grad_profile, float *d_grad_velocities,
                                 double *grad_drag);
/* Test hook: the fixed events of every step of the last profile forward, host arrays:
 * key[steps*N] (collision cell, storage order, or 0xFFFFFFFF if not collided),
 * lab[steps*N] (lab cell, storage order, | 0x80000000 if the streaming after that
 * step bounced the particle), ncell[steps*C] (particles + ghosts of each collided cell,
 * storage order), lab_count[steps*C] (storage order), bounce0[N] (0x80000000 if the streaming into the
 * first step bounced the particle).  Any pointer may be NULL. */
int32_t mpcd_gb_profile_tape(mpcd_gb_handle *h, uint32_t *key, uint32_t *lab, uint32_t *ncell, uint32_t *lab_count,
                             uint32_t *bounce0);

/* Device allocations (cudaMalloc calls, successful or not) the library has made in
 * this process, all handles together: every device buffer of the library goes through
 * one allocator that counts them.  No counterpart in the reference; a diagnostic for
 * callers that must know that a call allocates nothing. */
uint64_t mpcd_gb_device_allocations(void);

/* ---- allocation-free cell offsets (no counterpart in the reference) ---- */

/* Largest cell count (C) that mpcd_gb_cell_offsets_noalloc accepts. */
#define MPCD_GB_NOALLOC_MAX_CELLS 33554432u

/* Where each cell's particles begin in the current layout, written to device memory
 * without allocating anything on the device.
 *
 * d_offsets: device buffer of n_offsets >= C + 1 uint32 entries.  d_offsets[s] is the
 * number of bucketed particles in the cells before cell s, cells in storage order
 * (z fastest, then x, then y), i.e. the index at which cell s's run starts in the
 * mpcd_gb_dump_layout order; d_offsets[C] is the number of bucketed particles
 * (particles in the cell overflow list, if any, are not counted).
 *
 * Who needs it: a caller that cannot allocate device memory while it runs.  A coupled
 * code (a solute or MD solver stepping with the fluid) that has handed all free HBM to
 * its own memory pool, or a per-step loop that must not stall on cudaFree (which
 * synchronises the whole device), can still read the cell layout every step.
 * mpcd_gb_dump_layout allocates device buffers per call and cannot serve them.
 *
 * Scratch: the prefix scan's look-back status words and its tile counter live in one
 * fixed 128 KiB array in the library's device memory, one per device.  No device memory
 * is allocated or freed; on success no host memory either (an error message may).
 * Limit: C <= MPCD_GB_NOALLOC_MAX_CELLS (16384 scan tiles of 2048 cells).  A larger C,
 * a NULL d_offsets or n_offsets < C + 1 returns MPCD_GB_EINVAL before any work.
 * What must start at zero: the status words of the tiles in use and the tile counter.
 * Every call zeroes them on the handle's stream before its scan, so nothing needs to be
 * cleared by the caller.
 *
 * Set-up: the first call on a device, with that device made current for the look-up,
 * finds the scratch address with cudaGetSymbolAddress, which may load the library's
 * device code.  If the calling stream is going to be captured, make that first call
 * before the capture begins.
 *
 * Concurrency: the work is queued on the handle's stream (mpcd_gb_set_stream) and the
 * call returns without waiting; order reads of d_offsets after that stream.  All calls
 * on one device share the one scratch array, so two calls that overlap in time race and
 * both results are undefined: calls queued on one stream are ordered and safe, calls on
 * different streams, handles or host threads of one device must be serialised by the
 * caller.  A look-back wait that times out sets error bit 1 (mpcd_gb_counters), which
 * the next mpcd_gb_step, mpcd_gb_step_and_sample or setter reports as MPCD_GB_EDEVICE,
 * and makes the call write 0xFFFFFFFF to d_offsets[C] in place of the particle count:
 * a caller that reads the offsets every step can tell a bad result from the buffer
 * alone.  The scratch address found at set-up is kept for the life of the process:
 * after cudaDeviceReset on that device (which frees the library's device memory) the
 * entry point must not be called again. */
int32_t mpcd_gb_cell_offsets_noalloc(mpcd_gb_handle *h, uint32_t *d_offsets, uint64_t n_offsets);

#ifdef __cplusplus
}
#endif
#endif
