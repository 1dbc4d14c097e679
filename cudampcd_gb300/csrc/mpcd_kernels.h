// Launchers of the GB300 MPCD kernels (host side).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "mpcd_types.h"

namespace mpcd_gb {

// Dynamic shared memory of the step kernel: a particle buffer of `pbuf`
// entries and tiles of `cells` cells.
size_t step_smem_bytes(uint32_t pbuf, uint32_t cells, int algorithm);
// Opt the step kernels into that much shared memory and report resident CTAs per SM.
cudaError_t configure_step(int algorithm, uint32_t pbuf, uint32_t cells, int* blocks_per_sm);
// Side streams on which an ensemble's second and third batch classes run beside the
// first: the step's stream forks to them and joins them again, so that each class's
// launch fills the tail of the one before it.  Null streams: one after another.
struct RunBranches {
    cudaStream_t side[2] = {nullptr, nullptr};
    cudaEvent_t fork = nullptr;
    cudaEvent_t join[2] = {nullptr, nullptr};
};
// One step of every box (algorithm 0 = SRD, 1 = extended; table = injected draws).
cudaError_t launch_step(const StepArgs& a, int algorithm, bool table, uint32_t pbuf, int grid, cudaStream_t st,
                        const RunBranches* branches = nullptr);
// Whether srd_run_kernel can run this step (SRD, Philox draws, no replay or
// pressure estimator, the adjoint tape only for one sampled box, n <= 64 in every
// box, a run table for ensembles and the wall-ghost array when boxes have walls);
// the caller then sets a.run_kernel, which launch_step and the step's prologue follow.
bool run_kernel_takes(const StepArgs& a, int algorithm, bool table);
// state->step_base += steps (the last node of a replayed step graph).
cudaError_t launch_advance(DeviceState* state, unsigned steps, cudaStream_t st);
// Key dense clean particles for step a.step + 1 and scatter them into a.out_*.
cudaError_t launch_scatter(const StepArgs& a, const float* pos, const float* vel, uint64_t n_total, int grid,
                           cudaStream_t st);
// Before a step (not a replay): the particles the reference keeps in each cell past
// its bucket depth into the extension area after the buckets, the others left in
// the overflow list (in_* / ov_*: the step's input buckets and list, a.in_count,
// ov_head and a.ov_next_in its chains).  A second call for the same step does nothing.
cudaError_t launch_overflow_select(const StepArgs& a, Slot* in_slots, float4* ov_pos, float4* ov_vel,
                                   uint32_t* ov_head, int grid, cudaStream_t st);
// Lab-grid sample of one step into the FP64 running sums (and clear the step sums).
cudaError_t launch_sample_finalize(float4* samp, SampleAcc* acc, uint64_t cells, int snapshot, int grid,
                                   cudaStream_t st, uint32_t* lab_count = nullptr);
// Density and velocity means of one box in reference order (x fastest) from the
// FP64 sums (storage order), divided by the sample count: inverse = 1 / samples.
cudaError_t launch_mean_fields(const SampleAcc* acc, const BoxDesc& b, double inverse, float* density, float* velocity,
                               cudaStream_t st);
// Adjoint of the sampled x-velocity profile (single box, SRD): U(z) from the sample
// sums of `samples` steps; one reverse step (both passes) at absolute step `step`;
// dL/dV0 from the final adjoint and the bounce bits of the initial streaming.
cudaError_t launch_profile(const SampleAcc* acc, const BoxDesc& b, uint64_t samples, float* profile, cudaStream_t st);
// cellsum: 2 C entries (the cell sums of mu, then each cell's axis and sampling term).
cudaError_t launch_adjoint_step(const BoxDesc& b, uint64_t step, uint64_t samples, float* lam, const uint32_t* key,
                                const uint32_t* lab, const uint32_t* ncell, const uint32_t* lab_count,
                                const float* dU, float4* cellsum, double* gsum, int grid, cudaStream_t st);
cudaError_t launch_adjoint_finish(uint32_t n, const float* lam, const uint32_t* b0, float* out, int grid,
                                  cudaStream_t st);
// Layout dump, after the step's overflow selection: cells in storage order, stable
// order within a cell (decoupled look-back scan of the counts, then one thread per
// cell), then the overflow list's particles that do not collide, in any order;
// their number lands in *tile_counter.  offsets: cells + 1 entries.
cudaError_t launch_layout(const StepArgs& a, const uint32_t* count, const Slot* slots,
                          uint32_t* offsets, uint64_t cells, uint64_t n_total, unsigned long long* status,
                          unsigned int* tile_counter, const float4* ov_pos, const float4* ov_vel, unsigned parity,
                          uint32_t* out_cell, uint32_t* out_slot, uint32_t* out_prev, uint32_t* out_id, int grid,
                          cudaStream_t st);
size_t scan_status_words(uint64_t cells);
// Exclusive scan of min(count, cap) into offsets (cells + 1 entries), its scratch
// in a static per-device array: allocates nothing.  cells <= MPCD_GB_NOALLOC_MAX_CELLS.
cudaError_t launch_cell_offsets_static(const StepArgs& a, const uint32_t* count, uint64_t cells, uint32_t* offsets,
                                       int device, cudaStream_t st);
// Initial particles (uniform positions, Maxwell-Boltzmann velocities).
cudaError_t launch_init(const BoxDesc* boxes, int nboxes, float* pos, float* vel, uint64_t n_total, int grid,
                        cudaStream_t st);
cudaError_t launch_momentum_partial(const float* vel, uint64_t begin, uint64_t end, double* partial, int grid,
                                    cudaStream_t st);
cudaError_t launch_subtract(float* vel, uint64_t begin, uint64_t end, float mx, float my, float mz, int grid,
                            cudaStream_t st);

}  // namespace mpcd_gb
