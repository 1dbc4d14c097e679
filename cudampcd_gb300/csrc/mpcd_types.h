// Host/device data structures of the GB300 MPCD step.
//
// Particles live in per-cell buckets: cell c of a box owns `depth` slots of 32
// bytes each, one DRAM sector: pos = (x, y, z, 0), vel = (vx, vy, vz, id).  The
// reference's cell table is 4n deep (cap, backend_context.cu:24): up to cap
// particles of a cell collide.  depth = min(cap, n + ceil(4 sqrt(n)) + 2) holds
// all but about one cell in 10^4..10^5 at equilibrium; the particles of a cell
// past its depth go to the overflow list, and the step's prologue
// (overflow_select_kernel) copies such a cell's colliding set -- its cap lowest
// ids -- into a contiguous extension area after the buckets, records the
// extension offset in pos.w of the cell's first bucket slot, and marks the list
// entries it took as taken (id kTakenId).
// A bucket set for step k holds every particle as it enters the collision of
// step k: streamed and shifted by the grid shift of step k, in the bucket of the
// cell it then occupies (the reference's translate output, simulation_functions.cpp:38-103).
// Cells are numbered in storage order, z fastest, then x, then y, so that the
// up to 27 source cells of any destination cell are processed within a short
// window of the sweep.  Two bucket sets alternate by step parity; the cell
// counts rotate over three arrays so that the inputs of the last step survive
// it (the getters replay that step's collision from them).
#pragma once

#include <cstdint>
#include <vector_types.h>

namespace mpcd_gb {

// One bucket slot: a particle's position and velocity with its id in vel.w (the
// bit pattern of a float), 32 bytes, so that a particle is one full sector in
// DRAM and one 256-bit access.
struct alignas(32) Slot {
    float4 pos;
    float4 vel;
};

constexpr int kThreads = 256;        // threads per CTA of the step kernel
constexpr int kMaxInjectedShifts = 4;

// One simulation box (a "replica" in a batched ensemble).
struct BoxDesc {
    int32_t L[3];          // container size incl. wall layers
    float Lf[3];
    float L15[3], L2x[3], L3x[3], Lh[3];   // 1.5 L, 2 L, 3 L, L / 2 (float products, as the reference forms them)
    int32_t periodic[3];
    int32_t wall_z;        // periodicity.z == 0: bounce-back walls and ghost layers in z
    int32_t channel;       // ExperimentType::channel
    float dt;
    float drag_dt;         // drag * dt, added to v.x after a collision
    float tv;              // thermal velocity sqrt(T)
    float R2;              // channel radius^2, (Lz - 2)^2 / 4
    float cos_a, sin_a;    // SRD rotation by 120 degrees (host libm, as the reference)
    uint32_t n;            // particles per cell
    uint32_t cap;          // colliding particles per cell at most, 4n
    uint32_t C;            // cells
    uint32_t N;            // particles
    uint32_t cell_base;    // first global cell of this box
    uint32_t tile_base;    // first tile of this box
    uint32_t tiles;        // tiles of this box
    uint32_t tile_cells;   // cells per tile
    uint64_t slot_base;    // first global slot of this box
    uint64_t dense_base;   // first particle of this box in dense (getter) arrays
    uint64_t div_z, div_x; // ceil(2^48 / Lz), ceil(2^48 / Lx): exact division of cell indices < 2^31
    uint32_t seed_lo, seed_hi;
    uint64_t wall_base;    // first wall-ghost entry of this box (2 per column, with walls in z)
    uint32_t run_batch;    // srd_run_kernel: cells summed and finished together (4, 8 or 16)
    uint32_t depth;        // bucket slots per cell (<= cap)
};

// The step kernel copies a box descriptor into shared memory 16 bytes per thread.
static_assert(sizeof(BoxDesc) % 16 == 0, "BoxDesc must be a whole number of 16-byte words");

// One tile of an ensemble launch (host-built table, read as one 16-byte load).
struct alignas(16) TileEntry {
    uint32_t first;   // first global cell (storage order)
    uint32_t cells;   // cells of this tile | cells per tile of its box << 16
    uint32_t box;
    uint32_t unused;
};

// The wall ghosts of one wall cell for one step (srd_run_kernel): their count
// and the exact sum of their velocities (multiples of 2^-24).
struct alignas(32) GhostSum {
    long long sx, sy, sz;
    uint32_t n;
    uint32_t unused;
};

// FP64 running sums of the lab-grid sample of one cell.
struct alignas(32) SampleAcc {
    double n, vx, vy, vz;
};

// Device-resident bookkeeping shared by all launches of a handle.
struct DeviceState {
    unsigned long long overflow_total;   // particles that found their bucket full
    unsigned int error_flags;            // kErr* bits
    unsigned int ov_count[3];            // overflow list fill, by step modulo 3
    // injected grid shifts (test hook), valid when inject_valid[i] != 0
    unsigned long long inject_step[kMaxInjectedShifts];
    float inject_shift[kMaxInjectedShifts][4];
    unsigned int inject_valid[kMaxInjectedShifts];
    unsigned long long step_base;        // graph replays: absolute step of the replay's first step
    double wall_impulse[2];              // pressure estimator: outward impulse on the z walls {bottom, top}
    unsigned int ext_count[2];           // bucket extension fill, by step parity
};

enum : unsigned int {
    kErrOverflowListFull = 1u,
    kErrWaitTimeout = 2u,
    kErrKeyMismatch = 4u,
    kErrExtensionFull = 8u,
};

constexpr uint32_t kTakenId = 0xFFFFFFFFu;    // overflow-list entry moved to its cell's extension
constexpr uint32_t kChainDone = 0xFFFFFFFFu;  // chain head of a cell the selection has handled
constexpr uint32_t kNoExt = 0xFFFFFFFFu;      // extension offset of a cell whose extension failed

// Injected per-cell draws (reference cell order of box 0), test hook.
struct DrawTables {
    const uint32_t* ghost_count;
    const float* ghost_pos;
    const float* ghost_vel;
    const float* axis;
    const float* gate_u;
    const float* gauss;
    uint32_t gmax, pmax;
};

struct StepArgs {
    BoxDesc box0;                 // the only box of a single-box launch (kernel-parameter space)
    const BoxDesc* boxes;
    int32_t nboxes;
    uint32_t boxes_tile_cells;    // the largest tile (cells) of any box of the launch
    const TileEntry* tile_info;   // ensembles: one entry per tile
    uint32_t num_tiles;
    uint64_t total_slots;         // bucket slots of all boxes; the extension area follows them
    uint32_t ext_cap;             // extension slots (>= every box's cap)
    uint64_t step;                // k: this launch completes step k (step_base: k - *step_base)
    const unsigned long long* step_base;   // non-null in graph replays: k = *step_base + step
    // buckets holding the particles entering collision k (streamed, shifted)
    const Slot* in_slots;
    const uint32_t* in_count;
    // buckets receiving the particles entering collision k+1
    Slot* out_slots;
    uint32_t* out_count;
    uint32_t* zero_count;         // counts of step k-1: cleared here for step k+1
    // overflow lists: in = pending for step k, out = for step k+1
    const float4* ov_in_pos;
    const float4* ov_in_vel;
    float4* ov_out_pos;
    float4* ov_out_vel;
    uint32_t ov_cap;
    uint32_t ov_in_slot, ov_out_slot, ov_zero_slot;   // indices into DeviceState::ov_count
    // overflow chains: per cell the list entry of the last particle that found the
    // cell's bucket full, per entry the one before it.  Heads alternate by step
    // parity and are never cleared: a step reads the head of a cell only when the
    // cell's count exceeds its depth, so the previous step's claims wrote it, and
    // it follows exactly count - depth links (the last one would lead to older
    // entries).  The selection sets a handled cell's head to kChainDone, so that a
    // second selection of the same step (the layout dump runs one) changes nothing.
    const uint32_t* ov_head_in;
    uint32_t* ov_head_out;
    const uint32_t* ov_next_in;   // by entry of ov_in
    uint32_t* ov_next_out;        // by entry of ov_out
    // replay: recompute collision k and write the post-collision state to dense
    // (N, 3) arrays by particle id, changing nothing else
    int32_t replay;
    float* dense_pos;
    float* dense_vel;
    DeviceState* state;
    int32_t sample;               // accumulate the lab-grid sample of clean(k+1)
    float4* samp;                 // [global lab cells, storage order] (sum vx, vy, vz, count)
    // srd_run_kernel sampled steps: the previous step's sample (the other parity's
    // buffer) to fold into acc, or null (the engine folds it with sample_finalize_kernel)
    float4* fold_samp;
    SampleAcc* acc;
    float ext_axis[13][3];        // discrete axis set of the extended collision
    DrawTables draws;             // used by the injected-draw instantiation
    // adjoint tape of this step, by particle id / cell (null: not recorded):
    //   tape_key[id]  = collision cell (global storage index) if the particle was
    //                   collided (cell with n > 1), else kTapeNone;
    //   tape_lab[id]  = lab cell it was sampled in (global storage index) |
    //                   kTapeBounce if the streaming that follows bounced it;
    //   tape_ncell[c] = particles incl. ghosts of collided cell c (storage index).
    // The scatter records only the bounce bit of its streaming in tape_lab.
    uint32_t* tape_key;
    uint32_t* tape_lab;
    uint32_t* tape_ncell;
    // pressure estimator on: accumulate the z impulse the fluid gives the walls
    // (bounce-backs and collisions in the wall-layer cells) into state->wall_impulse
    int32_t pressure;
    // srd_run_kernel steps: the wall ghosts of step k, drawn by the step's
    // prologue (overflow_select_kernel), entry wall_base + 2 (x + Lx y) + top
    GhostSum* ghosts;
    // runs of up to 32 consecutive cells of one box (srd_run_kernel): per run
    // {first global cell, cells | box << 6}; a single box computes them
    const uint2* run_info;
    uint32_t num_runs;
    uint32_t run_class[4];        // runs [run_class[c], run_class[c+1]) take batches of 16, 8, 4 cells (c = 0, 1, 2)
    uint32_t boxes_n_max;         // the largest density of any box
    uint64_t total_walls;         // wall-ghost entries of all boxes
    float4* box_shifts;           // ensembles: grid shifts of steps k and k+1 per box (drawn by the prologue)
    int32_t run_kernel;           // this step runs srd_run_kernel (the engine's choice, run_kernel_takes)
};

constexpr uint32_t kTapeNone = 0xFFFFFFFFu;
constexpr uint32_t kTapeBounce = 0x80000000u;

}  // namespace mpcd_gb
