/*
 * MPCD oracle -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference CPU backend of azantop/cudaMPCD for
 * the MPCD time step (grid shift -> streaming + bounce-back -> cell table ->
 * SRD or extended-MPC collision -> lab-grid sampling).  It exists to check the
 * CUDA kernels of cudampcd_gb300; nothing in the product links or calls it.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Parity pins (see tests/test_oracle_*.py):
 *   - against the reference itself, compiled from its own sources into
 *     oracle/_ref/ (only where the reference sources are present), bit-exact;
 *   - against golden vectors generated from that build and committed under
 *     tests/golden/ (generator: tests/golden/make_golden.py);
 *   - against the reference's own known-answer tests
 *     (tests/unit/cpp/test_simulation_functions.cpp:4-43) and RNG statistics
 *     tests (tests/statistics/test_statistics.py:6-48).
 *
 * Three sources of random draws share one collision implementation:
 *   ORC_DRAWS_XOSHIRO  consume a Xoshiro128+ stream in exactly the order the
 *                      reference CPU code does (and optionally record every
 *                      draw into the tables below);
 *   ORC_DRAWS_TABLE    replay recorded draws (the same tables the CUDA kernel
 *                      accepts in its injected-draw mode);
 *   ORC_DRAWS_PHILOX   the counter-based Philox4x32-10 draw model of the GPU
 *                      backend, restated independently here.
 *
 * Compile with -ffp-contract=off: the reference's float arithmetic is
 * reproduced operation by operation and must not be fused.
 */
#ifndef MPCD_ORACLE_H
#define MPCD_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_STANDARD = 0, ORC_CHANNEL = 1 };
enum { ORC_SRD = 0, ORC_EXTENDED = 1 };
enum { ORC_DRAWS_XOSHIRO = 0, ORC_DRAWS_TABLE = 1, ORC_DRAWS_PHILOX = 2 };

/* Geometry and physics of one box (SimulationParameters,
 * include/mpcd/api/simulation_parameters.hpp:70-102).  L is the container size
 * including wall layers, as the reference's volume_size. */
typedef struct {
    int32_t L[3];
    int32_t periodic[3];
    int32_t experiment;      /* ORC_STANDARD / ORC_CHANNEL */
    int32_t algorithm;       /* ORC_SRD / ORC_EXTENDED */
    float dt;
    float drag;
    float thermal_velocity;
    uint32_t n_density;      /* n: mean particles per cell */
    uint32_t cap;            /* cell table depth, 4n in the reference (backend_context.cu:24) */
} orc_params;

/* Xoshiro128+ with the Box-Muller cache (common/random.hpp:24-258). */
typedef struct {
    uint32_t s[4];
    int32_t generate_f;
    float z1_f;
} orc_xoshiro;

typedef struct {
    int32_t mode;
    orc_xoshiro *rng;        /* XOSHIRO mode */
    uint64_t seed;           /* PHILOX mode: key */
    uint64_t step;           /* PHILOX mode: step counter */
    uint32_t gmax;           /* ghost slots per cell in the tables (>= n) */
    uint32_t pmax;           /* thermal-draw slots per cell (>= cap + n) */
    /* per-cell tables, indexed by reference cell index x + Lx*(y + Ly*z);
     * any may be NULL in XOSHIRO / PHILOX mode (then nothing is recorded) */
    uint32_t *ghost_count;   /* [C] */
    float *ghost_pos;        /* [C][gmax][3] absolute (shifted-frame) position */
    float *ghost_vel;        /* [C][gmax][3] */
    float *axis;             /* [C][3] rotation axis (SRD) / split axis (extended) */
    float *gate_u;           /* [C] extended: uniform compared with the gate */
    float *gauss;            /* [C][pmax] extended: thermal draws, one per particle */
    uint8_t *collided;       /* [C] out: 1 if the cell collided (extended gate / SRD n>1) */
} orc_draws;

/* ---- RNG: reference Xoshiro128+ ------------------------------------------------ */
void orc_xoshiro_seed(orc_xoshiro *r, uint64_t a, uint64_t b);
uint32_t orc_xoshiro_next(orc_xoshiro *r);
float orc_xoshiro_uniform(orc_xoshiro *r);
int32_t orc_xoshiro_uniform_int(orc_xoshiro *r, int32_t lo, int32_t hi);
float orc_xoshiro_gaussian(orc_xoshiro *r);
void orc_xoshiro_unit_vector(orc_xoshiro *r, float out[3]);
/* kind: 0 = u32, 1 = uniform float, 2 = gaussianf, 3 = unit vector (3 floats each) */
void orc_xoshiro_sequence(uint64_t a, uint64_t b, int32_t kind, size_t n, void *out);

/* ---- RNG: Philox4x32-10 draw model of the GPU backend ------------------------ */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
void orc_gb_shift(uint64_t seed, uint64_t step, float out[3]);
void orc_gb_ext_axis_table(float table[13][3]);

/* ---- cell geometry ----------------------------------------------------------- */
uint32_t orc_cell_index(const orc_params *p, const float pos[3]);
uint32_t orc_storage_index(const orc_params *p, uint32_t ref_index);

/* ---- reference functions, restated --------------------------------------------- */
/* cpu_backend/simulation_functions.cpp:7-33 */
void orc_distribute(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N, orc_xoshiro *r);
/* cpu_backend/simulation_functions.cpp:38-103; counter must be zeroed by the caller
 * (cpu_backend.cpp:132) */
void orc_translate(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                   const float shift[3], uint32_t *counter, uint32_t *table);
/* cpu_backend/simulation_functions.cpp:108-202 */
int orc_srd_collision(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                      const float shift[3], const uint32_t *counter, const uint32_t *table,
                      orc_draws *d);
/* cpu_backend/simulation_functions.cpp:207-406 */
int orc_extended_collision(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                           const float shift[3], const uint32_t *counter, const uint32_t *table,
                           orc_draws *d);

/* ---- lab-grid sampling ----------------------------------------------------------- */
typedef struct {
    size_t C;
    int32_t in_progress;     /* SAMPLING_IN_PROGRESS / COMPLETED (cpu_backend.hpp:74-79) */
    uint64_t sample_counter;
    /* reference model: FP32 running sums with Kahan compensation */
    float *density, *velocity;          /* [C], [3C] */
    float *kahan_density, *kahan_velocity;
    /* GPU model: exact per-step fixed-point sums, FP64 running sums */
    double *acc_density, *acc_velocity; /* [C], [3C] */
    uint32_t *step_count;               /* [C] scratch */
    int64_t *step_sum;                  /* [3C] scratch */
    float *step_mean;                   /* [3C] scratch */
} orc_sampler;

/* cpu_backend.cpp:176-213 (reference model, FP32 Kahan) */
void orc_sample_reference(const orc_params *p, orc_sampler *s, const float *pos, const float *vel, size_t N);
/* cpu_backend.cpp:215-226: divides by the sample counter (S-1 for S samples) */
void orc_sample_mean_reference(orc_sampler *s, float *density, float *velocity);
/* GPU sampling model: per step exact fixed-point velocity sums (2^-32 units),
 * float per-cell mean, FP64 accumulation; same snapshot / S-1 semantics */
void orc_sample_gb(const orc_params *p, orc_sampler *s, const float *pos, const float *vel, size_t N);
void orc_sample_mean_gb(orc_sampler *s, float *density, float *velocity);

/* ---- whole steps ------------------------------------------------------------------ */
/* CPUBackend::step (cpu_backend.cpp:127-174): shift from the Xoshiro stream,
 * translate, collide.  table scratch: C*cap, counter: C. */
int orc_reference_steps(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                        orc_xoshiro *r, int32_t nsteps, uint32_t *counter, uint32_t *table,
                        orc_sampler *sampler);

/* Stable counting sort by key: perm[j] = index of the j-th element in sorted order. */
void orc_stable_perm(const uint32_t *key, size_t N, uint32_t nkeys, uint32_t *perm);

/* Wall-clock helper for the CPU baseline: run `steps` reference steps on a
 * freshly distributed box; returns elapsed seconds of the stepping loop. */
double orc_time_reference_steps(const orc_params *p, uint64_t seed, int32_t steps);

/* A persistent box advanced by the restated reference step (CPU baseline). */
typedef struct orc_run orc_run;
orc_run *orc_run_create(const orc_params *p, uint64_t seed);
int orc_run_steps(orc_run *r, int32_t n);
size_t orc_run_particles(const orc_run *r);
/* Wall pressure estimator over n steps: outward z impulse on {bottom, top} walls
 * (bounce-backs + wall-layer collisions); layer_count[Lz] (or NULL) accumulates the
 * particles per lab z layer after every step. */
int orc_run_pressure_steps(orc_run *r, int32_t n, double impulse[2], double *layer_count);
void orc_run_destroy(orc_run *r);

#ifdef __cplusplus
}
#endif
#endif
