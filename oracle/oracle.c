/*
 * MPCD oracle -- TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Every function below restates, operation by operation, the reference CPU
 * code it cites (paths relative to the azantop/cudaMPCD tree).  The float
 * expressions keep the reference's evaluation order; the file must be built
 * with -ffp-contract=off so that no multiply-add is fused.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ======================================================================= RNG */

/* common/random.hpp:66-74 */
void orc_xoshiro_seed(orc_xoshiro *r, uint64_t a, uint64_t b)
{
    r->s[0] = (uint32_t)(a >> 2);
    r->s[1] = (uint32_t)b;
    r->s[2] = (uint32_t)(b >> 2);
    r->s[3] = (uint32_t)a;
    r->z1_f = 0.0f;
    r->generate_f = 0;
}

static inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

/* common/random.hpp:80-92 */
uint32_t orc_xoshiro_next(orc_xoshiro *r)
{
    uint32_t *s = r->s;
    const uint32_t result = s[0] + s[3];
    const uint32_t t = s[1] << 9;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl32(s[3], 11);
    return result;
}

/* common/random.hpp:126-129: u32 * (1/UINT32_MAX) in float, range [0, 1] */
float orc_xoshiro_uniform(orc_xoshiro *r)
{
    return (float)orc_xoshiro_next(r) * (1.0f / (float)UINT32_MAX);
}

/* common/random.hpp:134-136 */
int32_t orc_xoshiro_uniform_int(orc_xoshiro *r, int32_t lo, int32_t hi)
{
    return (int32_t)(orc_xoshiro_next(r) / 2) % (hi - lo + 1) + lo;
}

/* common/random.hpp:141-164 (host branch): Box-Muller, second value cached */
float orc_xoshiro_gaussian(orc_xoshiro *r)
{
    r->generate_f = !r->generate_f;
    if (!r->generate_f)
        return r->z1_f;
    float u1 = logf(orc_xoshiro_uniform(r) + FLT_MIN);
    float u2 = (float)orc_xoshiro_next(r) * (2.0f / (float)UINT32_MAX);
    r->z1_f = sinf(u2 * (float)M_PI);
    u2 = cosf(u2 * (float)M_PI);
    r->z1_f *= sqrtf(-2 * u1);
    return u2 * sqrtf(-2 * u1);
}

/* common/random.hpp:237-253 (host branch): Marsaglia's method */
void orc_xoshiro_unit_vector(orc_xoshiro *r, float out[3])
{
    float rsq, rd1, rd2;
    do {
        rd1 = 1.0f - 2.0f * orc_xoshiro_uniform(r);
        rd2 = 1.0f - 2.0f * orc_xoshiro_uniform(r);
        rsq = rd1 * rd1 + rd2 * rd2;
    } while (rsq > 1.0f);
    float rdh = 2.0f * sqrtf(1.0f - rsq);
    out[0] = rd1 * rdh;
    out[1] = rd2 * rdh;
    out[2] = 1.0f - 2.0f * rsq;
}

void orc_xoshiro_sequence(uint64_t a, uint64_t b, int32_t kind, size_t n, void *out)
{
    orc_xoshiro r;
    orc_xoshiro_seed(&r, a, b);
    for (size_t i = 0; i < n; ++i) {
        switch (kind) {
        case 0: ((uint32_t *)out)[i] = orc_xoshiro_next(&r); break;
        case 1: ((float *)out)[i] = orc_xoshiro_uniform(&r); break;
        case 2: ((float *)out)[i] = orc_xoshiro_gaussian(&r); break;
        default: orc_xoshiro_unit_vector(&r, (float *)out + 3 * i); break;
        }
    }
}

/* ------------------------------------------------------------- Philox4x32-10
 * Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
 * SC'11.  Multipliers 0xD2511F53 / 0xCD9E8D57, Weyl key increments
 * 0x9E3779B9 / 0xBB67AE85, ten rounds. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        if (round) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Draw model of the GPU backend.  Counter = {a, step_lo, purpose | step_hi << 8, d},
 * key = seed.  Purposes: */
enum { GB_SHIFT = 1, GB_AXIS = 2, GB_GHOST_COUNT = 3, GB_GHOST = 4, GB_THERMAL = 5, GB_GHOST_SUM = 7 };

static void gb_draw(uint64_t seed, uint64_t step, uint32_t purpose, uint32_t a, uint32_t d, uint32_t out[4])
{
    uint32_t ctr[4] = {a, (uint32_t)step, purpose | ((uint32_t)(step >> 32) << 8), d};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    orc_philox4x32_10(ctr, key, out);
}

/* [0, 1) with 24 random bits */
static inline float gb_u01(uint32_t u) { return (float)(u >> 8) * 0x1p-24f; }
/* (0, 1] with 24 random bits */
static inline float gb_u01_open(uint32_t u) { return (float)((u >> 8) + 1u) * 0x1p-24f; }

/* Box-Muller: r = sqrt(-2 ln u_a), angle = 2 pi u_b */
static inline void gb_box_muller(uint32_t ua, uint32_t ub, float *g0, float *g1)
{
    float r = sqrtf(-2.0f * logf(gb_u01_open(ua)));
    double t = (double)(2.0f * gb_u01(ub));
    *g0 = r * (float)cos(M_PI * t);
    *g1 = r * (float)sin(M_PI * t);
}

void orc_gb_shift(uint64_t seed, uint64_t step, float out[3])
{
    uint32_t o[4];
    gb_draw(seed, step, GB_SHIFT, 0, 0, o);
    for (int i = 0; i < 3; ++i)
        out[i] = gb_u01(o[i]) - 0.5f;
}

/* The discrete axis set of the extended collision, built exactly as
 * cpu_backend/simulation_functions.cpp:272-290 builds one axis: select in
 * [0, 12], phi_i = select % 4 + 1, theta_i = select / 4 + 1, "edge" polar
 * angle 0.9553166 for odd/odd. */
void orc_gb_ext_axis_table(float table[13][3])
{
    const int steps = 4;
    for (int select = 0; select <= 12; ++select) {
        int phi_i = select % steps + 1, theta_i = select / steps + 1;
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
}

/* ================================================================= geometry */

/* float -> uint32 as the reference's x86-64 build converts (via a 64-bit
 * signed truncation), so that out-of-range coordinates wrap identically. */
static inline uint32_t f2u_ref(float x) { return (uint32_t)(int64_t)x; }

/* cpu_backend/volume_container.hpp:330-336 */
uint32_t orc_cell_index(const orc_params *p, const float pos[3])
{
    uint32_t x = f2u_ref(floorf(pos[0] + (float)p->L[0] * 0.5f)) % (uint32_t)p->L[0];
    uint32_t y = f2u_ref(floorf(pos[1] + (float)p->L[1] * 0.5f)) % (uint32_t)p->L[1];
    uint32_t z = f2u_ref(floorf(pos[2] + (float)p->L[2] * 0.5f)) % (uint32_t)p->L[2];
    return x + (y * (uint32_t)p->L[0]) + (z * (uint32_t)(p->L[0] * p->L[1]));
}

/* Storage order of the GPU backend's cell buckets: z fastest, then x, then y. */
uint32_t orc_storage_index(const orc_params *p, uint32_t ref)
{
    uint32_t Lx = (uint32_t)p->L[0], Ly = (uint32_t)p->L[1], Lz = (uint32_t)p->L[2];
    uint32_t x = ref % Lx, y = (ref / Lx) % Ly, z = ref / (Lx * Ly);
    return z + Lz * (x + Lx * y);
}

/* cpu_backend/volume_container.hpp:347-352 */
static void cell_centre(const orc_params *p, uint32_t idx, float out[3])
{
    uint32_t Lx = (uint32_t)p->L[0], xy = (uint32_t)(p->L[0] * p->L[1]);
    out[0] = (0.5f + (float)(idx % Lx)) - (float)p->L[0] * 0.5f;
    out[1] = (0.5f + (float)((idx % xy) / Lx)) - (float)p->L[1] * 0.5f;
    out[2] = (0.5f + (float)(idx / xy)) - (float)p->L[2] * 0.5f;
}

/* the apply_periodic_boundaries lambda, simulation_functions.cpp:46-51 */
static inline void pbc(const orc_params *p, float r[3])
{
    for (int a = 0; a < 3; ++a) {
        float L = (float)p->L[a];
        r[a] = fmodf(r[a] + 1.5f * L, L) - L * 0.5f;
    }
}

/* ============================================================ initialisation */

/* cpu_backend/simulation_functions.cpp:7-33 */
void orc_distribute(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N, orc_xoshiro *r)
{
    float scale[3];
    for (int a = 0; a < 3; ++a)
        scale[a] = (float)p->L[a] - (float)(2 * (1 - p->periodic[a]));
    float R2 = ((float)p->L[0] - 2) * ((float)p->L[0] - 2) * 0.25f;
    for (size_t i = 0; i < N; ++i) {
        float x[3];
        int replace;
        do {
            replace = 0;
            x[0] = orc_xoshiro_uniform(r);
            x[1] = orc_xoshiro_uniform(r);
            x[2] = orc_xoshiro_uniform(r);
            for (int a = 0; a < 3; ++a)
                x[a] = (x[a] - 0.5f) * scale[a];
            if (p->experiment == ORC_CHANNEL)
                replace = (x[2] * x[2] + x[1] * x[1]) > R2;
        } while (replace);
        float g0 = orc_xoshiro_gaussian(r);
        float g1 = orc_xoshiro_gaussian(r);
        float g2 = orc_xoshiro_gaussian(r);
        memcpy(pos + 3 * i, x, sizeof x);
        vel[3 * i + 0] = g0 * p->thermal_velocity;
        vel[3 * i + 1] = g1 * p->thermal_velocity;
        vel[3 * i + 2] = g2 * p->thermal_velocity;
        if (cell)
            cell[i] = orc_cell_index(p, x);
    }
}

/* ================================================================ streaming */

/* cpu_backend/simulation_functions.cpp:38-103 */
void orc_translate(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                   const float shift[3], uint32_t *counter, uint32_t *table)
{
    const uint32_t C = (uint32_t)(p->L[0] * p->L[1] * p->L[2]);
    const float Lz = (float)p->L[2];
    const float channel_radius2 = (Lz - 2) * (Lz - 2) * 0.25f;
    const float dt = p->dt;

    for (size_t idx = 0; idx < N; ++idx) {
        float *x = pos + 3 * idx, *v = vel + 3 * idx;
        if (p->experiment != ORC_CHANNEL) {
            if (!p->periodic[2]) {
                float z_wall = (0.5f * Lz - 1);
                float next_z = x[2] + v[2] * dt;
                if (fabsf(next_z) > z_wall) {
                    float time_left = (next_z > 0 ? z_wall - x[2] : -z_wall - x[2]) / v[2];
                    for (int a = 0; a < 3; ++a) x[a] += v[a] * time_left;
                    for (int a = 0; a < 3; ++a) v[a] = -v[a];
                    for (int a = 0; a < 3; ++a) x[a] += v[a] * (dt - time_left);
                } else {
                    for (int a = 0; a < 3; ++a) x[a] += v[a] * dt;
                }
            } else {
                for (int a = 0; a < 3; ++a) x[a] += v[a] * dt;
            }
        } else {
            for (int a = 0; a < 3; ++a) x[a] += v[a] * dt;
            if ((x[2] * x[2] + x[1] * x[1]) > channel_radius2) {
                for (int a = 0; a < 3; ++a) x[a] -= v[a] * dt;
                for (int a = 0; a < 3; ++a) v[a] = -v[a];
            }
        }

        for (int a = 0; a < 3; ++a) x[a] = x[a] + shift[a];
        pbc(p, x);
        uint32_t c = orc_cell_index(p, x);
        if (cell) cell[idx] = c;

        uint32_t slot = counter[c];
        counter[c] += 1;
        if (slot < p->cap) {
            table[c + (size_t)slot * C] = (uint32_t)idx;
        } else {
            for (int a = 0; a < 3; ++a) x[a] = x[a] - shift[a];
            pbc(p, x);
        }
    }
}

/* ================================================================ collisions */

typedef struct {
    float x[3], v[3];
    int64_t idx;  /* -1 for a ghost */
} orc_particle;

/* Wall-layer test shared by both collisions (simulation_functions.cpp:137-138). */
static void wall_layer(const orc_params *p, uint32_t c, unsigned sign, int *layer, int *add_ghosts)
{
    float zidx = (float)(c / (uint32_t)(p->L[0] * p->L[1]));
    *layer = zidx == ((float)p->L[2] - (sign ? 1 : 2));
    *add_ghosts = (!p->periodic[2]) && ((zidx == (float)sign) || *layer);
}

static uint32_t draw_ghost_count(const orc_params *p, orc_draws *d, uint32_t c, float shift, int layer,
                                 unsigned sign)
{
    uint32_t g = 0;
    if (d->mode == ORC_DRAWS_XOSHIRO) {
        for (uint32_t i = 0; i < p->n_density; ++i)
            if (((orc_xoshiro_uniform(d->rng) > shift) ^ layer ^ sign))
                ++g;
    } else if (d->mode == ORC_DRAWS_TABLE) {
        g = d->ghost_count[c];
    } else {
        uint32_t o[4];
        for (uint32_t i = 0; i < p->n_density; ++i) {
            if ((i & 3) == 0)
                gb_draw(d->seed, d->step, GB_GHOST_COUNT, c, i >> 2, o);
            if (((gb_u01(o[i & 3]) > shift) ^ layer ^ sign))
                ++g;
        }
    }
    if (d->mode != ORC_DRAWS_TABLE && d->ghost_count)
        d->ghost_count[c] = g;
    return g;
}

/* One ghost particle: simulation_functions.cpp:156-166. */
static void draw_ghost(const orc_params *p, orc_draws *d, uint32_t c, uint32_t j, const float centre[3],
                       float shift, int layer, unsigned sign, orc_particle *out)
{
    if (d->mode == ORC_DRAWS_XOSHIRO) {
        float z;
        do {
            z = orc_xoshiro_uniform(d->rng);
        } while (((z < shift) ^ layer) ^ sign);
        /* The reference builds Vector(U - 0.5f, U - 0.5f, z - 0.5f); its x86-64
         * GCC build evaluates the two constructor arguments right to left. */
        float uy = orc_xoshiro_uniform(d->rng);
        float ux = orc_xoshiro_uniform(d->rng);
        out->x[0] = (ux - 0.5f) + centre[0];
        out->x[1] = (uy - 0.5f) + centre[1];
        out->x[2] = (z - 0.5f) + centre[2];
        float g0 = orc_xoshiro_gaussian(d->rng);
        float g1 = orc_xoshiro_gaussian(d->rng);
        float g2 = orc_xoshiro_gaussian(d->rng);
        out->v[0] = g0 * p->thermal_velocity;
        out->v[1] = g1 * p->thermal_velocity;
        out->v[2] = g2 * p->thermal_velocity;
    } else if (d->mode == ORC_DRAWS_TABLE) {
        memcpy(out->x, d->ghost_pos + ((size_t)c * d->gmax + j) * 3, sizeof out->x);
        memcpy(out->v, d->ghost_vel + ((size_t)c * d->gmax + j) * 3, sizeof out->v);
    } else {
        uint32_t o[4];
        gb_draw(d->seed, d->step, GB_GHOST, c, 2 * j, o);
        float ux = gb_u01(o[0]), uy = gb_u01(o[1]), uz = gb_u01(o[2]);
        /* accept region of the reference's rejection loop: z < shift iff layer ^ sign */
        float z = (layer ^ sign) ? shift * uz : shift + (1.0f - shift) * uz;
        out->x[0] = (ux - 0.5f) + centre[0];
        out->x[1] = (uy - 0.5f) + centre[1];
        out->x[2] = (z - 0.5f) + centre[2];
        gb_draw(d->seed, d->step, GB_GHOST, c, 2 * j + 1, o);
        float g0, g1, g2, g3;
        gb_box_muller(o[0], o[1], &g0, &g1);
        gb_box_muller(o[2], o[3], &g2, &g3);
        out->v[0] = g0 * p->thermal_velocity;
        out->v[1] = g1 * p->thermal_velocity;
        out->v[2] = g2 * p->thermal_velocity;
    }
    out->idx = -1;
    if (d->mode != ORC_DRAWS_TABLE && d->ghost_pos && j < d->gmax) {
        memcpy(d->ghost_pos + ((size_t)c * d->gmax + j) * 3, out->x, sizeof out->x);
        memcpy(d->ghost_vel + ((size_t)c * d->gmax + j) * 3, out->v, sizeof out->v);
    }
}

static void draw_srd_axis(orc_draws *d, uint32_t c, float axis[3])
{
    if (d->mode == ORC_DRAWS_XOSHIRO) {
        orc_xoshiro_unit_vector(d->rng, axis);
    } else if (d->mode == ORC_DRAWS_TABLE) {
        memcpy(axis, d->axis + 3 * (size_t)c, 3 * sizeof(float));
    } else {
        uint32_t o[4];
        gb_draw(d->seed, d->step, GB_AXIS, c, 0, o);
        float z = 1.0f - 2.0f * gb_u01(o[0]);
        float rho = sqrtf(fmaxf(0.0f, 1.0f - z * z));
        double t = (double)(2.0f * gb_u01(o[1]));
        axis[0] = rho * (float)cos(M_PI * t);
        axis[1] = rho * (float)sin(M_PI * t);
        axis[2] = z;
    }
    if (d->mode != ORC_DRAWS_TABLE && d->axis)
        memcpy(d->axis + 3 * (size_t)c, axis, 3 * sizeof(float));
}

/* axis and gate uniform of the extended collision (simulation_functions.cpp:272-293, 346) */
static void draw_ext_axis(orc_draws *d, uint32_t c, float axis[3], uint32_t *gate_bits)
{
    if (d->mode == ORC_DRAWS_XOSHIRO) {
        const int steps = 4;
        int select = orc_xoshiro_uniform_int(d->rng, 0, steps * (steps - 1));
        int phi_i = select % steps + 1, theta_i = select / steps + 1;
        float theta, phi;
        if ((theta_i % 2) && (phi_i % 2))
            theta = theta_i == 1 ? 0.95531661812450927816f : (float)M_PI - 0.95531661812450927816f;
        else
            theta = theta_i * ((float)M_PI / steps);
        phi = phi_i * ((float)M_PI / steps);
        axis[0] = sinf(theta) * cosf(phi);
        axis[1] = sinf(theta) * sinf(phi);
        axis[2] = cosf(theta);
        if (orc_xoshiro_uniform_int(d->rng, 0, 1))
            for (int a = 0; a < 3; ++a) axis[a] = -axis[a];
    } else if (d->mode == ORC_DRAWS_TABLE) {
        memcpy(axis, d->axis + 3 * (size_t)c, 3 * sizeof(float));
    } else {
        static float table[13][3];
        static int have_table = 0;
        if (!have_table) {
            orc_gb_ext_axis_table(table);
            have_table = 1;
        }
        uint32_t o[4];
        gb_draw(d->seed, d->step, GB_AXIS, c, 0, o);
        uint32_t select = (o[0] >> 1) % 13u;
        memcpy(axis, table[select], 3 * sizeof(float));
        if ((o[1] >> 1) & 1u)
            for (int a = 0; a < 3; ++a) axis[a] = -axis[a];
        *gate_bits = o[2];
    }
    if (d->mode != ORC_DRAWS_TABLE && d->axis)
        memcpy(d->axis + 3 * (size_t)c, axis, 3 * sizeof(float));
}

static float draw_gate(orc_draws *d, uint32_t c, uint32_t gate_bits)
{
    float u;
    if (d->mode == ORC_DRAWS_XOSHIRO)
        u = orc_xoshiro_uniform(d->rng);
    else if (d->mode == ORC_DRAWS_TABLE)
        u = d->gate_u[c];
    else
        u = gb_u01(gate_bits);
    if (d->mode != ORC_DRAWS_TABLE && d->gate_u)
        d->gate_u[c] = u;
    return u;
}

static float draw_thermal(orc_draws *d, uint32_t c, uint32_t i)
{
    float g;
    if (d->mode == ORC_DRAWS_XOSHIRO) {
        g = orc_xoshiro_gaussian(d->rng);
    } else if (d->mode == ORC_DRAWS_TABLE) {
        g = d->gauss[(size_t)c * d->pmax + i];
    } else {
        uint32_t o[4];
        gb_draw(d->seed, d->step, GB_THERMAL, c, i >> 2, o);
        uint32_t pair = (i & 3u) >> 1;
        float g0, g1;
        gb_box_muller(o[2 * pair], o[2 * pair + 1], &g0, &g1);
        g = (i & 1u) ? g1 : g0;
    }
    if (d->mode != ORC_DRAWS_TABLE && d->gauss && i < d->pmax)
        d->gauss[(size_t)c * d->pmax + i] = g;
    return g;
}

static inline float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static inline void cross3(const float a[3], const float b[3], float o[3])
{
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* Write the real particles of a cell back (simulation_functions.cpp:191-200). */
static void write_back(const orc_params *p, orc_particle *buf, uint32_t n_real, float *pos, float *vel,
                       uint32_t *cell, size_t N)
{
    for (uint32_t i = 0; i < n_real; ++i) {
        if (buf[i].idx != -1 && (size_t)buf[i].idx < N) {
            size_t k = (size_t)buf[i].idx;
            memcpy(pos + 3 * k, buf[i].x, sizeof buf[i].x);
            memcpy(vel + 3 * k, buf[i].v, sizeof buf[i].v);
            if (cell) cell[k] = orc_cell_index(p, buf[i].x);
        }
    }
}

/* cpu_backend/simulation_functions.cpp:108-202.  The reference's per-cell
 * buffer holds `cap` particles and can be overrun when a wall cell has
 * cap real particles plus ghosts; this restatement sizes it cap + n. */
int orc_srd_collision(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                      const float shift3[3], const uint32_t *counter, const uint32_t *table,
                      orc_draws *d)
{
    const uint32_t C = (uint32_t)(p->L[0] * p->L[1] * p->L[2]);
    const uint32_t cap = p->cap;
    const float shift = fabsf(shift3[2]);
    const unsigned sign = shift3[2] > 0;
    const float sin_alpha = sinf((float)((M_PI * 120) / 180));
    const float cos_alpha = cosf((float)((M_PI * 120) / 180));
    const float drag = p->drag * p->dt;

    orc_particle *buf = (orc_particle *)malloc(sizeof(orc_particle) * (cap + p->n_density + 1));
    if (!buf) return -1;

    for (uint32_t c = 0; c < C; ++c) {
        uint32_t n = counter[c] < cap ? counter[c] : cap;
        int layer, add_ghosts;
        wall_layer(p, c, sign, &layer, &add_ghosts);
        uint32_t g = 0;
        if (add_ghosts)
            g = draw_ghost_count(p, d, c, shift, layer, sign);
        else if (d->ghost_count && d->mode != ORC_DRAWS_TABLE)
            d->ghost_count[c] = 0;
        n += g;

        uint32_t n_real = (n - g) < cap ? (n - g) : cap;
        for (uint32_t i = 0; i < n_real; ++i) {
            uint32_t k = table[c + (size_t)i * C];
            buf[i].idx = k;
            memcpy(buf[i].x, pos + 3 * (size_t)k, sizeof buf[i].x);
            memcpy(buf[i].v, vel + 3 * (size_t)k, sizeof buf[i].v);
        }
        if (add_ghosts && d->mode == ORC_DRAWS_PHILOX) {
            /* The GPU's draw model of SRD ghosts: their summed velocity, one
             * Gaussian of variance g T per component, carried by the first ghost
             * (the SRD collision uses the ghosts only through their sum). */
            float centre[3];
            cell_centre(p, c, centre);
            for (uint32_t i = n - g; i < n; ++i) {
                memcpy(buf[i].x, centre, sizeof buf[i].x);
                buf[i].v[0] = buf[i].v[1] = buf[i].v[2] = 0.0f;
                buf[i].idx = -1;
            }
            if (g) {
                uint32_t o[4];
                gb_draw(d->seed, d->step, GB_GHOST_SUM, c, 0, o);
                float g0, g1, g2, g3;
                gb_box_muller(o[0], o[1], &g0, &g1);
                gb_box_muller(o[2], o[3], &g2, &g3);
                float sc = sqrtf((float)g) * p->thermal_velocity;
                buf[n - g].v[0] = g0 * sc;
                buf[n - g].v[1] = g1 * sc;
                buf[n - g].v[2] = g2 * sc;
            }
        } else if (add_ghosts) {
            float centre[3];
            cell_centre(p, c, centre);
            for (uint32_t i = n - g; i < n; ++i)
                draw_ghost(p, d, c, i - (n - g), centre, shift, layer, sign, &buf[i]);
        }

        if (d->collided) d->collided[c] = n > 1;
        if (n > 1) {
            float mean[3] = {0, 0, 0};
            for (uint32_t i = 0; i < n; ++i)
                for (int a = 0; a < 3; ++a) mean[a] += buf[i].v[a];
            float inv = 1.0f / (float)n;
            for (int a = 0; a < 3; ++a) mean[a] *= inv;

            float axis[3];
            draw_srd_axis(d, c, axis);

            for (uint32_t i = 0; i < n; ++i) {
                float v[3], vpara[3], vperp[3], cr[3];
                for (int a = 0; a < 3; ++a) v[a] = buf[i].v[a] - mean[a];
                float vd = dot3(v, axis);
                for (int a = 0; a < 3; ++a) vpara[a] = axis[a] * vd;
                for (int a = 0; a < 3; ++a) vperp[a] = v[a] - vpara[a];
                cross3(vperp, axis, cr);
                for (int a = 0; a < 3; ++a)
                    buf[i].v[a] = (vpara[a] + cos_alpha * vperp[a]) + sin_alpha * cr[a];
            }
            for (uint32_t i = 0; i < n; ++i) {
                for (int a = 0; a < 3; ++a) buf[i].v[a] += mean[a];
                for (int a = 0; a < 3; ++a) buf[i].x[a] = buf[i].x[a] - shift3[a];
                pbc(p, buf[i].x);
                buf[i].v[0] += drag;
            }
        }
        write_back(p, buf, n_real, pos, vel, cell, N);
    }
    free(buf);
    return 0;
}

/* mechanic.hpp:52-79: SymmetricMatrix::inverse(tolerance); m = {xx,yy,zz,xy,xz,yz} */
static void sym_inverse(const float m[6], float tol, float out[6])
{
    float xx = m[0], yy = m[1], zz = m[2], xy = m[3], xz = m[4], yz = m[5];
    float det = xx * (yy * zz - yz * yz) + xz * (2 * xy * yz - yy * xz) - (xy * xy * zz);
    if (det < 0) det = 0;
    if (det > tol) {
        float inv = 1 / det;
        out[0] = (yy * zz - yz * yz) * inv;
        out[1] = (xx * zz - xz * xz) * inv;
        out[2] = (xx * yy - xy * xy) * inv;
        out[3] = (xz * yz - zz * xy) * inv;
        out[4] = (xy * yz - yy * xz) * inv;
        out[5] = (xy * xz - xx * yz) * inv;
    } else {
        float tr = xx + yy + zz;
        if (tr > tol) {
            float s = 4 / (tr * tr);
            for (int k = 0; k < 6; ++k) out[k] = m[k] * s;
        } else {
            for (int k = 0; k < 6; ++k) out[k] = 0.0f;
        }
    }
}

/* cpu_backend/simulation_functions.cpp:207-406.  Side flags are kept per
 * particle; the reference packs them into a uint64_t, which aliases particles
 * i and i+64 in cells of more than 64 particles. */
int orc_extended_collision(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                           const float shift3[3], const uint32_t *counter, const uint32_t *table,
                           orc_draws *d)
{
    const uint32_t C = (uint32_t)(p->L[0] * p->L[1] * p->L[2]);
    const uint32_t cap = p->cap;
    const float shift = fabsf(shift3[2]);
    const unsigned sign = shift3[2] > 0;
    const float scale = 0.01f;
    const float drag = p->drag * p->dt;
    const float tv = p->thermal_velocity;

    orc_particle *buf = (orc_particle *)malloc(sizeof(orc_particle) * (cap + p->n_density + 1));
    uint8_t *side = (uint8_t *)malloc(cap + p->n_density + 1);
    if (!buf || !side) { free(buf); free(side); return -1; }

    for (uint32_t c = 0; c < C; ++c) {
        uint32_t n = counter[c] < cap ? counter[c] : cap;
        int layer, add_ghosts;
        wall_layer(p, c, sign, &layer, &add_ghosts);
        uint32_t g = 0;
        if (add_ghosts)
            g = draw_ghost_count(p, d, c, shift, layer, sign);
        else if (d->ghost_count && d->mode != ORC_DRAWS_TABLE)
            d->ghost_count[c] = 0;
        n += g;
        if (n > cap) n = cap;

        for (uint32_t i = 0; i < n - g; ++i) {
            uint32_t k = table[c + (size_t)i * C];
            buf[i].idx = k;
            memcpy(buf[i].x, pos + 3 * (size_t)k, sizeof buf[i].x);
            memcpy(buf[i].v, vel + 3 * (size_t)k, sizeof buf[i].v);
        }
        float offset[3];
        cell_centre(p, c, offset);
        if (add_ghosts)
            for (uint32_t i = n - g; i < n; ++i)
                draw_ghost(p, d, c, i - (n - g), offset, shift, layer, sign, &buf[i]);

        if (d->collided) d->collided[c] = 0;
        if (n > 1) {
            float axis[3];
            uint32_t gate_bits = 0;
            draw_ext_axis(d, c, axis, &gate_bits);

            float com[3] = {0, 0, 0}, mean[3] = {0, 0, 0};
            for (uint32_t i = 0; i < n; ++i)
                for (int a = 0; a < 3; ++a) {
                    com[a] += (buf[i].x[a] - offset[a]);
                    mean[a] += buf[i].v[a];
                }
            float inv = 1.0f / (float)n;
            for (int a = 0; a < 3; ++a) {
                com[a] = com[a] * inv + offset[a];
                mean[a] = mean[a] * inv;
            }

            float projection_0 = 0.0f, projection_1;
            int size_0 = 0;
            for (uint32_t i = 0; i < n; ++i) {
                for (int a = 0; a < 3; ++a) buf[i].x[a] -= com[a];
                for (int a = 0; a < 3; ++a) buf[i].v[a] -= mean[a];
                side[i] = dot3(buf[i].x, axis) < 0;
                if (side[i]) {
                    projection_0 += dot3(buf[i].v, axis);
                    size_0 += 1;
                }
            }
            int size_1 = (int)n - size_0;
            projection_1 = -projection_0 / (float)size_1;
            projection_0 = projection_0 / (float)size_0;

            float probability = 1 - expf(scale * (projection_1 - projection_0) * (float)size_0 * (float)size_1);
            float omega[3] = {0, 0, 0};
            int collide = draw_gate(d, c, gate_bits) < probability;
            if (d->collided) d->collided[c] = (uint8_t)collide;

            if (collide) {
                float transfer_0 = projection_1 * ((float)size_1 / (float)size_0);
                float transfer_1 = projection_0 * ((float)size_0 / (float)size_1);
                float mean_0 = 0.0f, mean_1 = 0.0f;
                float I[6] = {0, 0, 0, 0, 0, 0};
                float dL[3] = {0, 0, 0};
                for (uint32_t i = 0; i < n; ++i) {
                    float v_random = draw_thermal(d, c, i) * tv;
                    if (side[i]) mean_0 += v_random; else mean_1 += v_random;
                    float cr[3];
                    cross3(buf[i].x, buf[i].v, cr);
                    for (int a = 0; a < 3; ++a) dL[a] += cr[a];
                    float kick = (v_random - dot3(buf[i].v, axis)) + (side[i] ? transfer_0 : transfer_1);
                    for (int a = 0; a < 3; ++a) buf[i].v[a] += axis[a] * kick;
                    const float *x = buf[i].x;
                    float sq[3] = {x[0] * x[0], x[1] * x[1], x[2] * x[2]};
                    I[0] += sq[1] + sq[2];
                    I[1] += sq[0] + sq[2];
                    I[2] += sq[0] + sq[1];
                    I[3] += -x[0] * x[1];
                    I[4] += -x[0] * x[2];
                    I[5] += -x[1] * x[2];
                }
                float vm0[3], vm1[3];
                float m0 = mean_0 / (float)size_0, m1 = mean_1 / (float)size_1;
                for (int a = 0; a < 3; ++a) { vm0[a] = axis[a] * m0; vm1[a] = axis[a] * m1; }
                for (uint32_t i = 0; i < n; ++i) {
                    const float *vm = side[i] ? vm0 : vm1;
                    for (int a = 0; a < 3; ++a) buf[i].v[a] -= vm[a];
                    float cr[3];
                    cross3(buf[i].x, buf[i].v, cr);
                    for (int a = 0; a < 3; ++a) dL[a] -= cr[a];
                }
                float Ii[6];
                sym_inverse(I, 1e-5f, Ii);
                omega[0] = Ii[0] * dL[0] + Ii[3] * dL[1] + Ii[4] * dL[2];
                omega[1] = Ii[3] * dL[0] + Ii[1] * dL[1] + Ii[5] * dL[2];
                omega[2] = Ii[4] * dL[0] + Ii[5] * dL[1] + Ii[2] * dL[2];
            }

            for (uint32_t i = 0; i < n - g; ++i) {
                for (int a = 0; a < 3; ++a) buf[i].v[a] += mean[a];
                buf[i].v[0] += drag;
                float cr[3];
                cross3(buf[i].x, omega, cr);
                for (int a = 0; a < 3; ++a) buf[i].v[a] -= cr[a];
                for (int a = 0; a < 3; ++a) buf[i].x[a] = (com[a] + buf[i].x[a]) - shift3[a];
                pbc(p, buf[i].x);
            }
        }
        write_back(p, buf, n - g, pos, vel, cell, N);
    }
    free(buf);
    free(side);
    return 0;
}

/* ================================================================= sampling */

/* cpu_backend.cpp:176-213 */
void orc_sample_reference(const orc_params *p, orc_sampler *s, const float *pos, const float *vel, size_t N)
{
    size_t C = s->C;
    uint32_t *density = (uint32_t *)calloc(C, sizeof(uint32_t));
    float *mv = (float *)calloc(3 * C, sizeof(float));
    for (size_t i = 0; i < N; ++i) {
        uint32_t c = orc_cell_index(p, pos + 3 * i);
        density[c] += 1;
        for (int a = 0; a < 3; ++a) mv[3 * c + a] += vel[3 * i + a];
    }
    for (size_t c = 0; c < C; ++c)
        if (density[c] > 0) {
            float inv = 1.0f / (float)density[c];
            for (int a = 0; a < 3; ++a) mv[3 * c + a] = mv[3 * c + a] * inv;
        }
    if (!s->in_progress) {
        s->in_progress = 1;
        s->sample_counter = 0;
        memset(s->kahan_density, 0, sizeof(float) * C);
        memset(s->kahan_velocity, 0, sizeof(float) * 3 * C);
        for (size_t c = 0; c < C; ++c) {
            s->density[c] = (float)density[c];
            for (int a = 0; a < 3; ++a) s->velocity[3 * c + a] = mv[3 * c + a];
        }
    } else {
        s->sample_counter++;
        for (size_t c = 0; c < C; ++c) {
            {
                float y = (float)density[c] - s->kahan_density[c];
                float t = s->density[c] + y;
                s->kahan_density[c] = (t - s->density[c]) - y;
                s->density[c] = t;
            }
            for (int a = 0; a < 3; ++a) {
                float y = mv[3 * c + a] - s->kahan_velocity[3 * c + a];
                float t = s->velocity[3 * c + a] + y;
                s->kahan_velocity[3 * c + a] = (t - s->velocity[3 * c + a]) - y;
                s->velocity[3 * c + a] = t;
            }
        }
    }
    free(density);
    free(mv);
}

/* cpu_backend.cpp:215-226 */
void orc_sample_mean_reference(orc_sampler *s, float *density, float *velocity)
{
    double inverse = 1.0 / (double)s->sample_counter;
    for (size_t c = 0; c < s->C; ++c) {
        density[c] = (float)(s->density[c] * inverse);
        for (int a = 0; a < 3; ++a) velocity[3 * c + a] = (float)(s->velocity[3 * c + a] * inverse);
    }
    s->in_progress = 0;
}

void orc_sample_gb(const orc_params *p, orc_sampler *s, const float *pos, const float *vel, size_t N)
{
    size_t C = s->C;
    memset(s->step_count, 0, sizeof(uint32_t) * C);
    memset(s->step_sum, 0, sizeof(int64_t) * 3 * C);
    for (size_t i = 0; i < N; ++i) {
        uint32_t c = orc_cell_index(p, pos + 3 * i);
        s->step_count[c] += 1;
        for (int a = 0; a < 3; ++a)
            s->step_sum[3 * c + a] += llrint((double)vel[3 * i + a] * 4294967296.0);
    }
    int snapshot = !s->in_progress;
    if (snapshot) {
        s->in_progress = 1;
        s->sample_counter = 0;
    } else {
        s->sample_counter++;
    }
    for (size_t c = 0; c < C; ++c) {
        uint32_t k = s->step_count[c];
        for (int a = 0; a < 3; ++a) {
            float m = k ? (float)((double)s->step_sum[3 * c + a] * 0x1p-32 / (double)k) : 0.0f;
            if (snapshot) s->acc_velocity[3 * c + a] = (double)m;
            else s->acc_velocity[3 * c + a] += (double)m;
        }
        if (snapshot) s->acc_density[c] = (double)k;
        else s->acc_density[c] += (double)k;
    }
}

void orc_sample_mean_gb(orc_sampler *s, float *density, float *velocity)
{
    double inverse = 1.0 / (double)s->sample_counter;
    for (size_t c = 0; c < s->C; ++c) {
        density[c] = (float)(s->acc_density[c] * inverse);
        for (int a = 0; a < 3; ++a) velocity[3 * c + a] = (float)(s->acc_velocity[3 * c + a] * inverse);
    }
    s->in_progress = 0;
}

/* ============================================================== whole steps */

/* CPUBackend::step / stepAndAccumulateSample, cpu_backend.cpp:127-213 */
int orc_reference_steps(const orc_params *p, float *pos, float *vel, uint32_t *cell, size_t N,
                        orc_xoshiro *r, int32_t nsteps, uint32_t *counter, uint32_t *table,
                        orc_sampler *sampler)
{
    const size_t C = (size_t)p->L[0] * p->L[1] * p->L[2];
    orc_draws d;
    memset(&d, 0, sizeof d);
    d.mode = ORC_DRAWS_XOSHIRO;
    d.rng = r;
    for (int32_t s = 0; s < nsteps; ++s) {
        float shift[3];
        shift[0] = orc_xoshiro_uniform(r) - 0.5f;
        shift[1] = orc_xoshiro_uniform(r) - 0.5f;
        shift[2] = orc_xoshiro_uniform(r) - 0.5f;
        memset(counter, 0, sizeof(uint32_t) * C);
        orc_translate(p, pos, vel, cell, N, shift, counter, table);
        int rc = p->algorithm == ORC_SRD ? orc_srd_collision(p, pos, vel, cell, N, shift, counter, table, &d)
                                         : orc_extended_collision(p, pos, vel, cell, N, shift, counter, table, &d);
        if (rc) return rc;
        if (sampler) orc_sample_reference(p, sampler, pos, vel, N);
    }
    return 0;
}

/* ============================================================== utilities */

void orc_stable_perm(const uint32_t *key, size_t N, uint32_t nkeys, uint32_t *perm)
{
    size_t *start = (size_t *)calloc((size_t)nkeys + 1, sizeof(size_t));
    for (size_t i = 0; i < N; ++i) start[key[i] + 1]++;
    for (uint32_t k = 0; k < nkeys; ++k) start[k + 1] += start[k];
    for (size_t i = 0; i < N; ++i) perm[start[key[i]]++] = (uint32_t)i;
    free(start);
}

double orc_time_reference_steps(const orc_params *p, uint64_t seed, int32_t steps)
{
    const size_t C = (size_t)p->L[0] * p->L[1] * p->L[2];
    size_t N = p->n_density;
    for (int a = 0; a < 3; ++a) N *= (size_t)(p->L[a] - 2 * (1 - p->periodic[a]));
    float *pos = (float *)malloc(sizeof(float) * 3 * N);
    float *vel = (float *)malloc(sizeof(float) * 3 * N);
    uint32_t *cell = (uint32_t *)malloc(sizeof(uint32_t) * N);
    uint32_t *counter = (uint32_t *)malloc(sizeof(uint32_t) * C);
    uint32_t *table = (uint32_t *)malloc(sizeof(uint32_t) * C * p->cap);
    if (!pos || !vel || !cell || !counter || !table) {
        free(pos); free(vel); free(cell); free(counter); free(table);
        return -1.0;
    }
    orc_xoshiro r;
    orc_xoshiro_seed(&r, seed, seed ^ 0x9E3779B97F4A7C15ull);
    orc_distribute(p, pos, vel, cell, N, &r);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    orc_reference_steps(p, pos, vel, cell, N, &r, steps, counter, table, NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(pos); free(vel); free(cell); free(counter); free(table);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

struct orc_run {
    orc_params p;
    size_t N, C;
    float *pos, *vel;
    uint32_t *cell, *counter, *table;
    orc_xoshiro rng;
};

orc_run *orc_run_create(const orc_params *p, uint64_t seed)
{
    orc_run *r = (orc_run *)calloc(1, sizeof(orc_run));
    if (!r) return NULL;
    r->p = *p;
    r->C = (size_t)p->L[0] * p->L[1] * p->L[2];
    r->N = p->n_density;
    for (int a = 0; a < 3; ++a) r->N *= (size_t)(p->L[a] - 2 * (1 - p->periodic[a]));
    r->pos = (float *)malloc(sizeof(float) * 3 * r->N);
    r->vel = (float *)malloc(sizeof(float) * 3 * r->N);
    r->cell = (uint32_t *)malloc(sizeof(uint32_t) * r->N);
    r->counter = (uint32_t *)malloc(sizeof(uint32_t) * r->C);
    r->table = (uint32_t *)malloc(sizeof(uint32_t) * r->C * p->cap);
    if (!r->pos || !r->vel || !r->cell || !r->counter || !r->table) {
        orc_run_destroy(r);
        return NULL;
    }
    orc_xoshiro_seed(&r->rng, seed, seed ^ 0x9E3779B97F4A7C15ull);
    orc_distribute(p, r->pos, r->vel, r->cell, r->N, &r->rng);
    return r;
}

int orc_run_steps(orc_run *r, int32_t n)
{
    return orc_reference_steps(&r->p, r->pos, r->vel, r->cell, r->N, &r->rng, n, r->counter, r->table, NULL);
}

/* Wall pressure estimator (test infrastructure; the reference has none): the
 * outward z impulse the fluid gives the walls over n reference steps,
 * impulse[0] bottom, impulse[1] top: 2|v_z| per bounce-back in translate
 * (simulation_functions.cpp:53-82), and minus the real particles' z momentum
 * change in the collisions of the two wall layers on each side, whose ghost
 * particles stand for the wall (simulation_functions.cpp:116-167, 137-138).
 * The collision cell is taken before the collision, which writes the particle's
 * new cell back (simulation_functions.cpp:191-200, 395-400).
 * layer_count (Lz entries, may be NULL) accumulates the particles per z layer
 * of the lab grid after every step. */
int orc_run_pressure_steps(orc_run *r, int32_t n, double impulse[2], double *layer_count)
{
    const orc_params *p = &r->p;
    const size_t N = r->N;
    const uint32_t Lxy = (uint32_t)(p->L[0] * p->L[1]);
    const uint32_t Lz = (uint32_t)p->L[2];
    float *vz = (float *)malloc(sizeof(float) * N);
    uint32_t *cz = (uint32_t *)malloc(sizeof(uint32_t) * N);   /* collision cell z: the collision rewrites cell[] */
    if (!vz || !cz) {
        free(vz);
        free(cz);
        return -1;
    }
    orc_draws d;
    memset(&d, 0, sizeof d);
    d.mode = ORC_DRAWS_XOSHIRO;
    d.rng = &r->rng;
    int rc = 0;
    for (int32_t s = 0; s < n && !rc; ++s) {
        float shift[3];
        shift[0] = orc_xoshiro_uniform(&r->rng) - 0.5f;
        shift[1] = orc_xoshiro_uniform(&r->rng) - 0.5f;
        shift[2] = orc_xoshiro_uniform(&r->rng) - 0.5f;
        memset(r->counter, 0, sizeof(uint32_t) * r->C);
        for (size_t i = 0; i < N; ++i) vz[i] = r->vel[3 * i + 2];
        orc_translate(p, r->pos, r->vel, r->cell, N, shift, r->counter, r->table);
        for (size_t i = 0; i < N; ++i)
            if (!p->periodic[2] && r->vel[3 * i + 2] != vz[i]) impulse[vz[i] > 0 ? 1 : 0] += 2.0 * fabs((double)vz[i]);
        for (size_t i = 0; i < N; ++i) {
            vz[i] = r->vel[3 * i + 2];
            cz[i] = r->cell[i] / Lxy;
        }
        rc = p->algorithm == ORC_SRD
                 ? orc_srd_collision(p, r->pos, r->vel, r->cell, N, shift, r->counter, r->table, &d)
                 : orc_extended_collision(p, r->pos, r->vel, r->cell, N, shift, r->counter, r->table, &d);
        for (size_t i = 0; i < N && !p->periodic[2]; ++i) {
            const double dv = (double)r->vel[3 * i + 2] - (double)vz[i];
            if (cz[i] <= 1) impulse[0] += dv;
            else if (cz[i] + 2 >= Lz) impulse[1] -= dv;
        }
        if (layer_count)
            for (size_t i = 0; i < N; ++i) layer_count[orc_cell_index(p, r->pos + 3 * i) / Lxy] += 1.0;
    }
    free(vz);
    free(cz);
    return rc;
}

size_t orc_run_particles(const orc_run *r) { return r->N; }

void orc_run_destroy(orc_run *r)
{
    if (!r) return;
    free(r->pos); free(r->vel); free(r->cell); free(r->counter); free(r->table);
    free(r);
}
