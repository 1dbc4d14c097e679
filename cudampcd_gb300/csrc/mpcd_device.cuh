// Device helpers of the GB300 MPCD step: Philox draws and cell geometry.
//
// Compiled with --fmad=false: every float expression below is evaluated as
// separately rounded IEEE operations in the order written, which is the order
// of the reference CPU code (src/libmpcd/cpu_backend/simulation_functions.cpp),
// so streaming, periodic wrapping and cell indices are bit-exact with it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mpcd_types.h"

namespace mpcd_gb {

// ------------------------------------------------------------------ Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3" (SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

// Draw purposes; counter = {a, step_lo, purpose | step_hi << 8, d}, key = box seed.
enum : uint32_t { kShift = 1, kAxis = 2, kGhostCount = 3, kGhost = 4, kThermal = 5, kInit = 6, kGhostSum = 7 };

__device__ __forceinline__ uint4 draw(const BoxDesc& b, uint64_t step, uint32_t purpose, uint32_t a, uint32_t d)
{
    return philox4x32_10(make_uint4(a, (uint32_t)step, purpose | ((uint32_t)(step >> 32) << 8), d), b.seed_lo,
                         b.seed_hi);
}

__device__ __forceinline__ float u01(uint32_t u) { return (float)(u >> 8) * 0x1p-24f; }
__device__ __forceinline__ float u01_open(uint32_t u) { return (float)((u >> 8) + 1u) * 0x1p-24f; }

// Box-Muller: r = sqrt(-2 ln u_a), angle = 2 pi u_b.
__device__ __forceinline__ void box_muller(uint32_t ua, uint32_t ub, float& g0, float& g1)
{
    const float r = sqrtf(-2.0f * logf(u01_open(ua)));
    float s, c;
    sincospif(2.0f * u01(ub), &s, &c);
    g0 = r * c;
    g1 = r * s;
}

// Grid shift of a step: injected (test hook, box 0 only) or drawn.
__device__ __forceinline__ float3 grid_shift(const BoxDesc& b, int box_index, uint64_t step, const DeviceState* st)
{
    if (box_index == 0) {
#pragma unroll
        for (int i = 0; i < kMaxInjectedShifts; ++i)
            if (st->inject_valid[i] && st->inject_step[i] == step)
                return make_float3(st->inject_shift[i][0], st->inject_shift[i][1], st->inject_shift[i][2]);
    }
    const uint4 o = draw(b, step, kShift, 0, 0);
    return make_float3(u01(o.x) - 0.5f, u01(o.y) - 0.5f, u01(o.z) - 0.5f);
}

// ------------------------------------------------------------------ geometry

// apply_periodic_boundaries of the reference: fmodf(r + 1.5 L, L) - 0.5 L.
// For a = r + 1.5L in [0, 3L) the remainder is a - qL with q in {0,1,2}, and
// that difference is exact (Sterbenz), i.e. identical to fmodf.  The common
// case is evaluated branch-free; arguments outside [0, 3L) take fmodf itself.
// L15 = 1.5f * L, L2 = 2.0f * L, L3 = 3.0f * L, Lh = L * 0.5f (exact float products).
__device__ __forceinline__ float pbc1(float r, float L, float L15, float L2, float L3, float Lh)
{
    const float a = r + L15;
    const float q = a >= L2 ? L2 : (a >= L ? L : 0.0f);
    float m = a - q;
    if (__builtin_expect(!(a >= 0.0f && a < L3), 0)) m = fmodf(a, L);
    return m - Lh;
}

// Fast path of pbc1 without its range check.
__device__ __forceinline__ float pbc1_fast(float a, float L, float L2)
{
    return a - (a >= L2 ? L2 : (a >= L ? L : 0.0f));
}

// The general (fmodf) path of pbc for arguments far outside the box; kept out of
// line so the hot loops stay small.
__device__ __noinline__ float3 pbc_general(const BoxDesc& b, float3 r)
{
    return make_float3(pbc1(r.x, b.Lf[0], b.L15[0], b.L2x[0], b.L3x[0], b.Lh[0]),
                       pbc1(r.y, b.Lf[1], b.L15[1], b.L2x[1], b.L3x[1], b.Lh[1]),
                       pbc1(r.z, b.Lf[2], b.L15[2], b.L2x[2], b.L3x[2], b.Lh[2]));
}

// All three axes; one branch to the fmodf path when any a = r + 1.5L leaves [0, 3L).
__device__ __forceinline__ float3 pbc(const BoxDesc& b, float3 r)
{
    const float ax = r.x + b.L15[0], ay = r.y + b.L15[1], az = r.z + b.L15[2];
    // 0 <= a < 3L as one unsigned compare of the bits per axis (non-negative floats
    // order as their bits; negative values, -0 and NaN fail and take the general path)
    const bool in = (__float_as_uint(ax) < __float_as_uint(b.L3x[0])) & (__float_as_uint(ay) < __float_as_uint(b.L3x[1])) &
                    (__float_as_uint(az) < __float_as_uint(b.L3x[2]));
    if (__builtin_expect(in, 1))
        return make_float3(pbc1_fast(ax, b.Lf[0], b.L2x[0]) - b.Lh[0], pbc1_fast(ay, b.Lf[1], b.L2x[1]) - b.Lh[1],
                           pbc1_fast(az, b.Lf[2], b.L2x[2]) - b.Lh[2]);
    return pbc_general(b, r);
}

// pbc() of a position within half a cell of the box, such as x - s for a wrapped
// x and a grid shift |s| <= 1/2: a = r + 1.5L then lies in [0, 3L) for any L >= 1,
// so the range check is skipped; the arithmetic, and so the result, is pbc()'s.
__device__ __forceinline__ float3 pbc_near(const BoxDesc& b, float3 r)
{
    return make_float3(pbc1_fast(r.x + b.L15[0], b.Lf[0], b.L2x[0]) - b.Lh[0],
                       pbc1_fast(r.y + b.L15[1], b.Lf[1], b.L2x[1]) - b.Lh[1],
                       pbc1_fast(r.z + b.L15[2], b.Lf[2], b.L2x[2]) - b.Lh[2]);
}

// Coordinate of a cell along one axis: floor(x + L/2) mod L, with the
// float -> uint32 conversion of the reference's x86-64 build (via int64).
__device__ __forceinline__ uint32_t cell_coord(float x, float Lf, float Lh, uint32_t L)
{
    const float f = floorf(x + Lh);
    uint32_t c = (uint32_t)(int)f;
    c = c == L ? 0u : c;
    if (__builtin_expect(!(f >= 0.0f && f <= Lf), 0)) c = (uint32_t)(long long)f % L;
    return c;
}

// Cell of a position that pbc() produced: x + L/2 lies in [0, L] unless pbc()
// took its fmodf path on a wildly out-of-box argument; one unsigned compare
// routes that case to the general conversion.
__device__ __forceinline__ uint32_t cell_coord_wrapped(float x, float Lh, uint32_t L)
{
    const float f = floorf(x + Lh);
    const uint32_t c = (uint32_t)(int)f;
    if (__builtin_expect(c < L, 1)) return c;
    return c == L ? 0u : (uint32_t)(long long)f % L;
}

// One branch for the three axes on the common path (each axis's own slow path
// recomputes the same floor, so the result is cell_coord_wrapped's on every axis).
__device__ __forceinline__ uint3 cell_of_wrapped(const BoxDesc& b, float3 x)
{
    const float fx = floorf(x.x + b.Lh[0]), fy = floorf(x.y + b.Lh[1]), fz = floorf(x.z + b.Lh[2]);
    const uint32_t cx = (uint32_t)(int)fx, cy = (uint32_t)(int)fy, cz = (uint32_t)(int)fz;
    if (__builtin_expect((cx < (uint32_t)b.L[0]) & (cy < (uint32_t)b.L[1]) & (cz < (uint32_t)b.L[2]), 1))
        return make_uint3(cx, cy, cz);
    return make_uint3(cell_coord_wrapped(x.x, b.Lh[0], (uint32_t)b.L[0]),
                      cell_coord_wrapped(x.y, b.Lh[1], (uint32_t)b.L[1]),
                      cell_coord_wrapped(x.z, b.Lh[2], (uint32_t)b.L[2]));
}

__device__ __forceinline__ uint3 cell_of(const BoxDesc& b, float3 x)
{
    return make_uint3(cell_coord(x.x, b.Lf[0], b.Lh[0], (uint32_t)b.L[0]),
                      cell_coord(x.y, b.Lf[1], b.Lh[1], (uint32_t)b.L[1]),
                      cell_coord(x.z, b.Lf[2], b.Lh[2], (uint32_t)b.L[2]));
}

// reference cell index x + Lx*(y + Ly*z) (volume_container.hpp:330-336)
__device__ __forceinline__ uint32_t ref_index(const BoxDesc& b, uint3 c)
{
    return c.x + c.y * (uint32_t)b.L[0] + c.z * (uint32_t)(b.L[0] * b.L[1]);
}

// storage index z + Lz*(x + Lx*y)
__device__ __forceinline__ uint32_t storage_index(const BoxDesc& b, uint3 c)
{
    return c.z + (uint32_t)b.L[2] * (c.x + (uint32_t)b.L[0] * c.y);
}

// n / d for n < 2^31, d <= 2^16, with m = ceil(2^48 / d): floor(n m / 2^48)
// (the error n (m - 2^48/d) / 2^48 < 2^-17 stays below 1/d)
__device__ __forceinline__ uint32_t fast_div(uint32_t n, uint64_t m)
{
    return (uint32_t)__umul64hi((uint64_t)n << 16, m);
}

__device__ __forceinline__ uint3 storage_coords(const BoxDesc& b, uint32_t s)
{
    const uint32_t Lz = (uint32_t)b.L[2], Lx = (uint32_t)b.L[0];
    const uint32_t col = fast_div(s, b.div_z), z = s - col * Lz;
    const uint32_t y = fast_div(col, b.div_x), x = col - y * Lx;
    return make_uint3(x, y, z);
}

// centre of a cell in the shifted frame (volume_container.hpp:347-352)
__device__ __forceinline__ float3 cell_centre(const BoxDesc& b, uint3 c)
{
    return make_float3((0.5f + (float)c.x) - b.Lh[0], (0.5f + (float)c.y) - b.Lh[1], (0.5f + (float)c.z) - b.Lh[2]);
}

// Streaming with bounce-back (simulation_functions.cpp:53-82), in place.
__device__ __forceinline__ void stream(const BoxDesc& b, float3& x, float3& v)
{
    const float dt = b.dt;
    if (!b.channel) {
        if (b.wall_z) {
            const float z_wall = (b.Lh[2] - 1);   // 0.5f * Lz - 1
            const float next_z = x.z + v.z * dt;
            if (fabsf(next_z) > z_wall) {
                const float time_left = (next_z > 0 ? z_wall - x.z : -z_wall - x.z) / v.z;
                x.x += v.x * time_left; x.y += v.y * time_left; x.z += v.z * time_left;
                v.x = -v.x; v.y = -v.y; v.z = -v.z;
                const float rest = dt - time_left;
                x.x += v.x * rest; x.y += v.y * rest; x.z += v.z * rest;
            } else {
                x.x += v.x * dt; x.y += v.y * dt; x.z += v.z * dt;
            }
        } else {
            x.x += v.x * dt; x.y += v.y * dt; x.z += v.z * dt;
        }
    } else {
        x.x += v.x * dt; x.y += v.y * dt; x.z += v.z * dt;
        if ((x.z * x.z + x.y * x.y) > b.R2) {
            x.x -= v.x * dt; x.y -= v.y * dt; x.z -= v.z * dt;
            v.x = -v.x; v.y = -v.y; v.z = -v.z;
        }
    }
}

// Stream, shift and wrap: the position a particle has in the collision of a step.
__device__ __forceinline__ float3 stream_shift(const BoxDesc& b, float3 x, float3& v, float3 s)
{
    stream(b, x, v);
    return pbc(b, make_float3(x.x + s.x, x.y + s.y, x.z + s.z));
}

// Wall-layer test of a cell in the shifted frame (simulation_functions.cpp:137-138).
__device__ __forceinline__ void wall_layer(const BoxDesc& b, uint32_t cz, bool sign, bool& layer, bool& ghosts)
{
    layer = cz == (uint32_t)(b.L[2] - (sign ? 1 : 2));
    ghosts = b.wall_z && (cz == (uint32_t)sign || layer);
}

__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 a, float3 b)
{
    return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

}  // namespace mpcd_gb
