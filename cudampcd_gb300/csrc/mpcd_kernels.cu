// Kernels of the GB300 MPCD step.
//
// One launch of step_kernel completes step k of every box: for each cell it
// stages the cell's bucket (the particles as they enter collision k: streamed
// and shifted) in shared memory with bulk (TMA) copies, collides them (SRD or
// extended MPC), undoes the grid shift, accumulates the lab-grid sample if
// asked, streams each particle for step k+1 and scatters it into the bucket of
// the cell it then occupies (the other parity).  The post-collision state the
// reference exposes between steps is never stored: the getters recompute it by
// replaying the last collision from its (still intact) input buckets.
//
// Reference path being replaced: translateParticles (simulation_kernels.cu:65-143),
// srdCollision (srd_collision_strategy.cu:12-157), ext::fusedCollision
// (extended_collision_strategy.cu:17-332), the counting sort (sort_particles.cu)
// and the sampling kernels (simulation_kernels.cu:150-230); the arithmetic
// follows the CPU backend (cpu_backend/simulation_functions.cpp:38-406).
#include <algorithm>
#include <cstdio>
#include <mutex>

#include "mpcd_device.cuh"
#include "mpcd_kernels.h"
#include "mpcd_gb.h"

namespace mpcd_gb {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint64_t kWaitLimitNs = 2000000000ull;   // 2 s bound on any wait

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// As mbar_try_wait, but the thread may sleep up to `ns` nanoseconds in the
// barrier instead of spinning.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t ns)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
        : "memory");
    return ok != 0;
}

// Wait for the phase with the given parity; false after kWaitLimitNs.
__device__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity)
{
    if (mbar_try_wait_sleep(bar, parity, 1000000u)) return true;
    const uint64_t t0 = globaltimer();
    while (true) {
        if (mbar_try_wait_sleep(bar, parity, 1000000u)) return true;
        if (globaltimer() - t0 > kWaitLimitNs) return false;
    }
}

// Bulk copy global -> shared (16-byte aligned, size a multiple of 16), completing on bar.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One bucket slot (32 bytes, a full sector) with a single 256-bit store.
__device__ __forceinline__ void store_slot(Slot* dst, float4 p, float4 v)
{
    asm volatile("st.global.v8.f32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"l"(dst), "f"(p.x), "f"(p.y), "f"(p.z),
                 "f"(p.w), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w)
                 : "memory");
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Exclusive scan of one value per thread (blockDim == kThreads), total returned.
__device__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_tot, uint32_t& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < kThreads / 32 ? warp_tot[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < kThreads / 32) warp_tot[lane] = wi - w;
        if (lane == kThreads / 32 - 1) warp_tot[kThreads / 32] = wi;
    }
    __syncthreads();
    const uint32_t excl = incl - v + warp_tot[warp];
    total = warp_tot[kThreads / 32];
    __syncthreads();
    return excl;
}

__device__ __forceinline__ int box_of_particle(const BoxDesc* boxes, int nboxes, uint64_t id)
{
    int lo = 0, hi = nboxes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (boxes[mid].dense_base <= id) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Claim a slot in `count[key]` for every active lane; lanes that share a key
// are served by one atomic (warp-aggregated).  Returns the slot.
__device__ __forceinline__ uint32_t claim_slot(uint32_t* count, uint32_t key, bool active)
{
    // idle lanes share a key no cell has, so that the whole warp takes one path
    const unsigned peers = __match_any_sync(kFull, active ? key : 0xFFFFFFFFu);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (active && (int)(threadIdx.x & 31) == leader) base = atomicAdd(count + key, (uint32_t)__popc(peers));
    base = __shfl_sync(kFull, base, leader);
    return base + (uint32_t)__popc(peers & lanemask_lt());
}

// Fold one step's sample of lab cell c into the FP64 running sums: the cell's mean
// velocity (0 for an empty cell, as averageReduceOnly) and its count, snapshot or
// accumulate (cpu_backend.cpp:189-211), and clear the step's sums.
__device__ __forceinline__ void fold_sample(float4* samp, SampleAcc* acc, uint64_t c, int snapshot,
                                            uint32_t* lab_count)
{
    const float4 s = samp[c];
    if (lab_count) lab_count[c] = (uint32_t)s.w;   // adjoint tape: particles sampled in the cell
    float mx = s.x, my = s.y, mz = s.z;
    if (s.w > 0.0f) {
        const float inv = 1.0f / s.w;
        mx *= inv; my *= inv; mz *= inv;
    }
    SampleAcc r = snapshot ? SampleAcc{0, 0, 0, 0} : acc[c];
    r.n += (double)s.w;
    r.vx += (double)mx;
    r.vy += (double)my;
    r.vz += (double)mz;
    acc[c] = r;
    samp[c] = make_float4(0, 0, 0, 0);
}

// Accumulate (v, 1) into samp[lab] for every active lane: one vector atomic
// (red.global.add.v4.f32) per particle.
__device__ __forceinline__ void sample_add(float4* samp, uint32_t lab, float3 v, bool active)
{
    if (active) atomicAdd(samp + lab, make_float4(v.x, v.y, v.z, 1.0f));
}

// A particle that found the bucket of cell `key` full: into the overflow list of
// the next step, chained to its cell (overflow_select_kernel walks the chain).
__device__ __forceinline__ void push_overflow(const StepArgs& a, uint32_t key, float4 xp, float4 vp)
{
    atomicAdd(&a.state->overflow_total, 1ull);
    const unsigned q = atomicAdd(&a.state->ov_count[a.ov_out_slot], 1u);
    if (q < a.ov_cap) {
        a.ov_out_pos[q] = xp;
        a.ov_out_vel[q] = vp;
        a.ov_next_out[q] = atomicExch(a.ov_head_out + key, q);
    } else {
        atomicOr(&a.state->error_flags, kErrOverflowListFull);
    }
}

// Put one particle (already streamed and shifted for the next collision, in
// cell `key`) into its bucket, or into the overflow list when the bucket is full.
// pos.w = kNoExt: a cell the selection does not reach keeps reading its bucket.
__device__ __forceinline__ void store_particle(const StepArgs& a, const BoxDesc& b, float3 xs, float3 vs, uint32_t id,
                                               uint32_t key, bool active)
{
    const uint32_t slot = claim_slot(a.out_count, key, active);
    const float4 xp = make_float4(xs.x, xs.y, xs.z, __uint_as_float(kNoExt));
    const float4 vp = make_float4(vs.x, vs.y, vs.z, __uint_as_float(id));
    // the slot's index in 32 bits: every bucket slot index is below 2^32 (the engine checks)
    const uint32_t index = (uint32_t)b.slot_base + (key - b.cell_base) * b.depth + slot;
    if (active && slot < b.depth) store_slot(a.out_slots + index, xp, vp);
    if (__builtin_expect(active && slot >= b.depth, 0)) push_overflow(a, key, xp, vp);
}

// The colliding particles of box-local cell `local` (raw count `raw`): returns
// their number, with src at the first of them -- the cell's bucket, or, when the
// cell received more than its depth, the extension slots that
// overflow_select_kernel filled (offset in pos.w of the first bucket slot).  A
// cell without an extension (the selection ran out of room, kErrExtensionFull)
// collides the bucket's depth particles; its list entries stay untaken and skip
// the collision, so that every particle is still moved exactly once.
__device__ __forceinline__ uint32_t cell_source(const StepArgs& a, const BoxDesc& b, const Slot* slots,
                                                uint32_t local, uint32_t raw, const Slot*& src)
{
    src = slots + b.slot_base + (uint64_t)local * b.depth;
    if (raw <= b.depth) return raw;
    const uint32_t m = min(raw, b.cap);
    const uint32_t off = __float_as_uint(src->pos.w);
    if (off > a.ext_cap - m) return b.depth;
    src = slots + a.total_slots + off;
    return m;
}

// ------------------------------------------------------------------ draws

// SRD rotation axis of cell `ref` (box-local reference index) at `step`: uniform on the sphere.
__device__ __forceinline__ float3 srd_axis_philox(const BoxDesc& b, uint64_t step, uint32_t ref)
{
    const uint4 o = draw(b, step, kAxis, ref, 0);
    const float z = 1.0f - 2.0f * u01(o.x);
    const float rho = sqrtf(fmaxf(0.0f, 1.0f - z * z));
    float s, c;
    sincospif(2.0f * u01(o.y), &s, &c);
    return make_float3(rho * c, rho * s, z);
}

// Velocity of wall ghost j of cell `ref` (Maxwell-Boltzmann, sqrt(T) per component).
__device__ __forceinline__ float3 ghost_velocity(const BoxDesc& b, uint64_t step, uint32_t ref, uint32_t j)
{
    const uint4 o = draw(b, step, kGhost, ref, 2 * j + 1);
    float g0, g1, g2, g3;
    box_muller(o.x, o.y, g0, g1);
    box_muller(o.z, o.w, g2, g3);
    return make_float3(g0 * b.tv, g1 * b.tv, g2 * b.tv);
}

// Total velocity of the g wall ghosts of cell `ref` for the SRD collision, which
// uses the ghosts only through their sum: g independent Maxwell-Boltzmann
// velocities sum to one Gaussian of variance g T per component, drawn here once
// per cell (the reference draws each ghost, srd_collision_strategy.cu:79-94; the
// extended collision, which uses each ghost's position, still draws them one by one).
__device__ __forceinline__ float3 ghost_sum_velocity(const BoxDesc& b, uint64_t step, uint32_t ref, uint32_t g)
{
    const uint4 o = draw(b, step, kGhostSum, ref, 0);
    float g0, g1, g2, g3;
    box_muller(o.x, o.y, g0, g1);
    box_muller(o.z, o.w, g2, g3);
    const float sc = sqrtf((float)g) * b.tv;
    return make_float3(g0 * sc, g1 * sc, g2 * sc);
}

// SRD cell sums are exact: each velocity component is rounded to a multiple of
// 2^-24 and the multiples are summed as 64-bit integers, so the sum depends
// neither on the order of the bucket (the arrival order of the claims) nor on
// how it is split.  round(v 2^24) of any v, converted to 64 bits:
constexpr float kFixScale = 16777216.0f;   // 2^24
__device__ __forceinline__ long long fixed24(float v) { return __float2ll_rn(v * kFixScale); }

// The same value through the 32-bit conversion (the 64-bit one runs on the
// narrow FP64 pipe); exact while |v| < 32.  The largest |v| converted is tracked
// in `mx` (one max with an absolute-value operand) so that a caller can redo its
// sums with fixed24 when it reaches 32: then round(v 2^24) >= 2^29 in magnitude,
// or the conversion saturated (an infinity); a NaN converts to 0 and is ignored.
__device__ __forceinline__ int fixed24_narrow(float v, float& mx)
{
    mx = fmaxf(mx, fabsf(v));
    return __float2int_rn(v * kFixScale);
}
constexpr float kNarrowLimit = 32.0f;   // below it, four narrow values still sum in 32 bits

// Mean velocity of a cell of n > 1 entries (particles and ghosts) from its exact sums.
__device__ __forceinline__ float3 srd_mean(long long sx, long long sy, long long sz, uint32_t n)
{
    const float inv = 1.0f / (float)n;
    return make_float3((__ll2float_rn(sx) * 0x1p-24f) * inv, (__ll2float_rn(sy) * 0x1p-24f) * inv,
                       (__ll2float_rn(sz) * 0x1p-24f) * inv);
}

// SRD collision of one particle of a cell of more than one entry (srd_collision,
// simulation_functions.cpp:108-202): v' = u + v_par + cos a v_perp + sin a (v_perp x axis)
// with fused multiply-adds (compared to 1e-5, not bit-exactly), then the grid shift
// undone, x = pbc(x - s) (the staged x is wrapped and |s| <= 1/2), and the drag.
__device__ __forceinline__ void srd_collide(const BoxDesc& b, float3 s, float3 mean, float3 axis, float3& x, float3& v)
{
    const float3 vr = make_float3(v.x - mean.x, v.y - mean.y, v.z - mean.z);
    const float vd = __fmaf_rn(vr.x, axis.x, __fmaf_rn(vr.y, axis.y, vr.z * axis.z));
    const float3 vpara = make_float3(axis.x * vd, axis.y * vd, axis.z * vd);
    const float3 vperp = make_float3(vr.x - vpara.x, vr.y - vpara.y, vr.z - vpara.z);
    const float3 cr = make_float3(__fmaf_rn(vperp.y, axis.z, -(vperp.z * axis.y)),
                                  __fmaf_rn(vperp.z, axis.x, -(vperp.x * axis.z)),
                                  __fmaf_rn(vperp.x, axis.y, -(vperp.y * axis.x)));
    v = make_float3(__fmaf_rn(b.sin_a, cr.x, __fmaf_rn(b.cos_a, vperp.x, vpara.x)) + mean.x,
                    __fmaf_rn(b.sin_a, cr.y, __fmaf_rn(b.cos_a, vperp.y, vpara.y)) + mean.y,
                    __fmaf_rn(b.sin_a, cr.z, __fmaf_rn(b.cos_a, vperp.z, vpara.z)) + mean.z);
    x = pbc_near(b, make_float3(x.x - s.x, x.y - s.y, x.z - s.z));
    v.x += b.drag_dt;
}

template <bool TABLE>
struct Draws;

template <>
struct Draws<false> {   // Philox (production)
    __device__ static uint32_t ghost_count(const StepArgs&, const BoxDesc& b, uint64_t step, uint32_t ref,
                                           float shift, bool layer, bool sign)
    {
        uint32_t g = 0;
        uint4 o = make_uint4(0, 0, 0, 0);
        for (uint32_t i = 0; i < b.n; ++i) {
            if ((i & 3u) == 0) o = draw(b, step, kGhostCount, ref, i >> 2);
            const uint32_t u = (i & 3u) == 0 ? o.x : (i & 3u) == 1 ? o.y : (i & 3u) == 2 ? o.z : o.w;
            if ((u01(u) > shift) ^ layer ^ sign) ++g;
        }
        return g;
    }
    __device__ static void ghost(const StepArgs&, const BoxDesc& b, uint64_t step, uint32_t ref, uint32_t j,
                                 float3 centre, float shift, bool layer, bool sign, float3& x, float3& v)
    {
        const uint4 o = draw(b, step, kGhost, ref, 2 * j);
        const float uz = u01(o.z);
        const float z = (layer ^ sign) ? shift * uz : shift + (1.0f - shift) * uz;
        x = make_float3((u01(o.x) - 0.5f) + centre.x, (u01(o.y) - 0.5f) + centre.y, (z - 0.5f) + centre.z);
        v = ghost_velocity(b, step, ref, j);
    }
    __device__ static float3 srd_axis(const StepArgs&, const BoxDesc& b, uint64_t step, uint32_t ref)
    {
        return srd_axis_philox(b, step, ref);
    }
    __device__ static float3 ext_axis(const StepArgs& a, const BoxDesc& b, uint64_t step, uint32_t ref, float& gate)
    {
        const uint4 o = draw(b, step, kAxis, ref, 0);
        const uint32_t sel = (o.x >> 1) % 13u;
        float3 ax = make_float3(a.ext_axis[sel][0], a.ext_axis[sel][1], a.ext_axis[sel][2]);
        if ((o.y >> 1) & 1u) ax = make_float3(-ax.x, -ax.y, -ax.z);
        gate = u01(o.z);
        return ax;
    }
    __device__ static float thermal(const StepArgs&, const BoxDesc& b, uint64_t step, uint32_t ref, uint32_t i)
    {
        const uint4 o = draw(b, step, kThermal, ref, i >> 2);
        float g0, g1;
        if (((i & 3u) >> 1) == 0) box_muller(o.x, o.y, g0, g1);
        else box_muller(o.z, o.w, g0, g1);
        return (i & 1u) ? g1 : g0;
    }
};

template <>
struct Draws<true> {    // injected tables (test hook)
    __device__ static uint32_t ghost_count(const StepArgs& a, const BoxDesc&, uint64_t, uint32_t ref, float, bool,
                                           bool)
    {
        return a.draws.ghost_count[ref];
    }
    __device__ static void ghost(const StepArgs& a, const BoxDesc&, uint64_t, uint32_t ref, uint32_t j, float3,
                                 float, bool, bool, float3& x, float3& v)
    {
        const float* p = a.draws.ghost_pos + ((size_t)ref * a.draws.gmax + j) * 3;
        const float* q = a.draws.ghost_vel + ((size_t)ref * a.draws.gmax + j) * 3;
        x = make_float3(p[0], p[1], p[2]);
        v = make_float3(q[0], q[1], q[2]);
    }
    __device__ static float3 srd_axis(const StepArgs& a, const BoxDesc&, uint64_t, uint32_t ref)
    {
        const float* p = a.draws.axis + (size_t)ref * 3;
        return make_float3(p[0], p[1], p[2]);
    }
    __device__ static float3 ext_axis(const StepArgs& a, const BoxDesc&, uint64_t, uint32_t ref, float& gate)
    {
        const float* p = a.draws.axis + (size_t)ref * 3;
        gate = a.draws.gate_u[ref];
        return make_float3(p[0], p[1], p[2]);
    }
    __device__ static float thermal(const StepArgs& a, const BoxDesc&, uint64_t, uint32_t ref, uint32_t i)
    {
        return a.draws.gauss[(size_t)ref * a.draws.pmax + i];
    }
};

// SymmetricMatrix::inverse(tolerance) (common/mechanic.hpp:52-79); m = {xx,yy,zz,xy,xz,yz}
__device__ __forceinline__ void sym_inverse(const float m[6], float tol, float o[6])
{
    const float xx = m[0], yy = m[1], zz = m[2], xy = m[3], xz = m[4], yz = m[5];
    float det = xx * (yy * zz - yz * yz) + xz * (2 * xy * yz - yy * xz) - (xy * xy * zz);
    if (det < 0) det = 0;
    if (det > tol) {
        const float inv = 1 / det;
        o[0] = (yy * zz - yz * yz) * inv;
        o[1] = (xx * zz - xz * xz) * inv;
        o[2] = (xx * yy - xy * xy) * inv;
        o[3] = (xz * yz - zz * xy) * inv;
        o[4] = (xy * yz - yy * xz) * inv;
        o[5] = (xy * xz - xx * yz) * inv;
    } else {
        const float tr = xx + yy + zz;
        if (tr > tol) {
            const float s = 4 / (tr * tr);
            for (int k = 0; k < 6; ++k) o[k] = m[k] * s;
        } else {
            for (int k = 0; k < 6; ++k) o[k] = 0.0f;
        }
    }
}

// ------------------------------------------------------------------ step kernel
//
// One CTA processes tiles of consecutive cells (storage order).  Per tile:
//   counts (prefetched one tile ahead) and ghost counts, a group of G threads
//   per cell (G = kThreads / tile cells);
//   bulk (TMA) copies of every cell's bucket into shared memory + ghosts;
//   stream step k (recomputed, bit-identical to the scatter that keyed it);
//   per-cell collision quantities, one group per cell;
//   per particle: finish the collision, unshift, drag, sample, stream step
//   k+1 to find the next cell; claim bucket slots with warp-aggregated atomics
//   (all issued before any result is used) and write the particles out.
// Order within a cell is canonical: ascending particle id, i.e. the stable sort
// of the id-ordered particle array by cell.  SRD cell sums are exact 64-bit
// fixed-point sums (independent of summation order, hence deterministic and
// splittable over a group); the extended collision walks each cell in id
// order, as the reference walks it in index order.

constexpr uint32_t kNoKey = 0xFFFFFFFFu;
constexpr uint32_t kGhostFlag = 0x8000u;   // s_cell entries of ghost particles (tile cells < 2^15)
constexpr int kMaxPerThread = 8;   // particle buffer <= kMaxPerThread * kThreads

// Shared memory of one CTA, carved from the dynamic allocation:
//   particles: slots (pos, vel: the bucket layout, so that a cell is one bulk
//              copy; after the collision pass pos.w holds the next cell key),
//              cell (u16)
//   extended only: rank (u16), stable index (u16)
//   cells: cnt, ng, off, goff (u32, T + 1 each), c0, c1 (float4, T each)
//   extended only: omega (float4, T)
struct TileLayout {
    Slot* buf;
    uint16_t* cell;
    uint16_t* rank;
    uint16_t* inv;
    uint32_t *cnt, *ng, *off, *goff;
    float4 *c0, *c1, *omega;
};

__host__ __device__ inline size_t tile_smem_bytes(uint32_t pbuf, uint32_t cells, int algorithm)
{
    const size_t per_particle = 16 + 16 + 2 + (algorithm ? 4 : 0);
    size_t bytes = (size_t)pbuf * per_particle;
    bytes = (bytes + 15) / 16 * 16 + 4 * (size_t)(cells + 1) * 4;
    bytes = (bytes + 15) / 16 * 16 + (size_t)cells * 16 * (algorithm ? 3 : 2);
    return bytes;
}

__device__ inline TileLayout carve(unsigned char* base, uint32_t pbuf, uint32_t cells, int algorithm)
{
    TileLayout t;
    t.buf = reinterpret_cast<Slot*>(base);
    t.cell = reinterpret_cast<uint16_t*>(t.buf + pbuf);
    t.rank = t.cell + pbuf;
    t.inv = t.rank + (algorithm ? pbuf : 0);
    size_t at = (size_t)pbuf * (16 + 16 + 2 + (algorithm ? 4 : 0));
    at = (at + 15) / 16 * 16;
    uint32_t* u = reinterpret_cast<uint32_t*>(base + at);
    t.cnt = u;
    t.ng = u + (cells + 1);
    t.off = u + 2 * (cells + 1);
    t.goff = u + 3 * (cells + 1);
    at = (at + 4 * (size_t)(cells + 1) * 4 + 15) / 16 * 16;
    t.c0 = reinterpret_cast<float4*>(base + at);
    t.c1 = t.c0 + cells;
    t.omega = t.c1 + cells;
    return t;
}

// Entry of `tile`: {first global cell, cells | tile cells << 16, box, 0}; past
// the last tile {0, tile cells of the launch << 16, 0, 0}.  A single box computes
// it from the kernel parameters; an ensemble reads the host-built table (one
// load instead of a search over the boxes).
template <bool SINGLE>
__device__ __forceinline__ uint4 tile_entry(const StepArgs& a, uint32_t tile)
{
    if (tile >= a.num_tiles) return make_uint4(0u, a.boxes_tile_cells << 16, 0u, 0u);
    if (!SINGLE) return __ldg(reinterpret_cast<const uint4*>(a.tile_info) + tile);
    const BoxDesc& b = a.box0;
    const uint32_t c0 = tile * b.tile_cells;
    return make_uint4(b.cell_base + c0, min(b.tile_cells, b.C - c0) | (b.tile_cells << 16), 0u, 0u);
}

// Count of cell `c` of a tile (first thread of the cell's group); issued one
// tile ahead so its latency hides.  Outside a replay it also clears the same
// cell of the counts of step k-1, which step k+1 will fill.
__device__ __forceinline__ uint32_t fetch_count(const StepArgs& a, uint32_t first, uint32_t nc, uint32_t c,
                                                bool leader)
{
    if (!leader || c >= nc) return 0;
    const uint32_t g = first + c;
    if (!a.replay) a.zero_count[g] = 0;
    return a.in_count[g];
}

// Overflow particles of step k past their cell's colliding set (the cap lowest
// ids of a cell collide; the selection marked the entries it moved to the cell's
// extension kTakenId): as in the reference, they skip the collision and keep the
// unshifted position pbc(pbc(x + s) - s) (simulation_functions.cpp:90-93).
__device__ void overflow_pass(const StepArgs& a, uint64_t step)
{
    const uint32_t n = min(a.state->ov_count[a.ov_in_slot], a.ov_cap);
    for (uint32_t base = 0; base < n; base += kThreads) {
        const uint32_t q = base + threadIdx.x;
        const float4 w = q < n ? a.ov_in_vel[q] : make_float4(0, 0, 0, 0);
        const bool active = q < n && __float_as_uint(w.w) != kTakenId;
        int bi = 0;
        uint32_t id = 0, key = 0;
        float3 x = make_float3(0, 0, 0), v = x, xs = x, vs = x;
        if (active) {
            const float4 p = a.ov_in_pos[q];
            id = __float_as_uint(w.w);
            bi = box_of_particle(a.boxes, a.nboxes, id);
            const BoxDesc& b = a.boxes[bi];
            const float3 s = grid_shift(b, bi, step, a.state);
            x = pbc(b, make_float3(p.x - s.x, p.y - s.y, p.z - s.z));   // post-step state
            v = make_float3(w.x, w.y, w.z);
            if (a.replay) {
                const uint64_t i3 = 3 * (uint64_t)id;
                a.dense_pos[i3] = x.x; a.dense_pos[i3 + 1] = x.y; a.dense_pos[i3 + 2] = x.z;
                a.dense_vel[i3] = v.x; a.dense_vel[i3 + 1] = v.y; a.dense_vel[i3 + 2] = v.z;
            } else {
                vs = v;
                xs = stream_shift(b, x, vs, grid_shift(b, bi, step + 1, a.state));
                key = b.cell_base + storage_index(b, cell_of_wrapped(b, xs));
                if (a.pressure && b.wall_z && vs.z != v.z)   // bounce-back: 2 |v_z| outward
                    atomicAdd(&a.state->wall_impulse[v.z > 0.0f ? 1 : 0], 2.0 * fabs((double)v.z));
                if (a.tape_key) {
                    const bool bounced = vs.x != v.x || vs.y != v.y || vs.z != v.z;
                    a.tape_key[id] = kTapeNone;
                    a.tape_lab[id] = (b.cell_base + storage_index(b, cell_of_wrapped(b, x))) | (bounced ? kTapeBounce : 0u);
                }
            }
        }
        if (a.replay) continue;
        const BoxDesc& b = a.boxes[bi];
        if (a.sample) {
            const uint32_t lab = active ? b.cell_base + storage_index(b, cell_of_wrapped(b, x)) : 0;
            sample_add(a.samp, lab, v, active);
        }
        store_particle(a, b, xs, vs, id, key, active);
    }
}

constexpr int kExtLanes = 4;   // lanes per cell of the extended collision (tiles of <= 64 cells)

// log2 of the threads per cell, G = 256 / tile cells (tile cells a power of two, 8..128).
__device__ __forceinline__ uint32_t group_log2(uint32_t tile_cells) { return 8u - (31u - __clz(tile_cells)); }

// Sum over the G lanes of a cell group (G a power of two dividing 32).
template <class T>
__device__ __forceinline__ T group_sum(T v, uint32_t G)
{
    for (uint32_t o = 1; o < G; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

// 4 CTAs of 256 threads per SM: 64 registers, and at most about 56 KB of shared
// memory each (SRD: a 1408-particle buffer with 128-cell tiles; extended, whose
// tile carries two more arrays: 1344 particles with 64-cell tiles)
template <int ALGO, bool TABLE, bool SINGLE, bool REPLAY>
__global__ void __launch_bounds__(kThreads, 4) step_kernel(const StepArgs a, uint32_t pbuf)
{
    using D = Draws<TABLE>;
    extern __shared__ __align__(128) unsigned char dyn[];
    __shared__ uint32_t warp_tot[kThreads / 32 + 1];
    __shared__ uint64_t bar;
    __shared__ __align__(16) BoxDesc sbox;
    __shared__ uint32_t s_armed;   // the tile's copies were armed by the scan warp
    __shared__ float3 sshift[2];
    const uint32_t tcells = a.boxes_tile_cells;   // the largest tile of the launch (boxes may use smaller ones)
    const TileLayout L = carve(dyn, pbuf, tcells, ALGO);
    Slot* const s_buf = L.buf;
    uint16_t* const s_cell = L.cell;
    uint16_t* const s_rank = L.rank;   // extended only
    uint16_t* const s_inv = L.inv;     // extended only

    const int tid = threadIdx.x;
    const int lane = tid & 31;
    if (tid == 0) mbar_init(&bar);
    __syncthreads();
    uint32_t phase = 0;
    const uint64_t step = a.step_base ? *a.step_base + a.step : a.step;   // graph replays read the base
    float imp[2] = {0.0f, 0.0f};   // pressure estimator: this thread's outward wall impulses

    if (blockIdx.x == 0) {
        if (tid == 0 && !a.replay) a.state->ov_count[a.ov_zero_slot] = 0;   // list of step k-1, refilled by step k+1
        overflow_pass(a, step);
    }

    // the tile after the current one (tile_entry): its entry is read by one
    // thread (kLocator) while the current tile's ghosts are counted, its counts by
    // the cell leaders after the scan (a group of G = 256 / tile cells threads per
    // cell; a box's tile size sets G).  Two entries alternate, so that the write
    // for the next tile never meets a read of the current one.
    constexpr int kLocator = 64;   // warp 2: not the scan warp, not the box-switch threads
    __shared__ uint4 s_next[2];
    if (tid == kLocator) s_next[0] = tile_entry<SINGLE>(a, blockIdx.x);
    __syncthreads();
    uint32_t next_raw;
    {
        const uint32_t lg = group_log2(s_next[0].y >> 16);
        next_raw = fetch_count(a, s_next[0].x, s_next[0].y & 0xFFFFu, (uint32_t)tid >> lg, (tid & ((1 << lg) - 1)) == 0);
    }
    int cur_box = -1;   // box of the previous tile (every thread keeps the same value)
    uint32_t par = 0;   // s_next[par]: the current tile's entry
    for (uint32_t tile = blockIdx.x; tile < a.num_tiles; tile += gridDim.x, par ^= 1u) {
        const int bi = SINGLE ? 0 : (int)s_next[par].z;   // located while the previous tile was processed
        if (bi != cur_box) {   // box and its grid shifts change only between boxes: copy and
            cur_box = bi;      // draw them on separate warps
            const BoxDesc* bp = SINGLE ? &a.box0 : a.boxes + bi;
            if (!SINGLE && tid < (int)(sizeof(BoxDesc) / 16))
                reinterpret_cast<uint4*>(&sbox)[tid] = __ldg(reinterpret_cast<const uint4*>(bp) + tid);
            if (tid == 32) sshift[0] = grid_shift(*bp, bi, step, a.state);
            if (tid == 96) sshift[1] = grid_shift(*bp, bi, step + 1, a.state);
            __syncthreads();
        }
        // single box: geometry straight from the kernel parameters (constant bank)
        const BoxDesc& b = SINGLE ? a.box0 : sbox;
        const uint32_t lgG = group_log2(b.tile_cells);
        const uint32_t G = 1u << lgG;   // threads per cell of this box's tiles
        const uint32_t my_cell = (uint32_t)tid >> lgG, my_j = (uint32_t)tid & (G - 1u);
        const bool leader = my_j == 0;
        const uint32_t c0 = (tile - b.tile_base) * b.tile_cells;
        const uint32_t nc = min(b.tile_cells, b.C - c0);
        // the next tile's entry: loaded here, stored to shared memory after the
        // ghost counts (its readers all passed the previous tile's last barrier)
        uint4 next_entry = make_uint4(0u, 0u, 0u, 0u);
        if (tid == kLocator) next_entry = tile_entry<SINGLE>(a, tile + gridDim.x);

        const float3 s = sshift[0];
        const float3 sn = sshift[1];
        const float shift_abs = fabsf(s.z);
        const bool sign = s.z > 0;

        // counts (prefetched) and ghost counts, one group per cell
        const uint32_t my_raw = next_raw;   // the cell leader's raw count (it stages the cell)
        uint32_t mine = 0, mine_g = 0;
        {
            uint32_t gpart = 0;
            if (my_cell < nc) {
                const uint3 cc = storage_coords(b, c0 + my_cell);
                bool layer, ghosts;
                wall_layer(b, cc.z, sign, layer, ghosts);
                if (ghosts) {
                    const uint32_t ref = ref_index(b, cc);
                    if (TABLE) {
                        if (leader) gpart = D::ghost_count(a, b, step, ref, shift_abs, layer, sign);
                    } else {
                        for (uint32_t chunk = my_j; 4 * chunk < b.n; chunk += G) {   // 4 uniforms per Philox call
                            const uint4 o = draw(b, step, kGhostCount, ref, chunk);
                            const uint32_t u[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                if (4 * chunk + k < b.n && ((u01(u[k]) > shift_abs) ^ layer ^ sign)) ++gpart;
                        }
                    }
                }
            }
            gpart = group_sum(gpart, G);
            if (leader && my_cell < nc) {
                const Slot* src;
                mine = cell_source(a, b, a.in_slots, c0 + my_cell, my_raw, src);
                mine_g = gpart;
                L.cnt[my_cell] = mine;
                L.ng[my_cell] = mine_g;
            }
        }
        if (tid == kLocator) s_next[par ^ 1u] = next_entry;
        // SRD rotation axes (and the wall side for the pressure estimator) of the
        // tile's cells, one thread per cell; read after the scan's barriers
        if (ALGO == 0) {
            for (uint32_t i = (uint32_t)tid; i < nc; i += kThreads) {
                const uint3 cc = storage_coords(b, c0 + i);
                const float3 ax = D::srd_axis(a, b, step, ref_index(b, cc));
                uint32_t side = 0;
                if (a.pressure && b.wall_z) side = cc.z <= 1u ? 1u : (cc.z + 2u >= (uint32_t)b.L[2] ? 2u : 0u);
                L.c1[i] = make_float4(ax.x, ax.y, ax.z, __uint_as_float(side));
            }
        }
        // offsets of the tile's cells: one warp scans (particles << 16 | ghosts) of up
        // to 128 cells, 4 per lane (a tile holds fewer than 2^16 of either)
        __syncthreads();
        if (tid < 32) {
            uint32_t v[4], run = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t c = 4 * (uint32_t)tid + k;
                v[k] = c < nc ? ((L.cnt[c] + L.ng[c]) << 16) | L.ng[c] : 0u;
                run += v[k];
            }
            uint32_t incl = run;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t t = __shfl_up_sync(kFull, incl, d);
                if (tid >= d) incl += t;
            }
            uint32_t at = incl - run;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const uint32_t c = 4 * (uint32_t)tid + k;
                if (c < nc) {
                    L.off[c] = at >> 16;
                    L.goff[c] = at & 0xFFFFu;
                }
                at += v[k];
            }
            if (tid == 31) {
                L.off[nc] = incl >> 16;
                L.goff[nc] = incl & 0xFFFFu;
                // the whole tile fits the buffer (the common case): arm its copies here,
                // which spares the sub-tile loop a barrier
                const uint32_t total = incl >> 16, real = total - (incl & 0xFFFFu);
                s_armed = total <= pbuf;
                if (total <= pbuf && real) {
                    fence_proxy_async();
                    mbar_arrive_expect_tx(&bar, 32u * real);
                }
            }
        }
        __syncthreads();
        {
            const uint4 e = s_next[par ^ 1u];
            const uint32_t lg = group_log2(e.y >> 16);   // the next tile's groups
            next_raw = fetch_count(a, e.x, e.y & 0xFFFFu, (uint32_t)tid >> lg, (tid & ((1 << lg) - 1)) == 0);
        }

        // sub-tiles of consecutive cells whose particles fit the buffer
        uint32_t i0 = 0;
        while (i0 < nc) {
            uint32_t lo = i0 + 1, hi = nc;   // largest i1 with off[i1] - off[i0] <= pbuf
            if (L.off[nc] - L.off[i0] <= pbuf) lo = nc;   // the common case: the rest fits
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (L.off[mid] - L.off[i0] <= pbuf) lo = mid; else hi = mid - 1;
            }
            const uint32_t i1 = lo;
            const uint32_t pbase = L.off[i0];
            const uint32_t np = L.off[i1] - pbase;
            if (np > pbuf) {   // impossible while 5n <= pbuf (checked on the host)
                if (tid == 0) atomicOr(&a.state->error_flags, kErrKeyMismatch);
                return;
            }

            // stage real particles: one bulk copy per cell
            const uint32_t real_bytes = 32u * (np - (L.goff[i1] - L.goff[i0]));
            if (!(s_armed && i0 == 0)) {   // not armed by the scan warp: this sub-tile arms its own
                if (tid == 0 && real_bytes) {
                    fence_proxy_async();
                    mbar_arrive_expect_tx(&bar, real_bytes);
                }
                __syncthreads();
            }
            const bool in_sub = my_cell >= i0 && my_cell < i1;
            if (in_sub) {
                const uint32_t i = my_cell;
                const uint32_t n = L.cnt[i];
                const uint32_t o = L.off[i] - pbase, e = L.off[i + 1] - pbase;
                if (leader && n) {
                    const Slot* src;
                    cell_source(a, b, a.in_slots, c0 + i, my_raw, src);
                    fence_proxy_async();
                    bulk_g2s(s_buf + o, src, n * 32u, &bar);
                }
                for (uint32_t p = o + my_j; p < e; p += G)   // cell of the entry, kGhostFlag on ghosts
                    s_cell[p] = (uint16_t)(i | (p - o >= n ? kGhostFlag : 0u));
            }
            // ghosts, one thread per ghost (overlaps the copies)
            {
                const uint32_t gb = L.goff[i0], ge = L.goff[i1];
                for (uint32_t q = gb + tid; q < ge; q += kThreads) {
                    uint32_t lo2 = i0, hi2 = i1 - 1;   // cell with goff[i] <= q < goff[i+1]
                    while (lo2 < hi2) {
                        const uint32_t mid = (lo2 + hi2 + 1) >> 1;
                        if (L.goff[mid] <= q) lo2 = mid; else hi2 = mid - 1;
                    }
                    const uint32_t i = lo2, j = q - L.goff[i];
                    const uint3 cc = storage_coords(b, c0 + i);
                    bool layer, ghosts;
                    wall_layer(b, cc.z, sign, layer, ghosts);
                    float3 gx, gv;
                    if (ALGO == 0 && !TABLE) {   // SRD: the ghosts' summed velocity on the first, zero on the rest
                        gx = cell_centre(b, cc);
                        gv = j == 0 ? ghost_sum_velocity(b, step, ref_index(b, cc), L.ng[i]) : make_float3(0, 0, 0);
                    } else {
                        D::ghost(a, b, step, ref_index(b, cc), j, cell_centre(b, cc), shift_abs, layer, sign, gx, gv);
                    }
                    const uint32_t p = L.off[i] - pbase + L.cnt[i] + j;
                    s_buf[p].pos = make_float4(gx.x, gx.y, gx.z, 0.0f);
                    s_buf[p].vel = make_float4(gv.x, gv.y, gv.z, 0.0f);
                }
            }
            if (real_bytes) {
                int ok = 1;
                if (tid == 0) ok = mbar_wait_bounded(&bar, phase);
                ok = __syncthreads_and(ok);
                if (!ok) {
                    if (tid == 0) {
                        atomicOr(&a.state->error_flags, kErrWaitTimeout);
                        mbar_wait_bounded(&bar, phase);   // let copies in flight land
                    }
                    return;
                }
                mbar_try_wait(&bar, phase);   // completed phase: acquire for every thread
                phase ^= 1u;
            } else {
                __syncthreads();
            }

            // extended: rank of every real particle within its cell by particle id
            if (ALGO == 1) {
                for (uint32_t p = tid; p < np; p += kThreads) {
                    const uint32_t info = s_cell[p];
                    const uint32_t ci = info & ~kGhostFlag;
                    const uint32_t o = L.off[ci] - pbase;
                    const uint32_t n = L.cnt[ci];
                    if (!(info & kGhostFlag)) {
                        const uint32_t id = __float_as_uint(s_buf[p].vel.w);
                        uint32_t rank = 0;
                        for (uint32_t q = 0; q < n; ++q) rank += __float_as_uint(s_buf[o + q].vel.w) < id;
                        s_rank[p] = (uint16_t)rank;
                        s_inv[o + rank] = (uint16_t)p;
                    }
                }
                __syncthreads();
            }

            // Per particle: finish the collision (SRD rotation or extended update), unshift,
            // drag, lab-grid sample, stream step k+1 and find the next cell.  k0 = (mean,
            // n), k1 = (axis or centre of mass, wall side) of the particle's cell ci.
            auto finish = [&](uint32_t p, uint32_t ci, const float4 k0, const float4 k1) {
                const float4 xp = s_buf[p].pos, vp = s_buf[p].vel;
                float3 x = make_float3(xp.x, xp.y, xp.z);
                float3 v = make_float3(vp.x, vp.y, vp.z);
                const uint32_t n = __float_as_uint(k0.w);
                const float3 mean = make_float3(k0.x, k0.y, k0.z);
                bool collided = false;
                if (ALGO == 0) {
                    if (n > 1) {
                        srd_collide(b, s, mean, make_float3(k1.x, k1.y, k1.z), x, v);
                        collided = true;
                    }
                } else {
                    const float4 k2 = L.omega[ci];
                    const uint32_t m = __float_as_uint(k2.w);
                    if (n > 1 && s_rank[p] < m) {
                        const float3 com = make_float3(k1.x, k1.y, k1.z);
                        const float3 omega = make_float3(k2.x, k2.y, k2.z);
                        v.x += mean.x; v.y += mean.y; v.z += mean.z;
                        v.x += b.drag_dt;
                        const float3 cr = cross3(x, omega);
                        v.x -= cr.x; v.y -= cr.y; v.z -= cr.z;
                        // com + x rebuilds the wrapped staged position to within rounding
                        x = pbc_near(b, make_float3((com.x + x.x) - s.x, (com.y + x.y) - s.y, (com.z + x.z) - s.z));
                        collided = true;
                    }
                }
                if (REPLAY) {
                    const uint64_t i3 = 3 * (uint64_t)__float_as_uint(vp.w);
                    a.dense_pos[i3] = x.x; a.dense_pos[i3 + 1] = x.y; a.dense_pos[i3 + 2] = x.z;
                    a.dense_vel[i3] = v.x; a.dense_vel[i3 + 1] = v.y; a.dense_vel[i3 + 2] = v.z;
                    return;
                }
                float3 vn = v;
                const float3 xn = stream_shift(b, x, vn, sn);
                if (a.pressure) {
                    // collision in a wall-layer cell: the ghosts took up minus the real
                    // particles' z momentum change (extended: the leader has subtracted
                    // the participants' momentum before the collision)
                    const uint32_t side = __float_as_uint(k1.w);
                    if (side) {
                        const float sg = side == 1 ? 1.0f : -1.0f;
                        if (ALGO == 0) imp[side - 1] += sg * (v.z - vp.z);
                        else if (collided) imp[side - 1] += sg * v.z;
                    }
                    if (b.wall_z && vn.z != v.z) imp[v.z > 0.0f ? 1 : 0] += 2.0f * fabsf(v.z);   // bounce-back
                }
                const uint32_t next = b.cell_base + storage_index(b, cell_of_wrapped(b, xn));
                s_buf[p].pos = make_float4(xn.x, xn.y, xn.z, __uint_as_float(next));
                s_buf[p].vel = make_float4(vn.x, vn.y, vn.z, vp.w);
                const bool need_lab = a.sample || (ALGO == 0 && a.tape_key);
                const uint32_t lab = need_lab ? b.cell_base + storage_index(b, cell_of_wrapped(b, x)) : 0u;
                if (ALGO == 0 && a.tape_key) {
                    const uint32_t id = __float_as_uint(vp.w);
                    const bool bounced = vn.x != v.x || vn.y != v.y || vn.z != v.z;
                    a.tape_key[id] = n > 1 ? b.cell_base + c0 + ci : kTapeNone;
                    a.tape_lab[id] = lab | (bounced ? kTapeBounce : 0u);
                }
                if (a.sample) sample_add(a.samp, lab, v, true);
            };

            if (ALGO == 0) {
                // SRD: exact velocity sum of each cell (2^-24 fixed point, independent of
                // bucket order; ghosts included), one group per cell
                const uint32_t i = my_cell;
                const uint32_t o = in_sub ? L.off[i] - pbase : 0;
                const uint32_t n = in_sub ? L.cnt[i] + L.ng[i] : 0;
                long long sx = 0, sy = 0, sz = 0, tx = 0, ty = 0, tz = 0;   // two chains (integer: exact)
                uint32_t q = my_j;
                for (; q + G < n; q += 2 * G) {
                    const float4 va = s_buf[o + q].vel, vb = s_buf[o + q + G].vel;
                    sx += fixed24(va.x);
                    sy += fixed24(va.y);
                    sz += fixed24(va.z);
                    tx += fixed24(vb.x);
                    ty += fixed24(vb.y);
                    tz += fixed24(vb.z);
                }
                if (q < n) {
                    const float4 va = s_buf[o + q].vel;
                    sx += fixed24(va.x);
                    sy += fixed24(va.y);
                    sz += fixed24(va.z);
                }
                sx += tx;
                sy += ty;
                sz += tz;
                sx = group_sum(sx, G);
                sy = group_sum(sy, G);
                sz = group_sum(sz, G);
                if (in_sub && leader) {
                    const float3 mean = n > 1 ? srd_mean(sx, sy, sz, n) : make_float3(0, 0, 0);
                    L.c0[i] = make_float4(mean.x, mean.y, mean.z, __uint_as_float(n));   // axis: c1, drawn per tile
                    if (!REPLAY && a.tape_ncell) a.tape_ncell[b.cell_base + c0 + i] = n > 1 ? n : 0u;
                }
            } else {
                // Extended: the first kExtLanes threads of the cell's group walk the
                // participants in particle-id order (thread j takes ranks j, j + 4, ...) and
                // reduce with shuffles in a fixed tree, so the arithmetic does not depend on
                // the tiling (G >= 4 always: extended tiles hold at most 64 cells); every
                // lane runs every reduction (idle lanes and cells that do not collide add
                // zeros), only stores depend on the cell.
                const bool ext_lane = my_j < (uint32_t)kExtLanes;
                const uint32_t i = my_cell;
                const uint32_t o = in_sub ? L.off[i] - pbase : 0, cnt = in_sub ? L.cnt[i] : 0;
                const uint32_t g = in_sub ? L.ng[i] : 0;
                const uint3 cc = storage_coords(b, c0 + (in_sub ? i : 0));
                const uint32_t ref = ref_index(b, cc);
                const uint32_t n = in_sub ? min(cnt + g, b.cap) : 0;
                const uint32_t m = n - min(g, n);   // real participants (lowest ids)
                const bool live = in_sub && n > 1;
                uint32_t side = 0;   // wall layer of the cell for the pressure estimator: 1 bottom, 2 top
                if (!REPLAY && a.pressure && b.wall_z && in_sub)
                    side = cc.z <= 1u ? 1u : (cc.z + 2u >= (uint32_t)b.L[2] ? 2u : 0u);
                const float3 centre = cell_centre(b, cc);
                float gate = 1.0f;
                float3 axis = make_float3(0, 0, 1);
                if (live) axis = D::ext_axis(a, b, step, ref, gate);
                auto at = [&](uint32_t k) -> uint32_t { return k < m ? s_inv[o + k] : o + cnt + (k - m); };
                // centre of mass and mean velocity
                float3 com = make_float3(0, 0, 0), mean = make_float3(0, 0, 0);
                float real_vz = 0.0f;
                for (uint32_t k = my_j; ext_lane && live && k < n; k += kExtLanes) {
                    const uint32_t p = at(k);
                    const float4 xp = s_buf[p].pos, vp = s_buf[p].vel;
                    com.x += (xp.x - centre.x); com.y += (xp.y - centre.y); com.z += (xp.z - centre.z);
                    mean.x += vp.x; mean.y += vp.y; mean.z += vp.z;
                    if (k < m) real_vz += vp.z;
                }
                com = make_float3(group_sum(com.x, kExtLanes), group_sum(com.y, kExtLanes), group_sum(com.z, kExtLanes));
                mean = make_float3(group_sum(mean.x, kExtLanes), group_sum(mean.y, kExtLanes), group_sum(mean.z, kExtLanes));
                real_vz = group_sum(real_vz, kExtLanes);
                if (live && side && leader) imp[side - 1] -= (side == 1 ? 1.0f : -1.0f) * real_vz;
                const float inv = live ? 1.0f / (float)n : 0.0f;
                com = make_float3(com.x * inv + centre.x, com.y * inv + centre.y, com.z * inv + centre.z);
                mean = make_float3(mean.x * inv, mean.y * inv, mean.z * inv);
                // comoving frame; the side of the plane through the centre of mass
                float proj0 = 0.0f;
                int size0 = 0;
                for (uint32_t k = my_j; ext_lane && live && k < n; k += kExtLanes) {
                    const uint32_t p = at(k);
                    float4 xp = s_buf[p].pos, vp = s_buf[p].vel;
                    xp.x -= com.x; xp.y -= com.y; xp.z -= com.z;
                    vp.x -= mean.x; vp.y -= mean.y; vp.z -= mean.z;
                    s_buf[p].pos = xp;
                    s_buf[p].vel = vp;
                    if (dot3(make_float3(xp.x, xp.y, xp.z), axis) < 0) {
                        proj0 += dot3(make_float3(vp.x, vp.y, vp.z), axis);
                        size0 += 1;
                    }
                }
                proj0 = group_sum(proj0, kExtLanes);
                size0 = group_sum(size0, kExtLanes);
                const int size1 = (int)n - size0;
                const float proj1 = live ? -proj0 / (float)size1 : 0.0f;
                proj0 = live ? proj0 / (float)size0 : 0.0f;
                const float prob = live ? 1 - expf(0.01f * (proj1 - proj0) * (float)size0 * (float)size1) : 0.0f;
                const bool collide = live && gate < prob;
                // stochastic exchange along the axis, thermalised per side
                const float t0 = collide ? proj1 * ((float)size1 / (float)size0) : 0.0f;
                const float t1 = collide ? proj0 * ((float)size0 / (float)size1) : 0.0f;
                float mean0 = 0.0f, mean1 = 0.0f;
                float I[6] = {0, 0, 0, 0, 0, 0};
                float3 dL = make_float3(0, 0, 0);
                // Thermal draws: participant k uses Gaussian k & 3 of Philox block k >> 2.
                // With Philox draws, lane j of the group computes block 4u + j once per four
                // passes (all four Gaussians) and the group exchanges them by shuffles; the
                // trip count is uniform within the group so every shuffle is collective.
                const uint32_t passes = (ext_lane && collide) ? (n + kExtLanes - 1) / kExtLanes : 0u;
                const unsigned gmask = 0xFu << (lane & ~3);   // the cell's 4 collision lanes
                float gq[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                for (uint32_t t = 0; t < passes; ++t) {
                    const uint32_t k = kExtLanes * t + my_j;
                    float gk = 0.0f;
                    if (!TABLE) {
                        if ((t & 3u) == 0) {
                            const uint4 o = draw(b, step, kThermal, ref, t + my_j);
                            box_muller(o.x, o.y, gq[0], gq[1]);
                            box_muller(o.z, o.w, gq[2], gq[3]);
                        }
                        const int src = (lane & ~3) + (int)(t & 3u);   // the lane holding block t
                        const float q0 = __shfl_sync(gmask, gq[0], src), q1 = __shfl_sync(gmask, gq[1], src);
                        const float q2 = __shfl_sync(gmask, gq[2], src), q3 = __shfl_sync(gmask, gq[3], src);
                        gk = my_j == 0 ? q0 : my_j == 1 ? q1 : my_j == 2 ? q2 : q3;
                    }
                    if (k >= n) continue;
                    const uint32_t p = at(k);
                    const float4 xp = s_buf[p].pos;
                    float4 vp = s_buf[p].vel;
                    const float3 x = make_float3(xp.x, xp.y, xp.z);
                    float3 v = make_float3(vp.x, vp.y, vp.z);
                    const bool sd = dot3(x, axis) < 0;
                    const float vr = (TABLE ? D::thermal(a, b, step, ref, k) : gk) * b.tv;
                    if (sd) mean0 += vr; else mean1 += vr;
                    const float3 cr = cross3(x, v);
                    dL.x += cr.x; dL.y += cr.y; dL.z += cr.z;
                    const float kick = (vr - dot3(v, axis)) + (sd ? t0 : t1);
                    v.x += axis.x * kick; v.y += axis.y * kick; v.z += axis.z * kick;
                    s_buf[p].vel = make_float4(v.x, v.y, v.z, vp.w);
                    const float sx = x.x * x.x, sy = x.y * x.y, sz = x.z * x.z;
                    I[0] += sy + sz;
                    I[1] += sx + sz;
                    I[2] += sx + sy;
                    I[3] += -x.x * x.y;
                    I[4] += -x.x * x.z;
                    I[5] += -x.y * x.z;
                }
                mean0 = group_sum(mean0, kExtLanes);
                mean1 = group_sum(mean1, kExtLanes);
#pragma unroll
                for (int q = 0; q < 6; ++q) I[q] = group_sum(I[q], kExtLanes);
                const float m0 = collide ? mean0 / (float)size0 : 0.0f, m1 = collide ? mean1 / (float)size1 : 0.0f;
                const float3 vm0 = make_float3(axis.x * m0, axis.y * m0, axis.z * m0);
                const float3 vm1 = make_float3(axis.x * m1, axis.y * m1, axis.z * m1);
                for (uint32_t k = my_j; ext_lane && collide && k < n; k += kExtLanes) {
                    const uint32_t p = at(k);
                    const float4 xp = s_buf[p].pos;
                    float4 vp = s_buf[p].vel;
                    const float3 x = make_float3(xp.x, xp.y, xp.z);
                    const float3 vm = dot3(x, axis) < 0 ? vm0 : vm1;
                    vp.x -= vm.x; vp.y -= vm.y; vp.z -= vm.z;
                    s_buf[p].vel = vp;
                    const float3 cr = cross3(x, make_float3(vp.x, vp.y, vp.z));
                    dL.x -= cr.x; dL.y -= cr.y; dL.z -= cr.z;
                }
                dL = make_float3(group_sum(dL.x, kExtLanes), group_sum(dL.y, kExtLanes), group_sum(dL.z, kExtLanes));
                float3 omega = make_float3(0, 0, 0);
                if (collide) {
                    float Ii[6];
                    sym_inverse(I, 1e-5f, Ii);
                    omega = make_float3(Ii[0] * dL.x + Ii[3] * dL.y + Ii[4] * dL.z,
                                        Ii[3] * dL.x + Ii[1] * dL.y + Ii[5] * dL.z,
                                        Ii[4] * dL.x + Ii[5] * dL.y + Ii[2] * dL.z);
                }
                if (in_sub && leader) {
                    L.c0[i] = make_float4(mean.x, mean.y, mean.z, __uint_as_float(n));
                    L.c1[i] = make_float4(com.x, com.y, com.z, __uint_as_float(side));
                    L.omega[i] = make_float4(omega.x, omega.y, omega.z, __uint_as_float(m));
                }
            }
            __syncthreads();
            // particle-parallel finish over the sub-tile
            for (uint32_t pb = 0; pb < np; pb += kThreads) {
                const uint32_t p = pb + tid;
                if (p >= np) continue;
                const uint32_t info = s_cell[p];
                const uint32_t ci = info & ~kGhostFlag;
                if (info & kGhostFlag) s_buf[p].pos.w = __uint_as_float(kNoKey);
                else finish(p, ci, L.c0[ci], L.c1[ci]);
            }
            if (REPLAY) {
                __syncthreads();
                i0 = i1;
                continue;
            }

            // claim bucket slots (warp-aggregated atomics, all issued before any
            // result is used), then write the particles to their buckets; each
            // thread claims the entries p = tid + 256 j it finished itself, so no
            // barrier separates the two passes
            {
                uint32_t key[kMaxPerThread], peers[kMaxPerThread], base[kMaxPerThread];
                const int jmax = (int)((np + kThreads - 1) / kThreads);   // the same for every thread
#pragma unroll
                for (int j = 0; j < kMaxPerThread; ++j) {
                    key[j] = kNoKey;
                    peers[j] = 0;
                    base[j] = 0;
                    if (j >= jmax) continue;
                    const uint32_t p = (uint32_t)tid + (uint32_t)kThreads * j;
                    key[j] = p < np ? __float_as_uint(s_buf[p].pos.w) : kNoKey;
                    const bool act = key[j] != kNoKey;
                    const unsigned m = __ballot_sync(kFull, act);
                    peers[j] = 0;
                    base[j] = 0;
                    if (act) {
                        peers[j] = __match_any_sync(m, key[j]);
                        if (lane == __ffs(peers[j]) - 1) base[j] = atomicAdd(a.out_count + key[j], __popc(peers[j]));
                    }
                }
#pragma unroll
                for (int j = 0; j < kMaxPerThread; ++j) {
                    if (j >= jmax || key[j] == kNoKey) continue;
                    const uint32_t p = (uint32_t)tid + (uint32_t)kThreads * j;
                    const uint32_t slot =
                        __shfl_sync(peers[j], base[j], __ffs(peers[j]) - 1) + __popc(peers[j] & lanemask_lt());
                    const float4 xs = s_buf[p].pos, vp = s_buf[p].vel;
                    const float4 xp = make_float4(xs.x, xs.y, xs.z, __uint_as_float(kNoExt));
                    if (slot < b.depth) {
                        store_slot(a.out_slots + b.slot_base + (uint64_t)(key[j] - b.cell_base) * b.depth + slot, xp, vp);
                    } else {
                        push_overflow(a, key[j], xp, vp);
                    }
                }
            }
            __syncthreads();
            i0 = i1;
        }
    }
    if (a.pressure) {
#pragma unroll
        for (int w = 0; w < 2; ++w) {
            float v = imp[w];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
            if (lane == 0 && v != 0.0f) atomicAdd(&a.state->wall_impulse[w], (double)v);
        }
    }
}

// ------------------------------------------------------------------ SRD run kernel
//
// The production SRD step of one box or an ensemble (Philox draws; replays and the
// pressure estimator take step_kernel; TAPE: a sampled single-box step that records
// the adjoint tape, as step_kernel does): one warp per run of 32
// consecutive cells (storage order), lane l owning cell l of the run.  No
// CTA-wide barrier and no staging: each warp works alone on its runs with 1.5
// KB of shared memory of its own, and reads the particles straight from their
// buckets (a cell's bucket is contiguous).  Per run:
//   per cell (its lane): count, where its particles lie, wall ghosts (drawn by
//   the step's prologue), rotation axis; a prefix of the counts over the run;
//   then the run's particles, 32 consecutive ones at a time across cell and batch
//   boundaries: the collision, unshift, drag, lab-grid sample, streaming of step
//   k+1 and its cell, the slot claim (warp-aggregated) and one 256-bit store.
//   Before a group, the cells it reaches get their exact velocity sums and means,
//   a batch of 4, 8 or 16 cells (about 80 particles) at a time with 32 / batch
//   lanes per cell and four loads in flight each, so that the group's slots are
//   still in L1 from the sums.  Each batch asks L2 for the next batch's buckets.
// The arithmetic is step_kernel's (the same helpers), so a replay of this step
// by step_kernel (the getters) reproduces it bit for bit.

constexpr uint32_t kRunCells = 32;
// Cells summed together: BATCH = 4, 8 or 16, about 80 particles per batch (the
// engine picks it from n: a box's run_batch); 32 / BATCH lanes per cell in the sums.
constexpr int kRunWarps = kThreads / 32;
constexpr uint32_t kRunMaxN = 64;                     // densities this kernel takes

struct RunShared {                   // one per warp
    float4 cell[kRunCells];          // mean velocity, entries (particles + ghosts) as bits
    float4 axis[kRunCells];          // rotation axis
    long long gsum[kRunCells][3];    // exact velocity sums of the cell's ghosts
};

// Bring `bytes` (a multiple of 16, 16-byte aligned) of global memory into L2.
__device__ __forceinline__ void prefetch_l2(const void* src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

// A whole slot with one 256-bit load (the buckets of step k are read-only here).
__device__ __forceinline__ void load_slot(const Slot* src, float4& p, float4& v)
{
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(p.x), "=f"(p.y), "=f"(p.z), "=f"(p.w), "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
        : "l"(src));
}

// Run `run` of the launch: {first global cell, cells | box << 6}.
template <bool SINGLE>
__device__ __forceinline__ uint2 run_entry(const StepArgs& a, uint32_t run)
{
    if (run >= a.num_runs) return make_uint2(0u, 0u);
    if (!SINGLE) return __ldg(a.run_info + run);
    const uint32_t c0 = run * kRunCells;
    return make_uint2(a.box0.cell_base + c0, min(kRunCells, a.box0.C - c0));
}

template <bool SAMPLE, bool SINGLE, uint32_t BATCH, bool TAPE = false>
__global__ void __launch_bounds__(kThreads, 4) srd_run_kernel(const StepArgs a, uint32_t run_begin, uint32_t run_end,
                                                              bool first_launch)
{
    __shared__ RunShared shared_runs[kRunWarps];
    __shared__ __align__(16) BoxDesc shared_box[SINGLE ? 1 : kRunWarps];   // ensembles: the box of the warp's run
    const uint32_t lane = threadIdx.x & 31u;
    RunShared& sh = shared_runs[threadIdx.x >> 5];
    BoxDesc& sbox = shared_box[SINGLE ? 0 : threadIdx.x >> 5];
    const uint64_t step = a.step_base ? *a.step_base + a.step : a.step;   // graph replays read the base

    if (blockIdx.x == 0 && first_launch) {   // once per step (ensembles launch once per batch size)
        if (threadIdx.x == 0) a.state->ov_count[a.ov_zero_slot] = 0;   // list of step k-1, refilled by step k+1
        overflow_pass(a, step);
    }
    constexpr uint32_t kBatchCells = BATCH;
    constexpr uint32_t kBatchLanes = 32 / BATCH;   // lanes per cell in the sums
    static_assert(BATCH == 4 || BATCH == 8 || BATCH == 16, "batches of 4, 8 or 16 cells");
    // single box: geometry straight from the kernel parameters (constant bank)
    const BoxDesc& b = SINGLE ? a.box0 : sbox;
    float3 s = make_float3(0, 0, 0), sn = s;
    if (SINGLE) {
        s = grid_shift(b, 0, step, a.state);
        sn = grid_shift(b, 0, step + 1, a.state);
    }
    int cur_box = -1;
    const uint32_t warps = gridDim.x * (uint32_t)kRunWarps;
    uint32_t run = run_begin + blockIdx.x * (uint32_t)kRunWarps + (threadIdx.x >> 5);
    uint2 next = run_entry<SINGLE>(a, run < run_end ? run : a.num_runs);
    uint32_t raw_next = lane < (next.y & 63u) ? a.in_count[next.x + lane] : 0u;   // counts one run ahead
    if (SINGLE && lane < kBatchCells && raw_next)   // the first batch of the first run
        prefetch_l2(a.in_slots + b.slot_base + (uint64_t)(next.x - b.cell_base + lane) * b.depth,
                    min(raw_next, b.depth) * (uint32_t)sizeof(Slot));

    for (; run < run_end; run += warps) {
        const uint2 cur = next;
        if (!SINGLE && (int)(cur.y >> 6) != cur_box) {   // box and grid shifts (drawn by the prologue)
            cur_box = (int)(cur.y >> 6);
            __syncwarp();
            if (lane < sizeof(BoxDesc) / 16)
                reinterpret_cast<uint4*>(&sbox)[lane] = __ldg(reinterpret_cast<const uint4*>(a.boxes + cur_box) + lane);
            const float4 s0 = __ldg(a.box_shifts + 2 * cur_box), s1 = __ldg(a.box_shifts + 2 * cur_box + 1);
            s = make_float3(s0.x, s0.y, s0.z);
            sn = make_float3(s1.x, s1.y, s1.z);
            __syncwarp();
        }
        const bool sign = s.z > 0;
        const uint32_t c = cur.x - b.cell_base + lane;   // box-local cell of this lane
        const bool valid = lane < (cur.y & 63u);
        // the lane's cell: its colliding particles and the slot of the first (its
        // bucket, or for a cell past its depth its extension; below 2^32, which the
        // engine checks)
        const Slot* src_lane;
        const uint32_t cnt = cell_source(a, b, a.in_slots, c, raw_next, src_lane);
        const uint32_t src_slot = (uint32_t)(src_lane - a.in_slots);
        if (valid) a.zero_count[cur.x + lane] = 0;   // counts of step k-1: step k+1 fills them
        // sampled steps: the previous step's sample of this lane's (lab) cell into the
        // FP64 sums, where the engine defers it to this step (every cell is one lane's)
        if (SAMPLE && !TAPE && a.fold_samp && valid) fold_sample(a.fold_samp, a.acc, cur.x + lane, 0, nullptr);
        next = run_entry<SINGLE>(a, run + warps < run_end ? run + warps : a.num_runs);
        raw_next = lane < (next.y & 63u) ? a.in_count[next.x + lane] : 0u;
        const uint3 cc = storage_coords(b, valid ? c : 0u);
        bool layer, wall;
        wall_layer(b, cc.z, sign, layer, wall);
        wall = wall && valid;
        // wall ghosts (drawn by the step's prologue): count and exact velocity sums
        uint32_t ng = 0;
        {
            long long gx = 0, gy = 0, gz = 0;
            if (wall) {
                const GhostSum& g =
                    a.ghosts[b.wall_base + 2u * (cc.x + (uint32_t)b.L[0] * cc.y) + (cc.z == (uint32_t)sign ? 0u : 1u)];
                ng = g.n;
                gx = g.sx;
                gy = g.sy;
                gz = g.sz;
            }
            sh.gsum[lane][0] = gx;
            sh.gsum[lane][1] = gy;
            sh.gsum[lane][2] = gz;
        }
        const uint32_t m = cnt + ng;   // entries of the cell's collision
        if (TAPE && valid) a.tape_ncell[cur.x + lane] = m > 1 ? m : 0u;   // the adjoint tape: entries of collided cells
        {   // rotation axis (drawn for cells of more than one entry; zero for the others,
            // whose collision result the finish discards)
            float4 axw = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (m > 1) {
                const float3 ax = srd_axis_philox(b, step, ref_index(b, cc));
                axw = make_float4(ax.x, ax.y, ax.z, 0.0f);
            }
            sh.axis[lane] = axw;
        }
        __syncwarp();

        // the run's particles in order: cell c holds run particles [incl_c - cnt_c,
        // incl_c) (incl: inclusive prefix of the counts over the run's lanes), and run
        // particle t of cell c lies in slot rel_c + t (modulo 2^32)
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, incl, d);
            if ((int)lane >= d) incl += t;
        }
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        const uint32_t rel = src_slot - (incl - cnt);
        uint32_t summed = 0;           // cells [0, summed) have their means in sh.cell
        bool next_prefetched = false;  // the next run's first batch was asked of L2
        // 32 particles at a time, across batch boundaries
        for (uint32_t g0 = 0; g0 < total; g0 += 32) {
            // lanes past the run's last particle redo that particle and write nothing
            // (no branch around the particle's work)
            const bool active = g0 + lane < total;
            const uint32_t t = active ? g0 + lane : total - 1u;
            // cells of the group's first and last particles: the cells that end at or before them
            const uint32_t lo = __popc(__ballot_sync(kFull, incl <= g0));
            const uint32_t hi = __popc(__ballot_sync(kFull, incl <= min(g0 + 31u, total - 1u)));
            // exact sums and means of every cell up to hi, a batch of BATCH cells at a
            // time (kBatchLanes lanes per cell); each batch asks L2 for the next one's buckets
            while (summed <= hi) {
                const uint32_t c8 = summed;
                summed += kBatchCells;
                if (c8 + kBatchCells < kRunCells) {
                    if (lane >= c8 + kBatchCells && lane < c8 + 2 * kBatchCells && cnt)
                        prefetch_l2(a.in_slots + src_slot, cnt * (uint32_t)sizeof(Slot));
                } else {
                    next_prefetched = true;
                    if (SINGLE && lane < kBatchCells && raw_next)
                        prefetch_l2(a.in_slots + b.slot_base + (uint64_t)(next.x - b.cell_base + lane) * b.depth,
                                    min(raw_next, b.depth) * (uint32_t)sizeof(Slot));
                }
                const uint32_t L = c8 + lane / kBatchLanes, jl = lane % kBatchLanes;
                const uint32_t cntL = __shfl_sync(kFull, cnt, (int)L), mL = __shfl_sync(kFull, m, (int)L);
                const Slot* src = a.in_slots + __shfl_sync(kFull, src_slot, (int)L);
                long long sx = 0, sy = 0, sz = 0;
                float mx = 0.0f;
                for (uint32_t j = jl; j < cntL; j += 4 * kBatchLanes) {   // four loads in flight per lane
                    float4 v[4];
#pragma unroll
                    for (uint32_t u = 0; u < 4; ++u)
                        v[u] = j + u * kBatchLanes < cntL ? __ldg(&src[j + u * kBatchLanes].vel) : make_float4(0, 0, 0, 0);
                    int px = 0, py = 0, pz = 0;
#pragma unroll
                    for (uint32_t u = 0; u < 4; ++u) {
                        px += fixed24_narrow(v[u].x, mx);
                        py += fixed24_narrow(v[u].y, mx);
                        pz += fixed24_narrow(v[u].z, mx);
                    }
                    sx += px;
                    sy += py;
                    sz += pz;
                }
                if (__any_sync(kFull, mx >= kNarrowLimit)) {   // a speed of 32 or more in the batch: 64-bit sums
                    sx = sy = sz = 0;
                    for (uint32_t j = jl; j < cntL; j += kBatchLanes) {
                        const float4 v = __ldg(&src[j].vel);
                        sx += fixed24(v.x);
                        sy += fixed24(v.y);
                        sz += fixed24(v.z);
                    }
                }
#pragma unroll
                for (uint32_t o = 1; o < kBatchLanes; o <<= 1) {
                    sx += __shfl_xor_sync(kFull, sx, (int)o);
                    sy += __shfl_xor_sync(kFull, sy, (int)o);
                    sz += __shfl_xor_sync(kFull, sz, (int)o);
                }
                if (jl == 0) {
                    sx += sh.gsum[L][0];
                    sy += sh.gsum[L][1];
                    sz += sh.gsum[L][2];
                    const float3 mean = mL > 1 ? srd_mean(sx, sy, sz, mL) : make_float3(0, 0, 0);
                    sh.cell[L] = make_float4(mean.x, mean.y, mean.z, __uint_as_float(mL));
                }
            }
            __syncwarp();   // the means are written
            // cell i of particle t: the first cell that ends after t -- within [lo, lo + W)
            // when the group spans at most W cells (W = 4, or 8 with 16-cell batches), else
            // over the run (incl of lane 31 is the run's total, beyond every active t)
            constexpr uint32_t kWindow = BATCH == 16 ? 8u : 4u;
            uint32_t i;
            if (hi - lo < kWindow) {
                i = lo;
#pragma unroll
                for (uint32_t half = kWindow / 2; half; half >>= 1)
                    i += t >= __shfl_sync(kFull, incl, (int)min(i + half - 1u, 31u)) ? half : 0u;
            } else {
                i = 0;
#pragma unroll
                for (uint32_t half = 16; half; half >>= 1)
                    i += t >= __shfl_sync(kFull, incl, (int)(i + half - 1)) ? half : 0u;
            }
            const uint32_t slot = __shfl_sync(kFull, rel, (int)(i & 31u)) + t;
            uint32_t key = 0, id = 0;
            float3 xn = make_float3(0, 0, 0), vn = xn;
            {
                float4 xp, vp;
                load_slot(a.in_slots + slot, xp, vp);
                const float4 cd = sh.cell[i];
                const float4 ax = sh.axis[i];
                float3 x = make_float3(xp.x, xp.y, xp.z), v = make_float3(vp.x, vp.y, vp.z);
                {   // the collision computed for every lane, kept where the cell has more than one
                    // entry (a lone particle keeps its shifted position, as in the reference)
                    float3 xc = x, vc = v;
                    srd_collide(b, s, make_float3(cd.x, cd.y, cd.z), make_float3(ax.x, ax.y, ax.z), xc, vc);
                    const bool collided = __float_as_uint(cd.w) > 1;
                    x = collided ? xc : x;
                    v = collided ? vc : v;
                }
                vn = v;
                xn = stream_shift(b, x, vn, sn);
                key = b.cell_base + storage_index(b, cell_of_wrapped(b, xn));
                id = __float_as_uint(vp.w);
                const uint32_t lab = SAMPLE || TAPE ? b.cell_base + storage_index(b, cell_of_wrapped(b, x)) : 0u;
                if (SAMPLE) sample_add(a.samp, lab, v, active);
                if (TAPE && active) {   // collision cell (or none), lab cell and the bounce of the streaming that follows
                    const bool bounced = vn.x != v.x || vn.y != v.y || vn.z != v.z;
                    a.tape_key[id] = __float_as_uint(cd.w) > 1 ? cur.x + i : kTapeNone;
                    a.tape_lab[id] = lab | (bounced ? kTapeBounce : 0u);
                }
            }
            store_particle(a, b, xn, vn, id, key, active);
        }
        // a run whose last cells are empty: the next run's first batch
        if (SINGLE && !next_prefetched && lane < kBatchCells && raw_next)
            prefetch_l2(a.in_slots + b.slot_base + (uint64_t)(next.x - b.cell_base + lane) * b.depth,
                        min(raw_next, b.depth) * (uint32_t)sizeof(Slot));
        __syncwarp();   // the next run rewrites this warp's shared arrays
    }
}

// Before step k: every cell that received more particles than its bucket
// holds (raw count > depth) gets its colliding set -- all raw particles, or the
// cap lowest ids when raw > cap, whatever order the claims of step k-1 arrived
// in: the reference fills each cell's table in particle-index order, and the
// particles past its depth skip the collision (simulation_functions.cpp:87-93) --
// as min(raw, cap) contiguous slots of the extension area of step k's bucket set.
// The thread of a cell's last overflow entry (the head of the cell's chain)
// copies the bucket there, then walks the raw - depth entries of the chain: each
// fills the next free slot (its list entry is marked taken), or, once cap slots
// are filled, swaps with the set's largest id if its own id is smaller.  It then
// records the extension offset in pos.w of the cell's first bucket slot and marks
// the chain handled, so that a second selection of the same step changes
// nothing.  Overflow is rare: without any, every thread returns after one load.
// Run on the inputs of step k, so a replay of step k finds them in place.
// Block 0 also empties the extension of the other parity (step k+1's: step k-1,
// its last reader, is past replaying).
__global__ void __launch_bounds__(kThreads) overflow_select_kernel(const StepArgs a, Slot* in_slots, float4* ov_pos,
                                                                   float4* ov_vel, uint32_t* ov_head)
{
    // Wall ghosts of step k for srd_run_kernel: one thread per wall cell (the two
    // ghost layers of every column) draws the ghost count and the ghosts' summed
    // velocity, as step_kernel draws them, and stores the count and the exact
    // velocity sums.  Drawn here, every thread busy, instead of by a few lanes
    // of each run.
    const uint64_t step = a.step_base ? *a.step_base + a.step : a.step;
    if (a.run_kernel && a.box_shifts) {   // ensembles: every box's grid shifts of steps k and k+1
        for (uint32_t bi = blockIdx.x * blockDim.x + threadIdx.x; bi < (uint32_t)a.nboxes; bi += gridDim.x * blockDim.x) {
            const float3 s0 = grid_shift(a.boxes[bi], (int)bi, step, a.state);
            const float3 s1 = grid_shift(a.boxes[bi], (int)bi, step + 1, a.state);
            a.box_shifts[2 * bi] = make_float4(s0.x, s0.y, s0.z, 0.0f);
            a.box_shifts[2 * bi + 1] = make_float4(s1.x, s1.y, s1.z, 0.0f);
        }
    }
    if (a.run_kernel && a.ghosts) {
        for (uint64_t wg = blockIdx.x * blockDim.x + threadIdx.x; wg < a.total_walls;
             wg += (uint64_t)gridDim.x * blockDim.x) {
            int bi = 0;   // the box of entry wg: the last with wall_base <= wg (boxes without walls add none)
            if (a.nboxes > 1) {
                int hi = a.nboxes - 1;
                while (bi < hi) {
                    const int mid = (bi + hi + 1) >> 1;
                    if (a.boxes[mid].wall_base <= wg) bi = mid; else hi = mid - 1;
                }
            }
            const BoxDesc& b = a.nboxes > 1 ? a.boxes[bi] : a.box0;
            const float3 s = grid_shift(b, bi, step, a.state);
            const float shift_abs = fabsf(s.z);
            const bool sign = s.z > 0;
            const uint32_t Lx = (uint32_t)b.L[0], Lz = (uint32_t)b.L[2];
            const uint32_t w = (uint32_t)(wg - b.wall_base);
            const uint32_t col = w >> 1, y = fast_div(col, b.div_x), x = col - y * Lx;
            const uint32_t cz = (w & 1u) ? Lz - (sign ? 1u : 2u) : (sign ? 1u : 0u);
            bool layer, ghosts;
            wall_layer(b, cz, sign, layer, ghosts);
            const uint32_t ref = ref_index(b, make_uint3(x, y, cz));
            uint32_t g = 0;
            for (uint32_t chunk = 0; 4 * chunk < b.n; ++chunk) {
                const uint4 o = draw(b, step, kGhostCount, ref, chunk);
                const uint32_t u[4] = {o.x, o.y, o.z, o.w};
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (4 * chunk + k < b.n && ((u01(u[k]) > shift_abs) ^ layer ^ sign)) ++g;
            }
            GhostSum r{0, 0, 0, g, 0u};
            if (g) {
                const float3 v = ghost_sum_velocity(b, step, ref, g);
                r.sx = fixed24(v.x);
                r.sy = fixed24(v.y);
                r.sz = fixed24(v.z);
            }
            a.ghosts[wg] = r;
        }
    }
    const uint32_t par = (uint32_t)(a.step & 1u);
    if (blockIdx.x == 0 && threadIdx.x == 0) a.state->ext_count[par ^ 1u] = 0;
    const uint32_t n = min(a.state->ov_count[a.ov_in_slot], a.ov_cap);
    for (uint32_t e0 = blockIdx.x * blockDim.x + threadIdx.x; e0 < n; e0 += gridDim.x * blockDim.x) {
        const uint32_t id0 = __float_as_uint(ov_vel[e0].w);
        if (id0 == kTakenId) continue;
        const float4 p0 = ov_pos[e0];
        const int bi = box_of_particle(a.boxes, a.nboxes, id0);
        const BoxDesc& b = a.boxes[bi];
        const uint32_t key = b.cell_base + storage_index(b, cell_of_wrapped(b, make_float3(p0.x, p0.y, p0.z)));
        if (ov_head[key] != e0) continue;   // not the head of its cell's chain (or handled)
        ov_head[key] = kChainDone;
        const uint32_t raw = a.in_count[key];
        const uint32_t m = min(raw, b.cap);
        if (raw <= b.depth) continue;   // (an entry exists only past the depth)
        Slot* const bucket = in_slots + b.slot_base + (uint64_t)(key - b.cell_base) * b.depth;
        const uint32_t off = atomicAdd(&a.state->ext_count[par], m);
        if (off > a.ext_cap - m) {   // no room: the cell keeps its bucket, the step kernels read only that
            atomicOr(&a.state->error_flags, kErrExtensionFull);
            bucket->pos.w = __uint_as_float(kNoExt);
            continue;
        }
        Slot* const ext = in_slots + a.total_slots + off;
        for (uint32_t j = 0; j < b.depth; ++j) ext[j] = bucket[j];
        uint32_t filled = b.depth, e = e0;
        for (uint32_t t = b.depth; t < raw && e < a.ov_cap; ++t) {
            const uint32_t before = a.ov_next_in[e];
            const float4 pe = ov_pos[e], we = ov_vel[e];
            if (filled < m) {
                ext[filled].pos = pe;
                ext[filled].vel = we;
                ++filled;
                ov_vel[e].w = __uint_as_float(kTakenId);
            } else {
                uint32_t jmax = 0, idmax = __float_as_uint(ext[0].vel.w);
                for (uint32_t j = 1; j < m; ++j) {
                    const uint32_t id = __float_as_uint(ext[j].vel.w);
                    if (id > idmax) {
                        idmax = id;
                        jmax = j;
                    }
                }
                if (__float_as_uint(we.w) < idmax) {
                    ov_pos[e] = ext[jmax].pos;
                    ov_vel[e] = ext[jmax].vel;
                    ext[jmax].pos = pe;
                    ext[jmax].vel = we;
                }
            }
            e = before;
        }
        bucket->pos.w = __uint_as_float(off);
    }
}

// Advance the step base of graph replays by the steps one replay runs.
__global__ void advance_kernel(DeviceState* state, unsigned steps)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) state->step_base += steps;
}

// ------------------------------------------------------------------ prologue scatter

// Stream dense post-step particles for step k (a.step = k - 1: the launch plays
// the epilogue of step k-1), key them by the cell they then occupy and scatter
// them into the buckets of step k (a.out_*); particle id = dense index.
__global__ void __launch_bounds__(kThreads) scatter_kernel(StepArgs a, const float* pos, const float* vel,
                                                           uint64_t n_total)
{
    for (uint64_t base = (uint64_t)blockIdx.x * kThreads; base < n_total; base += (uint64_t)gridDim.x * kThreads) {
        const uint64_t i = base + threadIdx.x;
        const bool active = i < n_total;
        int bi = 0;
        uint32_t key = 0;
        float3 xs = make_float3(0, 0, 0), vs = xs;
        if (active) {
            bi = box_of_particle(a.boxes, a.nboxes, i);
            const BoxDesc& b = a.boxes[bi];
            vs = make_float3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
            const float3 v0 = vs;
            xs = stream_shift(b, make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), vs,
                              grid_shift(b, bi, a.step + 1, a.state));
            key = b.cell_base + storage_index(b, cell_of_wrapped(b, xs));
            if (a.tape_lab) a.tape_lab[i] = (vs.x != v0.x || vs.y != v0.y || vs.z != v0.z) ? kTapeBounce : 0u;
        }
        store_particle(a, a.boxes[bi], xs, vs, (uint32_t)i, key, active);
    }
}

// ------------------------------------------------------------------ sampling

// Per lab cell: fold_sample.  Any cell order (the sums are kept in storage order).
__global__ void sample_finalize_kernel(float4* samp, SampleAcc* acc, uint64_t cells, int snapshot,
                                       uint32_t* lab_count)
{
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells;
         c += (uint64_t)gridDim.x * blockDim.x)
        fold_sample(samp, acc, c, snapshot, lab_count);
}

// Mean fields of one box in reference order (x fastest) from the FP64 sums, which
// are kept in storage order: density n / S and velocity v / S per lab cell
// (cpu_backend.cpp:218, `inverse` = 1 / S).
__global__ void mean_fields_kernel(const SampleAcc* acc, BoxDesc b, double inverse, float* density, float* velocity)
{
    const uint32_t Lx = (uint32_t)b.L[0], Ly = (uint32_t)b.L[1], Lz = (uint32_t)b.L[2];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < b.C; r += gridDim.x * blockDim.x) {
        const uint32_t x = r % Lx, yz = r / Lx, y = yz % Ly, z = yz / Ly;
        const SampleAcc q = acc[b.cell_base + z + Lz * (x + Lx * y)];
        const uint64_t g = b.cell_base + (uint64_t)r;
        density[g] = (float)(q.n * inverse);
        velocity[3 * g + 0] = (float)(q.vx * inverse);
        velocity[3 * g + 1] = (float)(q.vy * inverse);
        velocity[3 * g + 2] = (float)(q.vz * inverse);
    }
}

// ------------------------------------------------------------------ compaction

// Decoupled look-back exclusive scan of min(count, cap) over all cells (the
// colliding particles of each cell)
// (Merrill & Garland, "Single-pass parallel prefix scan with decoupled look-back").
// status[t]: bits 62-63 flag (1 aggregate, 2 inclusive prefix), low 32 value.
constexpr int kScanItems = 8;
constexpr uint64_t kFlagAgg = 1ull << 62, kFlagPre = 2ull << 62;

__device__ __forceinline__ uint32_t cell_cap(const BoxDesc* boxes, int nboxes, uint64_t c)
{
    int lo = 0, hi = nboxes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (boxes[mid].cell_base <= c) lo = mid; else hi = mid - 1;
    }
    return boxes[lo].cap;
}

__global__ void __launch_bounds__(kThreads) scan_kernel(const uint32_t* count, const BoxDesc* boxes, int nboxes,
                                                        uint64_t cells, uint32_t* offsets,
                                                        unsigned long long* status, unsigned int* tile_counter,
                                                        DeviceState* state)
{
    __shared__ uint32_t warp_tot[kThreads / 32 + 1];
    __shared__ uint32_t s_tile, s_prefix;
    if (threadIdx.x == 0) s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t first = (uint64_t)tile * kThreads * kScanItems + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems], sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint64_t c = first + k;
        v[k] = c < cells ? min(count[c], cell_cap(boxes, nboxes, c)) : 0u;
        sum += v[k];
    }
    uint32_t total;
    const uint32_t excl = block_exclusive_scan(sum, warp_tot, total);
    if (threadIdx.x == 0) {
        uint32_t prefix = 0;
        if (tile == 0) {
            atomicExch(status + tile, kFlagPre | total);
        } else {
            atomicExch(status + tile, kFlagAgg | total);
            int64_t t = (int64_t)tile - 1;
            const uint64_t t0 = globaltimer();
            bool timed_out = false;
            while (t >= 0) {
                const unsigned long long w = atomicAdd(status + t, 0ull);
                const uint64_t flag = w & (3ull << 62);
                if (flag == 0) {
                    if (globaltimer() - t0 > kWaitLimitNs) { timed_out = true; break; }
                    continue;
                }
                prefix += (uint32_t)w;
                if (flag == kFlagPre) break;
                --t;
            }
            if (timed_out) {
                atomicOr(&state->error_flags, kErrWaitTimeout);
                __threadfence();   // the flag is visible before the (incomplete) prefix is
            }
            atomicExch(status + tile, kFlagPre | (uint32_t)(prefix + total));
        }
        s_prefix = prefix;
    }
    __syncthreads();
    uint32_t run = s_prefix + excl;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint64_t c = first + k;
        if (c < cells) offsets[c] = run;
        run += v[k];
    }
    if (tile == (uint32_t)((cells + kThreads * kScanItems - 1) / (kThreads * kScanItems)) - 1 &&
        threadIdx.x == kThreads - 1) {
        // a look-back that gave up anywhere before this tile published an incomplete
        // prefix: mark the result invalid in the buffer itself
        __threadfence();
        const bool bad = (atomicAdd(&state->error_flags, 0u) & kErrWaitTimeout) != 0;
        offsets[cells] = bad ? 0xFFFFFFFFu : s_prefix + total;
    }
}

// Layout dump: the particles of every cell, in stable order, cells in storage
// order, followed by the overflow list.  offsets from scan_kernel.
__global__ void __launch_bounds__(kThreads) compact_kernel(const StepArgs a, const uint32_t* count,
                                                           const Slot* slots,
                                                           const uint32_t* offsets, uint64_t cells, uint64_t n_total,
                                                           uint32_t* out_cell, uint32_t* out_slot, uint32_t* out_prev,
                                                           uint32_t* out_id)
{
    for (uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; c < cells;
         c += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = a.nboxes - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.boxes[mid].cell_base <= c) lo = mid; else hi = mid - 1;
        }
        const BoxDesc& b = a.boxes[lo];
        const Slot* src;
        const uint32_t n = cell_source(a, b, slots, (uint32_t)(c - b.cell_base), count[c], src);
        const uint64_t slot0 = (uint64_t)(src - slots);
        const uint32_t dst0 = offsets[c];
        const uint32_t ref = ref_index(b, storage_coords(b, (uint32_t)(c - b.cell_base)));
        for (uint32_t q = 0; q < n; ++q) {
            const uint32_t key = __float_as_uint(slots[slot0 + q].vel.w);   // particle id
            uint32_t rank = 0;
            for (uint32_t u = 0; u < n; ++u) {
                const uint32_t ku = __float_as_uint(slots[slot0 + u].vel.w);
                rank += ku < key || (ku == key && u < q);
            }
            const uint64_t d = (uint64_t)dst0 + rank;
            if (d >= n_total) {
                atomicOr(&a.state->error_flags, kErrKeyMismatch);
                continue;
            }
            if (out_cell) out_cell[d] = b.cell_base + ref;
            if (out_slot) out_slot[d] = (uint32_t)(slot0 + rank);
            if (out_prev) out_prev[d] = key;
            if (out_id) out_id[d] = __float_as_uint(slots[slot0 + q].vel.w);
        }
    }
}

// The overflow list's particles that do not collide (entries not taken into an
// extension), after the cells' particles in any order (the host orders them by
// cell and id); *placed counts them.  slot = total_slots + ext_cap + entry.
__global__ void compact_overflow_kernel(const BoxDesc* boxes, int nboxes, const float4* ov_pos,
                                        const float4* ov_vel, const DeviceState* st, unsigned parity, uint32_t ov_cap,
                                        const uint32_t* offsets, uint64_t cells, uint64_t n_total,
                                        uint64_t list_slot0, unsigned int* placed, uint32_t* out_cell,
                                        uint32_t* out_slot, uint32_t* out_prev, uint32_t* out_id)
{
    const uint32_t n = min(st->ov_count[parity], ov_cap);
    const uint32_t base = offsets[cells];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const uint32_t id = __float_as_uint(ov_vel[q].w);
        if (id == kTakenId) continue;
        const uint64_t d = (uint64_t)base + atomicAdd(placed, 1u);
        if (d >= n_total) continue;
        if (out_cell) {   // the cell the (already streamed) particle is keyed to
            const float4 p = ov_pos[q];
            const int bi = box_of_particle(boxes, nboxes, id);
            const BoxDesc& b = boxes[bi];
            out_cell[d] = b.cell_base + ref_index(b, cell_of(b, make_float3(p.x, p.y, p.z)));
        }
        if (out_slot) out_slot[d] = (uint32_t)(list_slot0 + q);
        if (out_prev) out_prev[d] = id;
        if (out_id) out_id[d] = id;
    }
}

// ------------------------------------------------------------------ initialisation

// Uniform positions in the fluid volume (channel: inside the cylinder of radius
// (Lz-2)/2 in y-z), Maxwell-Boltzmann velocities (simulation_kernels.cu:22-58).
__global__ void init_kernel(const BoxDesc* boxes, int nboxes, float* pos, float* vel, uint64_t n_total)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_total;
         i += (uint64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = nboxes - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (boxes[mid].dense_base <= i) lo = mid; else hi = mid - 1;
        }
        const BoxDesc& b = boxes[lo];
        const uint64_t k = i - b.dense_base;
        float sc[3];
        for (int d = 0; d < 3; ++d) sc[d] = b.Lf[d] - (float)(2 * (1 - b.periodic[d]));
        float3 x;
        uint32_t attempt = 0;
        while (true) {
            const uint4 o = philox4x32_10(make_uint4((uint32_t)k, (uint32_t)(k >> 32), kInit, 2 * attempt),
                                          b.seed_lo, b.seed_hi);
            x = make_float3((u01(o.x) - 0.5f) * sc[0], (u01(o.y) - 0.5f) * sc[1], (u01(o.z) - 0.5f) * sc[2]);
            if (!b.channel || (x.z * x.z + x.y * x.y) <= b.R2 || attempt > 64) break;
            ++attempt;
        }
        const uint4 o = philox4x32_10(make_uint4((uint32_t)k, (uint32_t)(k >> 32), kInit, 1u), b.seed_lo, b.seed_hi);
        float g0, g1, g2, g3;
        box_muller(o.x, o.y, g0, g1);
        box_muller(o.z, o.w, g2, g3);
        pos[3 * i] = x.x; pos[3 * i + 1] = x.y; pos[3 * i + 2] = x.z;
        vel[3 * i] = g0 * b.tv; vel[3 * i + 1] = g1 * b.tv; vel[3 * i + 2] = g2 * b.tv;
    }
}

// Velocity sums of particles [begin, end) in FP64, one partial per block, in a
// fixed order (the host adds the partials), so momentum removal is deterministic.
__global__ void momentum_partial_kernel(const float* vel, uint64_t begin, uint64_t end, double* partial)
{
    __shared__ double red[3][kThreads];
    double sx = 0, sy = 0, sz = 0;
    for (uint64_t i = begin + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < end;
         i += (uint64_t)gridDim.x * blockDim.x) {
        sx += vel[3 * i]; sy += vel[3 * i + 1]; sz += vel[3 * i + 2];
    }
    red[0][threadIdx.x] = sx; red[1][threadIdx.x] = sy; red[2][threadIdx.x] = sz;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int d = 0; d < 3; ++d) red[d][threadIdx.x] += red[d][threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; ++d) partial[3 * blockIdx.x + d] = red[d][0];
}

__global__ void subtract_kernel(float* vel, uint64_t begin, uint64_t end, float mx, float my, float mz)
{
    for (uint64_t i = begin + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < end;
         i += (uint64_t)gridDim.x * blockDim.x) {
        vel[3 * i] -= mx; vel[3 * i + 1] -= my; vel[3 * i + 2] -= mz;
    }
}

// ------------------------------------------------------------------ adjoint of the sampled profile
//
// With the discrete events of a trajectory held fixed (collision cells and their
// occupancy N_c incl. ghosts, grid shifts, rotation axes -- replayed from the
// Philox counters --, bounce-backs, lab cells), the velocities are affine in the
// initial velocities V0 and the body force g:
//   P_0 = B_0 V0,  Q_t = Coll_t(P_t) (+ g dt e_x on collided particles),  P_{t+1} = B_{t+1} Q_t,
//   Coll_t: v'_i = u_c + R_c (v_i - u_c),  u_c = (sum of the cell's particles and ghosts) / N_c,
//   U(z) = sum_t sum_{x,y} m_c(t) / (S Lx Ly),  m_c(t) = sum_{i in lab cell c} Q_{t,i,x} / count_c(t),
// where B flips the velocity of a bounced particle (simulation_functions.cpp:53-82) and
// positions enter only through the fixed events.  Reverse sweep, t = S-1 .. 0:
//   mu_t = B_{t+1} lambda_{t+1} + dU/dQ_t . dL/dU,
//   lambda_{t,i} = R_c^T (mu_i - s_c) + s_c,  s_c = sum_{j in c} mu_j / N_c  (collided i; else mu_i),
//   dL/dg += dt sum_{collided i} mu_{t,i,x},  and finally dL/dV0 = B_0 lambda_0.

// U(z) of one box from the FP64 sample sums (storage order): one block per z layer.
__global__ void __launch_bounds__(kThreads) profile_kernel(const SampleAcc* acc, BoxDesc b, double inv,
                                                           float* profile)
{
    __shared__ double red[kThreads];
    const uint32_t per = (uint32_t)(b.L[0] * b.L[1]);
    double s = 0;
    // layer z of the storage order: cells z + Lz k, k = x + Lx y
    for (uint32_t k = threadIdx.x; k < per; k += kThreads) s += acc[b.cell_base + blockIdx.x + (uint64_t)b.L[2] * k].vx;
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) profile[blockIdx.x] = (float)(red[0] * inv);
}

// Per cell of the step (storage order): clear the cell sums of mu, and store the
// cell's rotation axis (as a collision cell) and its sampling term dU(z) w / count
// (as a lab cell; FP64 quotient rounded to FP32) in cell_axis, so that the particle
// passes read them instead of drawing an axis and dividing per particle.
__global__ void __launch_bounds__(kThreads) adjoint_cells_kernel(BoxDesc b, uint64_t step, const uint32_t* lab_count,
                                                                 const float* dU, double w, float4* cellsum,
                                                                 float4* cell_axis)
{
    const uint32_t Lz = (uint32_t)b.L[2];
    for (uint32_t c = blockIdx.x * kThreads + threadIdx.x; c < b.C; c += gridDim.x * kThreads) {
        cellsum[c] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const uint32_t cnt = lab_count[b.cell_base + c];
        const float term = cnt ? (float)((double)dU[c % Lz] * w / (double)cnt) : 0.0f;   // z fastest
        const float3 a = srd_axis_philox(b, step, ref_index(b, storage_coords(b, c)));
        cell_axis[c] = make_float4(a.x, a.y, a.z, term);
    }
}

// mu = B_{t+1} lambda + sampling term; cell sums of mu over collided particles; dL/dg partial.
__global__ void __launch_bounds__(kThreads) adjoint_pass1_kernel(BoxDesc b, uint32_t n, float* lam,
                                                                 const uint32_t* key, const uint32_t* lab,
                                                                 const float4* cell_axis, float4* cellsum,
                                                                 double* gsum)
{
    __shared__ double red[kThreads];
    double gl = 0;
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
        float3 m = make_float3(lam[3 * i], lam[3 * i + 1], lam[3 * i + 2]);
        const uint32_t l = lab[i];
        if (l & kTapeBounce) m = make_float3(-m.x, -m.y, -m.z);
        const uint32_t c = l & ~kTapeBounce;
        m.x += __ldg(&cell_axis[c - b.cell_base].w);
        lam[3 * i] = m.x; lam[3 * i + 1] = m.y; lam[3 * i + 2] = m.z;
        const uint32_t k = key[i];
        if (k != kTapeNone) {
            atomicAdd(cellsum + k, make_float4(m.x, m.y, m.z, 0.0f));
            gl += (double)m.x;
        }
    }
    red[threadIdx.x] = gl;
    __syncthreads();
    for (int o = kThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(gsum, red[0]);
}

// lambda = R^T (mu - s_c) + s_c for collided particles (R^T: rotation by -alpha).
__global__ void __launch_bounds__(kThreads) adjoint_pass2_kernel(BoxDesc b, uint32_t n, float* lam,
                                                                 const uint32_t* key, const uint32_t* ncell,
                                                                 const float4* cellsum, const float4* cell_axis)
{
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
        const uint32_t k = key[i];
        if (k == kTapeNone) continue;
        const float inv = 1.0f / (float)ncell[k];
        const float4 cs = cellsum[k];
        const float3 sc = make_float3(cs.x * inv, cs.y * inv, cs.z * inv);
        const float4 ax = __ldg(&cell_axis[k - b.cell_base]);
        const float3 a = make_float3(ax.x, ax.y, ax.z);
        const float3 wv = make_float3(lam[3 * i] - sc.x, lam[3 * i + 1] - sc.y, lam[3 * i + 2] - sc.z);
        const float d = dot3(wv, a);
        const float3 para = make_float3(a.x * d, a.y * d, a.z * d);
        const float3 perp = make_float3(wv.x - para.x, wv.y - para.y, wv.z - para.z);
        const float3 cr = cross3(wv, a);
        lam[3 * i] = (para.x + b.cos_a * perp.x) - b.sin_a * cr.x + sc.x;
        lam[3 * i + 1] = (para.y + b.cos_a * perp.y) - b.sin_a * cr.y + sc.y;
        lam[3 * i + 2] = (para.z + b.cos_a * perp.z) - b.sin_a * cr.z + sc.z;
    }
}

// dL/dV0 = B_0 lambda_0.
__global__ void __launch_bounds__(kThreads) adjoint_finish_kernel(uint32_t n, const float* lam, const uint32_t* b0,
                                                                  float* out)
{
    for (uint32_t i = blockIdx.x * kThreads + threadIdx.x; i < n; i += gridDim.x * kThreads) {
        const float f = (b0[i] & kTapeBounce) ? -1.0f : 1.0f;
        out[3 * i] = f * lam[3 * i];
        out[3 * i + 1] = f * lam[3 * i + 1];
        out[3 * i + 2] = f * lam[3 * i + 2];
    }
}

}  // namespace

// ------------------------------------------------------------------ launchers

size_t step_smem_bytes(uint32_t pbuf, uint32_t cells, int algorithm) { return tile_smem_bytes(pbuf, cells, algorithm); }

namespace {
using StepFn = void (*)(const StepArgs, uint32_t);
// [algorithm][table draws][single box][replay]
const StepFn kStepFns[2][2][2][2] = {
    {{{step_kernel<0, false, false, false>, step_kernel<0, false, false, true>},
      {step_kernel<0, false, true, false>, step_kernel<0, false, true, true>}},
     {{step_kernel<0, true, false, false>, step_kernel<0, true, false, true>},
      {step_kernel<0, true, true, false>, step_kernel<0, true, true, true>}}},
    {{{step_kernel<1, false, false, false>, step_kernel<1, false, false, true>},
      {step_kernel<1, false, true, false>, step_kernel<1, false, true, true>}},
     {{step_kernel<1, true, false, false>, step_kernel<1, true, false, true>},
      {step_kernel<1, true, true, false>, step_kernel<1, true, true, true>}}}};
}  // namespace

using StepFnRun = void (*)(const StepArgs, uint32_t, uint32_t, bool);
// [sample][single box][batch class: 16, 8, 4 cells]
// single-box sampled steps that record the adjoint tape, by batch size
static const StepFnRun kRunTapeFns[3] = {srd_run_kernel<true, true, 16, true>, srd_run_kernel<true, true, 8, true>,
                                         srd_run_kernel<true, true, 4, true>};
static const StepFnRun kRunFns[2][2][3] = {
    {{srd_run_kernel<false, false, 16>, srd_run_kernel<false, false, 8>, srd_run_kernel<false, false, 4>},
     {srd_run_kernel<false, true, 16>, srd_run_kernel<false, true, 8>, srd_run_kernel<false, true, 4>}},
    {{srd_run_kernel<true, false, 16>, srd_run_kernel<true, false, 8>, srd_run_kernel<true, false, 4>},
     {srd_run_kernel<true, true, 16>, srd_run_kernel<true, true, 8>, srd_run_kernel<true, true, 4>}}};

bool run_kernel_takes(const StepArgs& a, int algorithm, bool table)
{
    return algorithm == 0 && !table && !a.replay && (!a.tape_key || (a.nboxes == 1 && a.sample)) && !a.pressure &&
           (a.ghosts || !a.total_walls) && (a.nboxes == 1 || (a.run_info && a.box_shifts)) &&
           a.boxes_n_max <= kRunMaxN;
}

cudaError_t launch_step(const StepArgs& a, int algorithm, bool table, uint32_t pbuf, int grid, cudaStream_t st,
                        const RunBranches* branches)
{
    if (a.run_kernel) {
        // one launch per batch size in use: a single box's, or an ensemble's density
        // classes, whose runs the run table lists class by class; with branches, the
        // second and third class on side streams (the classes share no cell and no
        // count: every write is an atomic claim or a lane's own cell)
        int used[3], nused = 0;
        for (int cls = 0; cls < 3; ++cls)
            if (a.run_class[cls] < a.run_class[cls + 1]) used[nused++] = cls;
        const bool fork = branches && branches->side[0] && branches->side[1] && nused > 1;
        cudaError_t e = cudaSuccess;
        if (fork) {
            e = cudaEventRecord(branches->fork, st);
            for (int i = 1; i < nused && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(branches->side[i - 1], branches->fork, 0);
            if (e != cudaSuccess) return e;
        }
        for (int i = 0; i < nused; ++i) {
            const int cls = used[i];
            const StepFnRun f = a.tape_key ? kRunTapeFns[cls] : kRunFns[a.sample ? 1 : 0][a.nboxes == 1 ? 1 : 0][cls];
            f<<<grid, kThreads, 0, fork && i > 0 ? branches->side[i - 1] : st>>>(a, a.run_class[cls],
                                                                                    a.run_class[cls + 1], i == 0);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
        }
        if (fork) {
            for (int i = 1; i < nused && e == cudaSuccess; ++i) {
                e = cudaEventRecord(branches->join[i - 1], branches->side[i - 1]);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(st, branches->join[i - 1], 0);
            }
        }
        return e;
    }
    const size_t smem = step_smem_bytes(pbuf, a.boxes_tile_cells, algorithm);
    kStepFns[algorithm ? 1 : 0][table ? 1 : 0][a.nboxes == 1 ? 1 : 0][a.replay ? 1 : 0]<<<grid, kThreads, smem, st>>>(
        a, pbuf);
    return cudaGetLastError();
}

cudaError_t configure_step(int algorithm, uint32_t pbuf, uint32_t cells, int* blocks_per_sm)
{
    // The shared-memory limit is an attribute of the kernel function, shared by
    // every handle of the process: it only ever grows, to the largest tile any
    // handle uses (per device: the attribute is per context).
    static std::mutex mu;
    static size_t granted[64] = {};
    const size_t smem = step_smem_bytes(pbuf, cells, algorithm);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    {
        std::lock_guard<std::mutex> lock(mu);
        const int slot = dev & 63;
        if (smem > granted[slot]) {
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    for (int k = 0; k < 2; ++k)
                        for (int r = 0; r < 2; ++r) {
                            e = cudaFuncSetAttribute((const void*)kStepFns[i][j][k][r],
                                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                            if (e == cudaSuccess)   // all of the unified L1/shared array as shared memory
                                e = cudaFuncSetAttribute((const void*)kStepFns[i][j][k][r],
                                                         cudaFuncAttributePreferredSharedMemoryCarveout, 100);
                            if (e != cudaSuccess) return e;
                        }
            granted[slot] = smem;
        }
    }
    // load the kernels that step graphs capture before any capture begins
    cudaFuncAttributes attr;
    e = cudaFuncGetAttributes(&attr, (const void*)advance_kernel);
    // the run kernel: about a quarter of the unified array as shared memory (4
    // CTAs of 14 KB), the rest L1, which holds each batch's slots between its two passes
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j)
            for (int k = 0; k < 3; ++k)
                if (e == cudaSuccess)
                    e = cudaFuncSetAttribute((const void*)kRunFns[i][j][k], cudaFuncAttributePreferredSharedMemoryCarveout,
                                             27);
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        e = cudaFuncSetAttribute((const void*)kRunTapeFns[k], cudaFuncAttributePreferredSharedMemoryCarveout, 27);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, (const void*)sample_finalize_kernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&attr, (const void*)overflow_select_kernel);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        blocks_per_sm, (const void*)kStepFns[algorithm ? 1 : 0][0][1][0], kThreads, smem);
}

cudaError_t launch_profile(const SampleAcc* acc, const BoxDesc& b, uint64_t samples, float* profile, cudaStream_t st)
{
    const double inv = 1.0 / ((double)samples * (double)b.L[0] * (double)b.L[1]);
    profile_kernel<<<(unsigned)b.L[2], kThreads, 0, st>>>(acc, b, inv, profile);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_step(const BoxDesc& b, uint64_t step, uint64_t samples, float* lam, const uint32_t* key,
                                const uint32_t* lab, const uint32_t* ncell, const uint32_t* lab_count,
                                const float* dU, float4* cellsum, double* gsum, int grid, cudaStream_t st)
{
    const double w = 1.0 / ((double)samples * (double)b.L[0] * (double)b.L[1]);
    float4* const cell_axis = cellsum + b.C;
    adjoint_cells_kernel<<<grid, kThreads, 0, st>>>(b, step, lab_count, dU, w, cellsum, cell_axis);
    adjoint_pass1_kernel<<<grid, kThreads, 0, st>>>(b, b.N, lam, key, lab, cell_axis, cellsum, gsum);
    adjoint_pass2_kernel<<<grid, kThreads, 0, st>>>(b, b.N, lam, key, ncell, cellsum, cell_axis);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_finish(uint32_t n, const float* lam, const uint32_t* b0, float* out, int grid,
                                  cudaStream_t st)
{
    adjoint_finish_kernel<<<grid, kThreads, 0, st>>>(n, lam, b0, out);
    return cudaGetLastError();
}

cudaError_t launch_advance(DeviceState* state, unsigned steps, cudaStream_t st)
{
    advance_kernel<<<1, 32, 0, st>>>(state, steps);
    return cudaGetLastError();
}

cudaError_t launch_scatter(const StepArgs& a, const float* pos, const float* vel, uint64_t n_total, int grid,
                           cudaStream_t st)
{
    scatter_kernel<<<grid, kThreads, 0, st>>>(a, pos, vel, n_total);
    return cudaGetLastError();
}

cudaError_t launch_overflow_select(const StepArgs& a, Slot* in_slots, float4* ov_pos, float4* ov_vel,
                                   uint32_t* ov_head, int grid, cudaStream_t st)
{
    overflow_select_kernel<<<grid, kThreads, 0, st>>>(a, in_slots, ov_pos, ov_vel, ov_head);
    return cudaGetLastError();
}

cudaError_t launch_sample_finalize(float4* samp, SampleAcc* acc, uint64_t cells, int snapshot, int grid,
                                   cudaStream_t st, uint32_t* lab_count)
{
    sample_finalize_kernel<<<grid, kThreads, 0, st>>>(samp, acc, cells, snapshot, lab_count);
    return cudaGetLastError();
}

cudaError_t launch_mean_fields(const SampleAcc* acc, const BoxDesc& b, double inverse, float* density, float* velocity,
                               cudaStream_t st)
{
    const unsigned grid = (unsigned)std::min<uint64_t>((b.C + kThreads - 1) / kThreads, 4096);
    mean_fields_kernel<<<grid, kThreads, 0, st>>>(acc, b, inverse, density, velocity);
    return cudaGetLastError();
}

cudaError_t launch_layout(const StepArgs& a, const uint32_t* count, const Slot* slots,
                          uint32_t* offsets, uint64_t cells, uint64_t n_total, unsigned long long* status,
                          unsigned int* tile_counter, const float4* ov_pos, const float4* ov_vel, unsigned parity,
                          uint32_t* out_cell, uint32_t* out_slot, uint32_t* out_prev, uint32_t* out_id, int grid,
                          cudaStream_t st)
{
    const uint64_t tiles = (cells + kThreads * kScanItems - 1) / (kThreads * kScanItems);
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(unsigned long long) * tiles, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(tile_counter, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    scan_kernel<<<(unsigned)tiles, kThreads, 0, st>>>(count, a.boxes, a.nboxes, cells, offsets, status, tile_counter,
                                                      a.state);
    compact_kernel<<<grid, kThreads, 0, st>>>(a, count, slots, offsets, cells, n_total, out_cell, out_slot,
                                              out_prev, out_id);
    e = cudaMemsetAsync(tile_counter, 0, sizeof(unsigned int), st);   // now the count of placed list entries
    if (e != cudaSuccess) return e;
    compact_overflow_kernel<<<8, kThreads, 0, st>>>(a.boxes, a.nboxes, ov_pos, ov_vel, a.state, parity, a.ov_cap,
                                                    offsets, cells, n_total, a.total_slots + a.ext_cap, tile_counter,
                                                    out_cell, out_slot, out_prev, out_id);
    return cudaGetLastError();
}

cudaError_t launch_init(const BoxDesc* boxes, int nboxes, float* pos, float* vel, uint64_t n_total, int grid,
                        cudaStream_t st)
{
    init_kernel<<<grid, kThreads, 0, st>>>(boxes, nboxes, pos, vel, n_total);
    return cudaGetLastError();
}

cudaError_t launch_momentum_partial(const float* vel, uint64_t begin, uint64_t end, double* partial, int grid,
                                    cudaStream_t st)
{
    momentum_partial_kernel<<<grid, kThreads, 0, st>>>(vel, begin, end, partial);
    return cudaGetLastError();
}

cudaError_t launch_subtract(float* vel, uint64_t begin, uint64_t end, float mx, float my, float mz, int grid,
                            cudaStream_t st)
{
    subtract_kernel<<<grid, kThreads, 0, st>>>(vel, begin, end, mx, my, mz);
    return cudaGetLastError();
}

size_t scan_status_words(uint64_t cells) { return (cells + kThreads * kScanItems - 1) / (kThreads * kScanItems); }

// ------------------------------------------------------------------ allocation-free cell offsets
//
// scan_kernel with its scratch in a fixed file-scope array instead of buffers
// allocated by the caller: kStaticScanTiles look-back status words followed by
// the tile counter (one 64-bit word).  16384 tiles of 2048 cells = 33,554,432
// cells; 128 KiB of device memory per device, allocated with the module.
constexpr uint64_t kStaticScanTiles = 16384;
constexpr int kMaxScratchDevices = 64;
static_assert(kStaticScanTiles * kThreads * kScanItems == MPCD_GB_NOALLOC_MAX_CELLS,
              "static scan scratch and the ABI limit disagree");

static __device__ __align__(256) unsigned long long g_static_scan_scratch[kStaticScanTiles + 1];

// Address of this device's scratch: looked up once per device, with that device current.
static cudaError_t static_scan_scratch(int device, unsigned long long** out)
{
    static std::mutex mu;
    static unsigned long long* address[kMaxScratchDevices] = {};
    if (device < 0 || device >= kMaxScratchDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mu);
    if (!address[device]) {
        int current = -1;
        cudaError_t e = cudaGetDevice(&current);
        if (e != cudaSuccess) return e;
        if (current != device && (e = cudaSetDevice(device)) != cudaSuccess) return e;
        unsigned long long* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_static_scan_scratch);
        if (current != device) {
            const cudaError_t r = cudaSetDevice(current);
            if (e == cudaSuccess) e = r;
        }
        if (e != cudaSuccess) return e;
        address[device] = ptr;
    }
    *out = address[device];
    return cudaSuccess;
}

cudaError_t launch_cell_offsets_static(const StepArgs& a, const uint32_t* count, uint64_t cells, uint32_t* offsets,
                                       int device, cudaStream_t st)
{
    if (cells == 0 || cells > MPCD_GB_NOALLOC_MAX_CELLS) return cudaErrorInvalidValue;
    unsigned long long* scratch = nullptr;
    cudaError_t e = static_scan_scratch(device, &scratch);
    if (e != cudaSuccess) return e;
    const uint64_t tiles = (cells + kThreads * kScanItems - 1) / (kThreads * kScanItems);
    // the status words of the tiles in use and the tile counter start at zero
    e = cudaMemsetAsync(scratch, 0, sizeof(unsigned long long) * tiles, st);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(scratch + kStaticScanTiles, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    scan_kernel<<<(unsigned)tiles, kThreads, 0, st>>>(count, a.boxes, a.nboxes, cells, offsets, scratch,
                                                      reinterpret_cast<unsigned int*>(scratch + kStaticScanTiles),
                                                      a.state);
    return cudaGetLastError();
}

}  // namespace mpcd_gb
