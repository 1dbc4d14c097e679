"""Adjoint of the sampled velocity profile (cudampcd_gb300.adjoint) on the GPU.

Loss: MSE of the sampled x-velocity profile over the fluid layers against the
analytic Poiseuille parabola with a 10 % larger peak.  Gradients are taken with
respect to the body force g and all initial velocities.

1. The FP64 reference.  The events the forward trajectory fixed are dumped by the
   test hook mpcd_gb_profile_tape, and the same affine map is rebuilt in torch
   float64:
   - collision cells and their occupancy N_c;
   - rotation axes, from the Philox draw model of the oracle;
   - lab cells and counts;
   - bounce-backs.
   Its vector-Jacobian product with the GPU's dL/dU must match the GPU adjoint.
2. Central finite differences with common random numbers.  The same seed and
   start step are used, so every Philox draw is shared.  They are run through the
   real simulation, on the body force and on a random direction of the initial
   velocities.  The perturbations are small enough that no discrete event flips,
   which is checked by comparing the event tapes of the runs.  MPCD is chaotic:
   at the 64 x 64 x 32 channel size, perturbations that FP32 can resolve flip
   thousands of events, and a single-trajectory difference quotient is then
   dominated by them.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle as O
from cudampcd_gb300 import capi

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

BOUNCE = 0x80000000
NONE = 0xFFFFFFFF
ALPHA = 2.0 * math.pi / 3.0


def target_profile(lz_container: int, drag: float, n: int, dt: float) -> torch.Tensor:
    """1.1 x the analytic Poiseuille profile n g (h^2 - z^2) / (2 eta) at the layer centres."""
    eta = (1.0 - math.cos(ALPHA)) / (18.0 * dt) * (n - 1 + math.exp(-n))
    h = lz_container / 2.0 - 1.0
    z = torch.arange(lz_container, dtype=torch.float64) + 0.5 - lz_container / 2.0
    u = n * drag * (h * h - z * z) / (2.0 * eta)
    return 1.1 * u


def loss_of(U: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    return ((U[1:-1].double() - target[1:-1].to(U.device)) ** 2).mean()


def srd_axes(seed: int, step: int, refs: np.ndarray) -> np.ndarray:
    """Rotation axes of the Philox draw model (purpose 2), in float64."""
    out = np.zeros((len(refs), 3))
    key = [seed & 0xFFFFFFFF, seed >> 32]
    for i, r in enumerate(refs):
        o = O.philox([int(r), step & 0xFFFFFFFF, 2 | ((step >> 32) << 8), 0], key)
        u0, u1 = (o[0] >> 8) * 2.0 ** -24, (o[1] >> 8) * 2.0 ** -24
        z = 1.0 - 2.0 * u0
        rho = math.sqrt(max(0.0, 1.0 - z * z))
        out[i] = (rho * math.cos(2 * math.pi * u1), rho * math.sin(2 * math.pi * u1), z)
    return out


def fp64_profile(tape, L, seed, s0, dt, V0, g):
    """The fixed-event affine map V0, g -> U in float64 (ghost velocities, a constant, left out)."""
    key, lab, ncell, cnt, b0 = tape
    S, N = key.shape
    Lx, Ly, Lz = L
    P = V0 * torch.from_numpy(np.where(b0 & BOUNCE, -1.0, 1.0))[:, None]
    U = torch.zeros(Lz, dtype=torch.float64)
    cos_a, sin_a = math.cos(ALPHA), math.sin(ALPHA)
    for t in range(S):
        k = key[t]
        coll = k != NONE
        kc = torch.from_numpy(k[coll].astype(np.int64))
        cells = np.unique(k[coll])
        z, col = cells % Lz, cells // Lz
        refs = (col % Lx) + Lx * ((col // Lx) + Ly * z)
        axes = np.zeros((Lx * Ly * Lz, 3))
        axes[cells] = srd_axes(seed, s0 + t, refs)
        idx = torch.from_numpy(np.nonzero(coll)[0])
        Pc = P[idx]
        sums = torch.zeros((Lx * Ly * Lz, 3), dtype=torch.float64).index_add(0, kc, Pc)
        u = sums[kc] / torch.from_numpy(ncell[t][k[coll]].astype(np.float64))[:, None]
        a = torch.from_numpy(axes[k[coll]])
        w = Pc - u
        d = (w * a).sum(1, keepdim=True)
        Rw = d * a + cos_a * (w - d * a) + sin_a * torch.cross(w, a, dim=1)
        Q = P.clone()
        Q[idx] = u + Rw
        Q[idx, 0] = Q[idx, 0] + g * dt
        labc = lab[t] & ~np.uint32(BOUNCE)
        w_lab = torch.from_numpy(1.0 / cnt[t][labc].astype(np.float64))
        U = U.index_add(0, torch.from_numpy((labc % Lz).astype(np.int64)), Q[:, 0] * w_lab)   # storage order
        P = torch.where(torch.from_numpy(lab[t] & BOUNCE != 0)[:, None], -Q, Q)
    return U / (S * Lx * Ly)


def run_profile(h, pos, v0, drag, steps, every):
    from cudampcd_gb300.adjoint import channel_profile

    return channel_profile(h, pos, v0, drag, steps, every)


def test_adjoint_matches_fp64_reference_on_small_box():
    L, n, drag0, dt, seed, S, K = (8, 8, 10), 10, 1e-3, 0.02, 21, 40, 10
    h = capi.Handle(L=L, periodic=(1, 1, 0), n=n, dt=dt, drag=drag0, seed=seed)
    try:
        s0 = h.step_index
        pos = torch.from_numpy(h.positions()).cuda()
        v0 = torch.from_numpy(h.velocities()).cuda().requires_grad_(True)
        g = torch.tensor(drag0, dtype=torch.float64, device="cuda", requires_grad=True)
        U = run_profile(h, pos, v0, g, S, K)
        target = target_profile(L[2], drag0, n, dt)
        Ud = U.detach().double().requires_grad_(True)
        loss_of(Ud, target).backward()
        dU = Ud.grad.cpu()
        loss_of(U, target).backward()
        tape = h.profile_tape(S)

        V0 = v0.detach().cpu().double().requires_grad_(True)
        g64 = torch.tensor(drag0, dtype=torch.float64, requires_grad=True)
        U64 = fp64_profile(tape, L, seed, s0, dt, V0, g64)
        ref_v, ref_g = torch.autograd.grad(U64, [V0, g64], grad_outputs=dU)
        gv = v0.grad.detach().cpu().double()
        err_v = ((gv - ref_v).norm() / ref_v.norm()).item()
        err_g = abs(g.grad.item() - ref_g.item()) / abs(ref_g.item())
        print(f"FP64 reference: |dV0| rel err {err_v:.2e}, dg rel err {err_g:.2e} (dg = {g.grad.item():.6e})")
        assert err_v < 1e-4 and err_g < 1e-4
    finally:
        h.close()


def _loss_and_tape(h, pos, v0, drag, S, K, target):
    with torch.no_grad():
        U = run_profile(h, pos, v0, torch.tensor(drag, dtype=torch.float64, device="cuda"), S, K)
    return loss_of(U, target).item(), h.profile_tape(S)


def _same_events(a, b) -> bool:
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def test_adjoint_matches_central_differences_with_common_random_numbers():
    """Central differences through the real simulation, same seed and start step
    (every Philox draw shared), with the largest perturbation of a short list for
    which no discrete event flips -- checked by comparing the full event tapes of
    the runs.  The map is then affine and the loss quadratic, so central
    differences are exact up to FP32 rounding.  A small box and a short horizon
    keep event flips rare at perturbations FP32 still resolves.

    The noise floor of a difference quotient is the FP32 profile: U is returned in
    float32 and its per-step cell sums are float atomics whose rounding varies from
    run to run, a few 1e-9 absolute on a profile of a few 1e-2.  The velocity
    direction is therefore chosen to move the loss as much as the event budget
    allows: eight particles, each component perturbed along the sign of the
    adjoint's own gradient (so dL/dV0 . delta = sum |dL/dV0_ij| over them, first
    order in any error of the adjoint, not a random projection), and each loss is
    the mean of five runs.  Bound 1e-3 on both gradients; the FP64 autograd test
    above pins the adjoint itself (to 1e-4, measured 6e-7)."""
    L, n, drag0, dt, seed, S, K = (4, 4, 6), 10, 1e-3, 0.02, 9, 12, 4
    h = capi.Handle(L=L, periodic=(1, 1, 0), n=n, dt=dt, drag=drag0, seed=seed)
    try:
        pos = torch.from_numpy(h.positions()).cuda()
        base_v = torch.from_numpy(h.velocities()).cuda()
        target = target_profile(L[2], drag0, n, dt)
        v0 = base_v.clone().requires_grad_(True)
        g = torch.tensor(drag0, dtype=torch.float64, device="cuda", requires_grad=True)
        loss_of(run_profile(h, pos, v0, g, S, K), target).backward()
        _, tape0 = _loss_and_tape(h, pos, base_v, drag0, S, K, target)

        def mean_loss(v, drag):
            runs = [_loss_and_tape(h, pos, v, drag, S, K, target) for _ in range(5)]
            same = all(_same_events(t, tape0) for _, t in runs)
            return float(np.mean([l for l, _ in runs])), same

        def central(perturb, eps_list):
            for eps in eps_list:
                lp, same_p = mean_loss(*perturb(eps))
                lm, same_m = mean_loss(*perturb(-eps))
                if same_p and same_m:
                    return (lp - lm) / (2 * eps), eps
            pytest.fail("every perturbation flipped an event")

        fd_g, eps_g = central(lambda e: (base_v, drag0 + e), [5e-4, 2e-4, 1e-4, 5e-5])
        err_g = abs(g.grad.item() - fd_g) / abs(fd_g)

        gen = torch.Generator(device="cuda").manual_seed(3)
        delta = torch.zeros_like(base_v)
        who = torch.randperm(h.N, generator=gen, device="cuda")[:8]
        delta[who] = torch.sign(v0.grad[who])
        fd_v, eps_v = central(lambda e: (base_v + e * delta, drag0), [2e-2, 1e-2, 5e-3, 2e-3, 1e-3, 5e-4])
        ad_v = (v0.grad * delta).sum().item()
        err_v = abs(ad_v - fd_v) / abs(fd_v)
        print(f"central differences: dL/dg adjoint {g.grad.item():.6e} FD {fd_g:.6e} (eps {eps_g:g}) rel {err_g:.2e}; "
              f"dL/dV0 . delta adjoint {ad_v:.6e} FD {fd_v:.6e} (eps {eps_v:g}) rel {err_v:.2e}")
        assert err_g < 1e-3
        assert err_v < 1e-3
    finally:
        h.close()


def test_differentiable_channel_workload_runs():
    """The 64 x 64 x 32 (+2 walls) channel, n = 10, 200 steps, checkpoints every 20:
    finite gradients, and the adjoint reproduces the forward's events (the
    backward's recomputation is bit-identical to the forward, so a second forward
    gives the same profile)."""
    L, n, drag0, dt, seed, S, K = (64, 64, 34), 10, 1e-3, 0.02, 5, 200, 20
    h = capi.Handle(L=L, periodic=(1, 1, 0), n=n, dt=dt, drag=drag0, seed=seed)
    try:
        pos = torch.from_numpy(h.positions()).cuda()
        v0 = torch.from_numpy(h.velocities()).cuda().requires_grad_(True)
        g = torch.tensor(drag0, dtype=torch.float64, device="cuda", requires_grad=True)
        target = target_profile(L[2], drag0, n, dt)
        U1 = run_profile(h, pos, v0, g, S, K)
        loss_of(U1, target).backward()
        assert torch.isfinite(v0.grad).all() and math.isfinite(g.grad.item())
        assert g.grad.item() < 0   # the flow is slower than the target: more force lowers the loss
        with torch.no_grad():
            U2 = run_profile(h, pos, v0.detach(), g.detach(), S, K)
        assert torch.allclose(U1, U2, rtol=0, atol=1e-6)
    finally:
        h.close()
