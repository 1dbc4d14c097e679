"""Differentiable sampled velocity profile of an SRD Poiseuille channel.

`ChannelProfile` is a torch.autograd.Function over the GB300 step.  Its forward
sets the initial state and the body force, runs `steps` sampled steps through
`mpcd_gb_profile_forward`, and returns the x-velocity profile U(z) of the
container layers.  The profile is averaged over x, y and the steps, from the
per-cell means of every step, as the reference samples them
(simulation_kernels.cu:150-204).

Its backward calls the hand-written adjoint `mpcd_gb_profile_backward`.  The
adjoint holds the discrete events of the forward trajectory fixed:
- cell assignments;
- grid shifts and rotation axes, replayed from the Philox counters instead of
  stored;
- ghost counts;
- wall bounces.

The state is checkpointed every `checkpoint_every` steps. The backward recomputes
one segment at a time, then sweeps it in reverse. It returns dL/dV0 for every
particle and dL/d(drag).
"""
from __future__ import annotations

import torch

from . import capi


class ChannelProfile(torch.autograd.Function):
    """U = ChannelProfile.apply(v0, drag, handle, positions, steps, checkpoint_every, start_step)

    v0, positions: (N, 3) float32 CUDA tensors (by particle id); drag: 0-d tensor;
    handle: a single-box SRD `capi.Handle` on the same device; start_step: the
    Philox step index of the first step (equal start steps give common random
    numbers).  Returns U, a float32 tensor of the container's Lz layers.
    """

    @staticmethod
    def forward(ctx, v0, drag, handle, positions, steps, checkpoint_every, start_step=0):
        v0c = v0.detach().contiguous().float()
        pos = positions.detach().contiguous().float()
        lz = int(handle.params.volume_size[2])
        profile = torch.empty(lz, dtype=torch.float32, device=v0.device)
        torch.cuda.current_stream(v0.device).synchronize()   # the handle runs on its own stream
        handle.set_drag(float(drag))
        handle.set_step(int(start_step))
        handle.set_particles_device(pos.data_ptr(), v0c.data_ptr())
        handle.profile_forward(int(steps), int(checkpoint_every), profile.data_ptr())   # returns when done
        ctx.handle = handle
        ctx.drag_meta = (drag.dtype, drag.device)
        ctx.n = v0.shape[0]
        return profile

    @staticmethod
    def backward(ctx, grad_profile):
        g = grad_profile.detach().contiguous().float()
        dv0 = torch.empty((ctx.n, 3), dtype=torch.float32, device=g.device)
        torch.cuda.current_stream(g.device).synchronize()
        ddrag = ctx.handle.profile_backward(g.data_ptr(), dv0.data_ptr())   # returns when done
        dtype, device = ctx.drag_meta
        return dv0, torch.tensor(ddrag, dtype=dtype, device=device), None, None, None, None, None


def channel_profile(handle: capi.Handle, positions: torch.Tensor, v0: torch.Tensor, drag: torch.Tensor,
                    steps: int, checkpoint_every: int, start_step: int = 0) -> torch.Tensor:
    """Differentiable x-velocity profile U(z) of `steps` sampled steps from (positions, v0),
    starting at Philox step `start_step`."""
    return ChannelProfile.apply(v0, drag, handle, positions, steps, checkpoint_every, start_step)
