"""torch.autograd binding of the hand-written adjoint (include/xrt_diff.h).

`rollout(solver, frames, x0, v0, mass, stretch_compliance, bend_compliance)` steps a started
ClothSolver `frames` frames from the given state and parameters and returns the final positions
and velocities as tensors; their backward is the library's reverse pass (xrt_backward), which
replays each frame from its checkpoint on the GPU.  No torch op runs on the simulation path:
the tensors only carry values across the C ABI.

Inputs map to the library's parameters as
  x0, v0              (V, 3)   xrt_set_state
  mass                (V,)     xrt_set_inv_mass with 1 / mass on free vertices; pinned vertices
                               (inverse mass 0 in the solver) stay pinned, their mass gradient is 0
  stretch_compliance  (E,)     xrt_set_compliance(kind 0), xrt_get_edges order
  bend_compliance     (B,)     xrt_set_compliance(kind 1), xrt_get_bends order
"""
from typing import Optional, Tuple

import numpy as np
import torch

from .solver import ClothSolver


def _host(t: Optional[torch.Tensor]) -> Optional[np.ndarray]:
    if t is None:
        return None
    return np.ascontiguousarray(t.detach().to("cpu", torch.float32).numpy())


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, solver: ClothSolver, frames: int, x0, v0, mass, stretch_compliance,
                bend_compliance):
        pinned = solver.inv_mass() == 0.0
        m = _host(mass)
        w = np.where(pinned, 0.0, 1.0 / np.where(pinned, 1.0, m)).astype(np.float32)
        solver.set_compliance(0, _host(stretch_compliance))
        ctx.bends = bend_compliance.numel() > 0
        if ctx.bends:  # an empty tensor keeps the solver's bend compliance
            solver.set_compliance(1, _host(bend_compliance))
        solver.set_inv_mass(w)
        solver.set_state(_host(x0), _host(v0))
        solver.diff_begin()
        solver.step(frames)
        ctx.solver = solver
        ctx.devices = [t.device for t in (x0, v0, mass, stretch_compliance, bend_compliance)]
        x = torch.from_numpy(solver.host_positions()).to(x0.device)
        v = torch.from_numpy(solver.host_velocities()).to(x0.device)
        return x, v

    @staticmethod
    def backward(ctx, gx, gv):
        s: ClothSolver = ctx.solver
        V = s.sizes().num_vertices
        gx = torch.zeros(V, 3) if gx is None else gx
        g = s.backward(_host(gx), _host(gv))
        d = ctx.devices
        t = lambda a, k: torch.from_numpy(np.asarray(a)).to(d[k])  # noqa: E731
        return (None, None, t(g["position"], 0), t(g["velocity"], 1), t(g["mass"], 2),
                t(g["stretch_compliance"], 3), t(g["bend_compliance"], 4) if ctx.bends else None)


def rollout(solver: ClothSolver, frames: int, x0: torch.Tensor, v0: torch.Tensor,
            mass: torch.Tensor, stretch_compliance: torch.Tensor,
            bend_compliance: Optional[torch.Tensor] = None) -> Tuple[torch.Tensor, torch.Tensor]:
    """Final (positions, velocities) after `frames` frames; differentiable with respect to every
    tensor argument.  The solver must be started, without particle self-collision, Quality
    repulsion or bindings (xrt_diff_begin rejects those frames).  Without `bend_compliance` the
    solver's bend compliance is kept and not differentiated."""
    if bend_compliance is None:
        bend_compliance = torch.zeros(0, dtype=torch.float32)
    return _Rollout.apply(solver, int(frames), x0, v0, mass, stretch_compliance, bend_compliance)
