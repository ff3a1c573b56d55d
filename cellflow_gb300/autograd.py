"""torch.autograd binding of the differentiable rollout and the soft radial
distribution (cf_rollout_forward / cf_rollout_backward / cf_rdf /
cf_rdf_backward).

A thin binding: torch supplies device memory and the stream, the library's
kernels do the work.  Positions and velocities are (n, 3) float32 CUDA
tensors in the world's particle order; types come from the world.  The force
table is the (T, T) table the step uses (ParticleSimulation.cu:116), and
`phys` holds the six differentiable step parameters in GRAD_PARAMS order.
No counterpart in the reference.
"""

from __future__ import annotations

import dataclasses

import numpy as np
import torch

from ._lib import GRAD_PARAMS
from .world import ParticleSimulation, SimulationParams


class _LibraryStream:
    """Runs a block on a torch stream that the world also uses, ordered after the
    caller's current stream on entry and before it on exit.  (The caller's stream
    may be the legacy default stream, which the world's own non-blocking stream
    would not wait for.)  Tensors made inside and used after are recorded on the
    caller's stream."""

    def __init__(self, sim: ParticleSimulation):
        self.sim = sim

    def __enter__(self):
        s = getattr(self.sim, "_torch_stream", None)
        if s is None:
            s = torch.cuda.Stream()
            self.sim._torch_stream = s
            self.sim.set_stream(s.cuda_stream)
        self.caller = torch.cuda.current_stream()
        s.wait_stream(self.caller)
        self.ctx = torch.cuda.stream(s)
        self.ctx.__enter__()
        return self

    def keep(self, *tensors):
        for t in tensors:
            t.record_stream(self.caller)
        return tensors

    def __exit__(self, *exc):
        s = torch.cuda.current_stream()
        self.ctx.__exit__(*exc)
        self.caller.wait_stream(s)
        return False


def _as4(x: torch.Tensor | None, n: int) -> torch.Tensor:
    out = torch.zeros((n, 4), dtype=torch.float32, device="cuda")
    if x is not None:
        out[:, :3] = x
    return out


class Rollout(torch.autograd.Function):
    """(pos0, vel0, table, phys) -> (pos_K, vel_K) after `steps` steps."""

    @staticmethod
    def forward(ctx, pos, vel, table, phys, sim: ParticleSimulation, params: SimulationParams, steps: int,
                checkpoint_every: int = 16):
        n = sim.getParticleCount()
        values = {name: float(v) for name, v in zip(GRAD_PARAMS, phys.detach().cpu().tolist())}
        p = dataclasses.replace(params, **values)
        sim.setForceTable(table.detach().to("cpu", torch.float32).numpy())
        with _LibraryStream(sim) as ls:
            pos4, vel4 = _as4(pos.detach(), n), _as4(vel.detach(), n)
            out_p, out_v = torch.empty_like(pos4), torch.empty_like(vel4)
            sim.rollout_forward(p, steps, checkpoint_every, pos4.data_ptr(), vel4.data_ptr(), out_p.data_ptr(),
                                out_v.data_ptr())
            xk, vk = ls.keep(out_p[:, :3].contiguous(), out_v[:, :3].contiguous())
        ctx.sim = sim
        ctx.table_meta = (table.dtype, table.device)
        ctx.phys_meta = (phys.dtype, phys.device)
        return xk, vk

    @staticmethod
    def backward(ctx, gpos, gvel):
        sim = ctx.sim
        n = sim.getParticleCount()
        with _LibraryStream(sim) as ls:
            g4 = _as4(gpos, n) if gpos is not None else None
            gv4 = _as4(gvel, n) if gvel is not None else None
            out_g, out_v = torch.empty((n, 4), dtype=torch.float32, device="cuda"), torch.empty(
                (n, 4), dtype=torch.float32, device="cuda")
            gF, gp = sim.rollout_backward(g4.data_ptr() if g4 is not None else None,
                                          gv4.data_ptr() if gv4 is not None else None, out_g.data_ptr(),
                                          out_v.data_ptr())
            gx0, gv0 = ls.keep(out_g[:, :3].contiguous(), out_v[:, :3].contiguous())
        tdt, tdev = ctx.table_meta
        pdt, pdev = ctx.phys_meta
        return (gx0, gv0,
                torch.from_numpy(np.ascontiguousarray(gF)).to(device=tdev, dtype=tdt),
                torch.from_numpy(gp.astype(np.float64)).to(device=pdev, dtype=pdt), None, None, None, None)


class RadialDistribution(torch.autograd.Function):
    """pos (n, 3) -> soft type-resolved radial distribution (T, T, bins)."""

    @staticmethod
    def forward(ctx, pos, sim: ParticleSimulation, bins: int, r_max: float):
        n, T = sim.getParticleCount(), sim.getNumParticleTypes()
        with _LibraryStream(sim) as ls:
            pos4 = _as4(pos.detach(), n)
            hist = torch.empty((T, T, bins), dtype=torch.float32, device="cuda")
            sim.rdf(bins, r_max, hist.data_ptr(), pos4.data_ptr())
            ls.keep(hist, pos4)
        ctx.sim, ctx.bins, ctx.r_max = sim, bins, r_max
        ctx.save_for_backward(pos4)
        return hist

    @staticmethod
    def backward(ctx, ghist):
        (pos4,) = ctx.saved_tensors
        sim = ctx.sim
        with _LibraryStream(sim) as ls:
            gh = ghist.to(torch.float32).contiguous()
            g4 = torch.empty_like(pos4)
            sim.rdf_backward(ctx.bins, ctx.r_max, gh.data_ptr(), g4.data_ptr(), pos4.data_ptr())
            (gx,) = ls.keep(g4[:, :3].contiguous())
        return gx, None, None, None


def rollout(pos, vel, table, phys, sim, params, steps, checkpoint_every=16):
    return Rollout.apply(pos, vel, table, phys, sim, params, steps, checkpoint_every)


def radial_distribution(pos, sim, bins=32, r_max=0.2):
    return RadialDistribution.apply(pos, sim, bins, r_max)


def phys_tensor(params: SimulationParams, dtype=torch.float64) -> torch.Tensor:
    """The differentiable step parameters of `params` in GRAD_PARAMS order."""
    return torch.tensor([float(getattr(params, name)) for name in GRAD_PARAMS], dtype=dtype)
