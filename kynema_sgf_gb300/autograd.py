"""torch.autograd.Function wrappers of the advance's reverse mode.

A thin harness over the C ABI (ks_adjoint_step, ks_adjoint_run,
ks_get_ct_gradient): all arithmetic runs in the library's CUDA kernels; torch
only carries the device tensors between calls and chains the steps.

``AdvanceStep``  one step (velocity, gp) -> (velocity', gp') of a handle,
                 differentiable in velocity, gp and the disk thrust
                 coefficients; autograd stores every step's input state.
``AdjointRun``   J after ``nsteps`` steps as one node whose backward returns
                 dJ/dct computed with binomial checkpointing inside the
                 library (``snapshots`` device slots).
``box_mean_ke``  the objective (mean 0.5 |u|^2 over a box of cells) as a
                 torch expression, for chains of ``AdvanceStep``.
"""
import math

import torch


def _f64(t):
    return t.detach().to(dtype=torch.float64).contiguous()


def _field(sim, name, like):
    out = torch.empty(sim.layout(name), dtype=torch.float64, device=like.device)
    sim.get_field(name, out=out)
    return out


class AdvanceStep(torch.autograd.Function):
    """x^{n+1} = step(x^n; ct) for the handle ``sim`` (an Incflo whose deck is
    in the differentiable configuration)."""

    @staticmethod
    def forward(ctx, sim, velocity, gp, ct):
        sim.set_field("velocity", _f64(velocity))
        sim.set_field("gp", _f64(gp))
        sim.set_disk_ct(ct.detach().cpu().tolist())
        if not sim.step():
            raise RuntimeError("the deck's time.max_step / stop_time ended the run")
        ctx.sim = sim
        ctx.save_for_backward(_f64(velocity), _f64(gp), ct.detach().cpu().to(torch.float64))
        return _field(sim, "velocity", velocity), _field(sim, "gp", gp)

    @staticmethod
    def backward(ctx, velocity_bar, gp_bar):
        sim = ctx.sim
        velocity, gp, ct = ctx.saved_tensors
        sim.set_field("velocity", velocity)
        sim.set_field("gp", gp)
        sim.set_disk_ct(ct.tolist())
        sim.adjoint_reset()
        if velocity_bar is not None:
            sim.set_field("velocity_adjoint", _f64(velocity_bar))
        if gp_bar is not None:
            sim.set_field("gp_adjoint", _f64(gp_bar))
        sim.adjoint_step()
        ub = _field(sim, "velocity_adjoint", velocity)
        gpb = _field(sim, "gp_adjoint", gp)
        ctb = torch.as_tensor(sim.ct_gradient(), dtype=torch.float64)
        return None, ub, gpb, ctb


class AdjointRun(torch.autograd.Function):
    """J(ct) after ``nsteps`` steps from the handle's current state; backward
    gives dJ/dct from ks_adjoint_run (binomial checkpoints in device memory).
    The handle's forward state is restored to the initial state afterwards so
    that repeated evaluations start from the same point."""

    @staticmethod
    def forward(ctx, sim, ct, nsteps, snapshots):
        v0 = torch.empty(sim.layout("velocity"), dtype=torch.float64)
        g0 = torch.empty(sim.layout("gp"), dtype=torch.float64)
        p0 = torch.empty(sim.layout("p"), dtype=torch.float64)
        sim.get_field("velocity", out=v0)
        sim.get_field("gp", out=g0)
        sim.get_field("p", out=p0)
        sim.set_disk_ct(ct.detach().cpu().tolist())
        J = sim.adjoint_run(int(nsteps), int(snapshots))
        ctx.grad = torch.as_tensor(sim.ct_gradient(), dtype=torch.float64)
        sim.set_field("velocity", v0)
        sim.set_field("gp", g0)
        sim.set_field("p", p0)
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, J_bar):
        return None, J_bar * ctx.grad, None, None


def box_cells(lo, hi, prob_lo, dx, n):
    """Index ranges (k, j, i slices) of the cells whose centres lie in [lo, hi]."""
    sl = []
    for m in range(3):
        a = max(0, int(math.ceil((lo[m] - prob_lo[m]) / dx[m] - 0.5)))
        b = min(n[m] - 1, int(math.floor((hi[m] - prob_lo[m]) / dx[m] - 0.5)))
        sl.append(slice(a, b + 1))
    return sl[2], sl[1], sl[0]


def box_mean_ke(velocity, cells):
    """Mean of 0.5 |u|^2 over the cells (velocity shaped (3, nz, ny, nx))."""
    k, j, i = cells
    v = velocity[:, k, j, i]
    return 0.5 * (v * v).sum() / (v.shape[1] * v.shape[2] * v.shape[3])
