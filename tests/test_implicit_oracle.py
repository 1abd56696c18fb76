"""Crank-Nicolson and implicit tensor diffusion (incflo.diffusion_type 1 and 2)
in the oracle, for both schemes.

Known answer: a shear wave u_x = A sin(2 pi z / L) in a triply periodic box is
not advected and stays divergence-free, and the discrete tensor operator maps
it to lambda u_x with lambda = -nu (2 - 2 cos(2 pi / nz)) / dz^2.  One step
therefore multiplies it by the scheme's amplification factor: 1 + dt lambda +
(dt lambda)^2 / 2 (explicit with the RK2 correction, or MOL's Heun step),
(1 + dt lambda / 2) / (1 - dt lambda / 2) (Crank-Nicolson) and
1 / (1 - dt lambda) (implicit), the predictor_rhs factors of
src/equation_systems/CompRHSOps.H:46-57 and the solve of
src/equation_systems/DiffusionOps.cpp:154-159.
"""
import math

import numpy as np
import pytest

from kynema_sgf_gb300 import decks


def shear_deck(n, nu, dt, dtype, scheme):
    d = decks.tgv(n, steps=10, cfl=0.45).replace("incflo.physics = TaylorGreenVortex", "incflo.physics = FreeStream")
    d = d.replace("transport.viscosity = 0.000625", "transport.viscosity = %r" % nu)
    d = d.replace("time.fixed_dt = -1", "time.fixed_dt = %r" % dt)
    d = d.replace("incflo.diffusion_type = 0", "incflo.diffusion_type = %d" % dtype)
    d += "diffusion.mg_rtol = 1e-14\n"  # the known answer is checked well below the default solver tolerance
    return decks.mol(d) if scheme == "mol" else d


def shear_field(n, amp=0.7):
    z = (np.arange(n) + 0.5) * (2 * math.pi / n)
    v = np.zeros((3, n, n, n))
    v[0] = amp * np.sin(z)[:, None, None]
    return v


def factor(dtype, x):
    if dtype == 0:
        return 1 + x + 0.5 * x * x
    if dtype == 1:
        return (1 + 0.5 * x) / (1 - 0.5 * x)
    return 1 / (1 - x)


@pytest.mark.parametrize("scheme", ["godunov", "mol"])
@pytest.mark.parametrize("dtype", [0, 1, 2])
def test_shear_wave_amplification(oracle_mod, scheme, dtype):
    n, nu, dt = 16, 0.05, 0.05
    o = oracle_mod.Oracle(shear_deck(n, nu, dt, dtype, scheme))
    v0 = shear_field(n)
    o.set_field("velocity", v0)
    o.InitData()
    h = 2 * math.pi / n
    lam = -nu * (2 - 2 * math.cos(2 * math.pi / n)) / (h * h)
    steps = 3
    for _ in range(steps):
        assert o.step()
    v = o.get_field("velocity")
    expect = factor(dtype, dt * lam) ** steps * v0
    assert np.abs(v - expect).max() < 1e-11 * np.abs(v0).max()
    if dtype:
        assert o.scalar("diff_iters") >= 1
        assert o.scalar("diff_res") <= max(2.2e-14, 1e-14 * max(o.scalar("diff_res0"), o.scalar("diff_rhs_norm")))


def test_crank_nicolson_close_to_explicit(oracle_mod):
    base = decks.tgv(24, steps=6, cfl=0.45).replace("time.fixed_dt = -1", "time.fixed_dt = 0.02")
    outs = {}
    for t in (0, 1, 2):
        o = oracle_mod.Oracle(base.replace("incflo.diffusion_type = 0", "incflo.diffusion_type = %d" % t))
        o.InitData()
        for _ in range(4):
            o.step()
        outs[t] = o.get_field("velocity")
    ref = np.linalg.norm(outs[0])
    assert np.linalg.norm(outs[1] - outs[0]) / ref < 1e-8   # both second order in the (small) diffusion term
    assert np.linalg.norm(outs[2] - outs[0]) / ref < 1e-4


def test_default_is_crank_nicolson_and_drops_diffusion_cfl(oracle_mod):
    d = decks.tgv(16, steps=2).replace("incflo.diffusion_type = 0\n", "").replace("transport.viscosity = 0.000625",
                                                                                   "transport.viscosity = 0.5")
    o = oracle_mod.Oracle(d)
    o.InitData()
    assert o.step()
    assert o.scalar("diff_iters") >= 1          # the solve ran: Crank-Nicolson by default
    assert o.scalar("diff_cfl") == 0.0           # no diffusion CFL without explicit diffusion
    e = oracle_mod.Oracle(d + "incflo.diffusion_type = 0\n")
    e.InitData()
    e.step()
    assert e.scalar("diff_cfl") > 0.0 and e.scalar("dt") < o.scalar("dt")
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.Oracle(d + "incflo.diffusion_type = 3\n")
