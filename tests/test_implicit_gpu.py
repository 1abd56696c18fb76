"""GPU: Crank-Nicolson and implicit tensor diffusion (multigrid solve of
rho u - dt_diff divtau(u) = rho u_rhs) against the shear-wave known answer and
against the oracle (its Jacobi solve of the same discrete system)."""
import math

import numpy as np
import pytest

from kynema_sgf_gb300 import decks

from test_implicit_oracle import factor, shear_deck, shear_field

pytestmark = pytest.mark.gpu
TOL = 1e-9


def rel(a, b, name=""):
    if name == "p":
        a = a - a.mean()
        b = b - b.mean()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def check(g, o, names, tol=TOL):
    for f in names:
        e = rel(g.get_field(f), o.get_field(f), f)
        assert e < tol, "%s rel err %.3e" % (f, e)


@pytest.mark.parametrize("scheme", ["godunov", "mol"])
@pytest.mark.parametrize("dtype", [1, 2])
def test_shear_wave_amplification(cuda_dev, scheme, dtype):
    n, nu, dt = 16, 0.05, 0.05
    g = cuda_dev.Incflo(shear_deck(n, nu, dt, dtype, scheme))
    v0 = shear_field(n)
    g.set_field("velocity", v0)
    g.InitData()
    h = 2 * math.pi / n
    lam = -nu * (2 - 2 * math.cos(2 * math.pi / n)) / (h * h)
    for _ in range(3):
        assert g.step()
    assert np.abs(g.get_field("velocity") - factor(dtype, dt * lam) ** 3 * v0).max() < 1e-11 * np.abs(v0).max()
    assert g.scalar("diff_iters") >= 1


@pytest.mark.parametrize("case", ["tgv_cn", "tgv_implicit_mol", "abl_cn", "abl_cn_mol", "tgv_stiff"])
def test_implicit_parity(cuda_dev, oracle_mod, case):
    if case.startswith("tgv"):
        d = decks.tgv(32 if case != "tgv_stiff" else 16, steps=4, cfl=0.45)
    else:
        d = decks.abl(32, 32, 16, steps=4, cfl=0.45)
    d = d.replace("incflo.diffusion_type = 0", "incflo.diffusion_type = %d" % (2 if "implicit" in case else 1))
    if case == "tgv_stiff":  # dt nu / h^2 ~ 0.5: the multigrid's coarse levels carry the solve
        d = d.replace("transport.viscosity = 0.000625", "transport.viscosity = 0.3")
    if case.endswith("mol"):
        d = decks.mol(d)
    # the two sides solve with different iterations; compare them well below the default tolerance
    d += "diffusion.mg_rtol = 1e-13\n"
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    g.InitData()
    o.InitData()
    check(g, o, ["velocity", "p", "gp"])
    for _ in range(3):
        assert g.step() and o.step()
        assert abs(g.scalar("dt") - o.scalar("dt")) <= 1e-12 * o.scalar("dt")
        check(g, o, ["velocity", "p", "gp", "velocity_mueff"])
        assert g.scalar("diff_res") <= max(2.2e-14, 1e-13 * max(g.scalar("diff_res0"), g.scalar("diff_rhs_norm")))
        assert 1 <= g.scalar("diff_iters") <= 30
