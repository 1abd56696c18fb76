"""GPU: temperature transport of the ABL physics (Boussinesq buoyancy,
ABLForcing, heat-flux wall model, fixed-gradient top) against the oracle, and
the known answers of test_temperature_oracle.py through the C ABI."""
import math

import numpy as np
import pytest

from kynema_sgf_gb300 import decks

from test_temperature_oracle import box_deck, factor

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


@pytest.mark.parametrize("case", ["godunov0", "godunov1", "mol0", "mol2"])
def test_stratified_abl_parity(cuda_dev, oracle_mod, case):
    """The reference's abl_godunov configuration (explicit, and Crank-Nicolson
    as in its default deck) and its MOL form (explicit; implicit as in the
    reference's abl_mol deck) at 32^3 for three steps."""
    dtype = int(case[-1])
    d = decks.abl_temperature((32, 32, 32), diffusion_type=dtype, fixed_dt=0.5 if dtype else -0.5)
    if case.startswith("mol"):
        d = decks.mol(d.replace("time.cfl = 0.95", "time.cfl = 0.45"))
    d += "diffusion.mg_rtol = 1e-13\n"
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    check(g, o, ["velocity", "temperature"], tol=1e-14)
    g.InitData()
    o.InitData()
    check(g, o, ["velocity", "p", "gp", "temperature"])
    for _ in range(3):
        assert g.step() and o.step()
        assert abs(g.scalar("dt") - o.scalar("dt")) <= 1e-12 * o.scalar("dt")
        assert abs(g.scalar("theta_mean") - o.scalar("theta_mean")) <= 1e-12 * o.scalar("theta_mean")
        for c in ("abl_forcing_x", "abl_forcing_y"):  # (target - mean) / dt: rounding of the mean over dt
            assert abs(g.scalar(c) - o.scalar(c)) <= 1e-9 * abs(o.scalar(c)) + 1e-12 * 10.0 / o.scalar("dt")
        check(g, o, ["velocity", "p", "gp", "temperature", "temperature_mueff", "src_term", "velocity_mueff"])


@pytest.mark.parametrize("scheme", ["godunov", "mol"])
@pytest.mark.parametrize("dtype", [0, 1, 2])
def test_scalar_diffusion_amplification(cuda_dev, dtype, scheme):
    n, nu, pr, dt = 16, 400.0, 0.7, 0.5
    d = box_deck(n=n, dtype=dtype, sources="", periodic_z=True, nu=nu, pr=pr, dt=dt,
                 extra="diffusion.mg_rtol = 1e-14\ntemperature_diffusion.mg_rtol = 1e-14\n")
    if scheme == "mol":
        d = decks.mol(d.replace("time.cfl = 0.9", "time.cfl = 0.45"))
    g = cuda_dev.Incflo(d)
    h = 1000.0 / n
    z = (np.arange(n) + 0.5) * h
    th0 = np.broadcast_to((300.0 + 2.0 * np.cos(2 * math.pi * z / 1000.0))[None, :, None, None], (1, n, n, n)).copy()
    g.set_field("temperature", th0)
    g.InitData()
    lam = -(nu / pr) * (2 - 2 * math.cos(2 * math.pi / n)) / (h * h)
    for _ in range(3):
        assert g.step()
    expect = 300.0 + factor(dtype, dt * lam) ** 3 * (th0 - 300.0)
    assert np.abs(g.get_field("temperature") - expect).max() < 1e-11 * 300.0


def test_hydrostatic_balance(cuda_dev):
    g = cuda_dev.Incflo(box_deck(dtype=1))
    g.InitData()
    for _ in range(2):
        assert g.step()
    assert np.abs(g.get_field("velocity")).max() < 1e-11
    assert np.abs(g.get_field("gp")[2] - (-9.81) * (1.0 / 300.0) * (300.0 - 305.0)).max() < 1e-10


def test_temperature_rejections(cuda_dev):
    base = decks.abl_temperature((16, 16, 16))
    with pytest.raises(cuda_dev.KsError):
        cuda_dev.Incflo(base + "ABL.surface_temp_flux = 0.05\n")
