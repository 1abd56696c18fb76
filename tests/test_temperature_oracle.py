"""Temperature transport of the ABL physics in the oracle: initial fields
(ABLFieldInit), hydrostatic balance of the Boussinesq buoyancy, the scalar
diffusion's amplification factors, conservation between zero-flux walls, and
the deck checks."""
import math

import numpy as np
import pytest

from kynema_sgf_gb300 import decks


def box_deck(n=16, dtype=0, theta_vals=(305.0, 305.0), velocity="0 0 0", sources="BoussinesqBuoyancy", periodic_z=False, nu=1.0e-5,
             pr=0.7, dt=0.5, extra=""):
    zper = 1 if periodic_z else 0
    walls = "" if periodic_z else "zlo.type = slip_wall\nzhi.type = slip_wall\n"
    src = f"ICNS.source_terms = {sources}\n" if sources else ""
    return f"""
time.max_step = 10
time.fixed_dt = {dt}
time.cfl = 0.9
incflo.gravity = 0. 0. -9.81
incflo.density = 1.0
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = {dtype}
transport.viscosity = {nu!r}
transport.laminar_prandtl = {pr!r}
transport.reference_temperature = 300.0
turbulence.model = Laminar
incflo.physics = ABL
{src}incflo.velocity = {velocity}
ABL.perturb_velocity = 0
ABL.temperature_heights = 0.0 1000.0
ABL.temperature_values = {theta_vals[0]!r} {theta_vals[1]!r}
amr.n_cell = {n} {n} {n}
geometry.prob_lo = 0. 0. 0.
geometry.prob_hi = 1000. 1000. 1000.
geometry.is_periodic = 1 1 {zper}
{walls}{extra}"""


def test_initial_fields(oracle_mod):
    """ABLFieldInit.cpp:279-372: uniform wind plus the damped sinusoidal
    perturbation, piecewise-linear temperature (tv[0] outside the segments)."""
    n = 16
    o = oracle_mod.Oracle(decks.abl_temperature((n, n, n)))
    v, th = o.get_field("velocity"), o.get_field("temperature")
    h = 1000.0 / n
    c = (np.arange(n) + 0.5) * h
    z = c[:, None, None]
    damp = np.exp(-0.5 * (z / 50.0) ** 2)
    fac = math.exp(0.5) / 50.0
    u = 6.128355544951824 + fac * damp * z * np.cos(4 * 2 * math.pi / 1000.0 * c[None, :, None])
    w = 5.142300877492314 + fac * damp * z * np.cos(4 * 2 * math.pi / 1000.0 * c[None, None, :])
    assert np.abs(v[0] - u).max() < 1e-12 and np.abs(v[1] - w).max() < 1e-12 and np.abs(v[2]).max() == 0.0
    prof = np.where(c <= 650.0, 300.0, np.where(c <= 750.0, 300.0 + (c - 650.0) * 0.08, 308.0 + (c - 750.0) * 0.003))
    assert np.abs(th[0, :, 0, 0] - prof).max() < 1e-12


@pytest.mark.parametrize("dtype", [0, 1])
def test_hydrostatic_balance(oracle_mod, dtype):
    """Uniform theta != T0 at rest between slip walls: the buoyancy is a
    uniform vertical acceleration that the projection turns into the pressure
    gradient, gp_z = rho g beta (T0 - theta), and the fluid stays at rest."""
    o = oracle_mod.Oracle(box_deck(dtype=dtype))
    o.InitData()
    for _ in range(2):
        assert o.step()
    assert np.abs(o.get_field("velocity")).max() < 1e-11
    gp = o.get_field("gp")
    assert np.abs(gp[2] - (-9.81) * (1.0 / 300.0) * (300.0 - 305.0)).max() < 1e-10
    assert np.abs(gp[0]).max() < 1e-12 and np.abs(gp[1]).max() < 1e-12


def factor(dtype, x):
    if dtype == 0:
        return 1 + x + 0.5 * x * x
    if dtype == 1:
        return (1 + 0.5 * x) / (1 - 0.5 * x)
    return 1 / (1 - x)


@pytest.mark.parametrize("scheme", ["godunov", "mol"])
@pytest.mark.parametrize("dtype", [0, 1, 2])
def test_scalar_diffusion_amplification(oracle_mod, dtype, scheme):
    """theta = 300 + A cos(2 pi z / L) at rest in a periodic box: the discrete
    diffusion operator maps the wave to lambda times itself, lambda = -alpha
    (2 - 2 cos(2 pi / nz)) / dz^2, and each step multiplies it by the scheme's
    factor (explicit RK2 or MOL's Heun step, Crank-Nicolson, implicit)."""
    n, nu, pr, dt = 16, 400.0, 0.7, 0.5
    d = box_deck(n=n, dtype=dtype, sources="", periodic_z=True, nu=nu, pr=pr, dt=dt,
                 extra="diffusion.mg_rtol = 1e-14\ntemperature_diffusion.mg_rtol = 1e-14\n")
    if scheme == "mol":
        d = decks.mol(d.replace("time.cfl = 0.9", "time.cfl = 0.45"))
    o = oracle_mod.Oracle(d)
    h = 1000.0 / n
    z = (np.arange(n) + 0.5) * h
    th0 = np.broadcast_to((300.0 + 2.0 * np.cos(2 * math.pi * z / 1000.0))[None, :, None, None], (1, n, n, n)).copy()
    o.set_field("temperature", th0)
    o.InitData()
    lam = -(nu / pr) * (2 - 2 * math.cos(2 * math.pi / n)) / (h * h)
    for _ in range(3):
        assert o.step()
    th = o.get_field("temperature")
    expect = 300.0 + factor(dtype, dt * lam) ** 3 * (th0 - 300.0)
    assert np.abs(th - expect).max() < 1e-11 * 300.0
    assert np.abs(o.get_field("velocity")).max() < 1e-12


def test_temperature_conserved_between_zero_flux_walls(oracle_mod):
    d = decks.abl_temperature((16, 16, 16)).replace('zlo.type = "wall_model"', "zlo.type = slip_wall")
    d = d.replace('zhi.temperature_type = "fixed_gradient"\n', "")
    o = oracle_mod.Oracle(d)
    o.InitData()
    s0 = o.get_field("temperature").sum()
    for _ in range(3):
        assert o.step()
    assert abs(o.get_field("temperature").sum() - s0) < 1e-13 * abs(s0)


def test_mol_stratified_abl_close_to_godunov(oracle_mod):
    """The reference's abl_mol configuration (MOL with temperature, implicit
    diffusion) against the Godunov form of the same flow over a few steps."""
    base = decks.abl_temperature((16, 16, 16), diffusion_type=2, fixed_dt=0.5, cfl=0.45)
    out = {}
    for name, d in (("godunov", base), ("mol", decks.mol(base))):
        o = oracle_mod.Oracle(d)
        o.InitData()
        for _ in range(3):
            assert o.step()
        out[name] = (o.get_field("velocity"), o.get_field("temperature"))
    dv = np.abs(out["mol"][0] - out["godunov"][0]).max() / np.abs(out["godunov"][0]).max()
    dt = np.abs(out["mol"][1] - out["godunov"][1]).max()
    assert dv < 2e-2 and dt < 0.5


def test_deck_checks(oracle_mod):
    base = decks.abl_temperature((16, 16, 16))
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.Oracle(base + "ABL.surface_temp_flux = 0.05\n")
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.Oracle(base.replace("ABL.temperature_heights = 650.0 750.0 1000.0\n", ""))  # buoyancy without temperature
