"""Known-answer checks of the CPU oracle against the reference's unit tests.

Each test restates a unit test of Kynema-SGF (paths inside that repository)
with its inputs and expected values, driven through the oracle's C entry
points.  These pin the oracle before it is used as the parity checker.
"""
import math

import numpy as np
import pytest

from kynema_sgf_gb300 import decks

EPS = np.finfo(float).eps


def box_deck(n=(10, 20, 30), hi=(10.0, 10.0, 10.0), periodic=(1, 1, 1), extra=""):
    return f"""
geometry.prob_lo = 0 0 0
geometry.prob_hi = {hi[0]} {hi[1]} {hi[2]}
geometry.is_periodic = {periodic[0]} {periodic[1]} {periodic[2]}
amr.n_cell = {n[0]} {n[1]} {n[2]}
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = 0
{extra}
"""


def linear_field(shape, dx, srate):
    # init_field3 of unit_tests/turbulence/test_turbulence_LES.cpp:23-45:
    # u_n = x_n / sqrt(6) * srate at cell centres
    nc, nz, ny, nx = shape
    v = np.zeros(shape)
    x = (np.arange(nx) + 0.5) * dx[0]
    y = (np.arange(ny) + 0.5) * dx[1]
    z = (np.arange(nz) + 0.5) * dx[2]
    v[0] = x[None, None, :] / math.sqrt(6.0) * srate
    v[1] = y[None, :, None] / math.sqrt(6.0) * srate
    v[2] = z[:, None, None] / math.sqrt(6.0) * srate
    return v


def test_smagorinsky_constant_strain(oracle_mod):
    """unit_tests/turbulence/test_turbulence_LES.cpp:155-233: Cs = 0.16,
    mu = 1e-5, rho = 1.2, strain rate 0.5 -> mu_t = rho Cs^2 Delta^2 |S|."""
    Cs, visc, srate, rho0 = 0.16, 1.0e-5, 0.5, 1.2
    d = box_deck(extra=f"turbulence.model = Smagorinsky\nSmagorinsky_coeffs.Cs = {Cs}\ntransport.viscosity = {visc}\n"
                       f"incflo.density = {rho0}")
    o = oracle_mod.Oracle(d)
    dx = (1.0, 0.5, 1.0 / 3.0)
    o.set_field("velocity_old", linear_field(o.layout("velocity_old"), dx, srate))
    o.update_mueff()
    mu = o.get_field("velocity_mueff")[0]
    answer = rho0 * Cs ** 2 * np.cbrt(dx[0] * dx[1] * dx[2]) ** 2 * srate
    inner = mu[1:-1, 1:-1, 1:-1]  # periodic wrap breaks the linear field on the boundary layer
    assert np.allclose(inner, answer + visc, rtol=0, atol=1.0e4 * EPS)


def test_strain_rate_one_sided_at_wall(oracle_mod):
    """src/fvm/stencils.H:166-330 one-sided z stencils: exact for a linear
    field whose wall-normal component vanishes on the wall (z = 0)."""
    d = box_deck(periodic=(1, 1, 0), extra="zlo.type = slip_wall\nzhi.type = slip_wall\nturbulence.model = Smagorinsky\n"
                                           "Smagorinsky_coeffs.Cs = 0.16\ntransport.viscosity = 0.0")
    o = oracle_mod.Oracle(d)
    dx = (1.0, 0.5, 1.0 / 3.0)
    o.set_field("velocity_old", linear_field(o.layout("velocity_old"), dx, 0.5))
    o.update_mueff()
    mu = o.get_field("velocity_mueff")[0]
    answer = 0.16 ** 2 * np.cbrt(dx[0] * dx[1] * dx[2]) ** 2 * 0.5
    assert np.allclose(mu[:-1, 1:-1, 1:-1], answer, rtol=0, atol=1.0e4 * EPS)


def coriolis_deck(lat, extra=""):
    return box_deck(n=(8, 8, 8), extra=f"ICNS.source_terms = {extra}\nCoriolisForcing.latitude = {lat}\nincflo.density = 1.0")


def test_geostrophic_forcing_gold(oracle_mod):
    """unit_tests/wind_energy/test_abl_src.cpp:165-198: latitude 54,
    geostrophic wind (10, 6, 0)."""
    o = oracle_mod.Oracle(coriolis_deck(54.0, "GeostrophicForcing\nGeostrophicForcing.geostrophic_wind = 10.0 6.0 0.0"))
    o.compute_sources()
    src = o.get_field("src_term")
    corfac = 2.0 * 2.0 * math.pi / 86164.091 * 0.80901699437
    gold = [-corfac * 6.0, corfac * 10.0, 0.0]
    for n in range(3):
        assert np.allclose(src[n], gold[n], rtol=0, atol=1.0e4 * EPS)


@pytest.mark.parametrize("comp", [0, 1])
def test_coriolis_const_vel(oracle_mod, comp):
    """unit_tests/wind_energy/test_abl_src.cpp:359-420: latitude 45,
    constant velocity along x or y."""
    o = oracle_mod.Oracle(coriolis_deck(45.0, "CoriolisForcing"))
    vel_comp = 10.0 + 5.0 * (0.3141 - 0.5)
    v = np.zeros(o.layout("velocity_old"))
    v[comp] = vel_comp
    o.set_field("velocity_old", v)
    o.compute_sources()
    src = o.get_field("src_term")
    corfac = 2.0 * 2.0 * math.pi / 86164.091
    latfac = math.sin(math.radians(45.0))
    gold = [0.0, -corfac * latfac * vel_comp, corfac * latfac * vel_comp] if comp == 0 else [corfac * latfac * vel_comp, 0.0, 0.0]
    for n in range(3):
        assert np.allclose(src[n], gold[n], rtol=0, atol=1.0e4 * EPS)


def test_simtime_init_shrink_and_growth(oracle_mod):
    """unit_tests/core/test_simtime.cpp:32-60: cfl 0.45 and a convective
    CFL of 0.45 give dt = 1; the initialisation shrink gives 0.1 and the next
    step may grow by at most 10%."""
    d = box_deck(n=(8, 8, 8), hi=(8.0, 8.0, 8.0), extra="incflo.physics = FreeStream\nincflo.velocity = 0.45 0.0 0.0\n"
                                                          "time.cfl = 0.45\nincflo.initial_iterations = 0\nincflo.do_initial_proj = 0")
    o = oracle_mod.Oracle(d)
    dt0 = o.compute_dt()
    assert abs(dt0 - 0.1) < 1e4 * EPS
    assert o.step()
    assert abs(o.scalar("dt") - 1.1 * dt0) < 1e4 * EPS


def test_wall_model_utau_neutral(oracle_mod):
    """src/wind_energy/MOData.cpp:52-103, neutral: u_tau = kappa U /
    ln(z_ref / z0) with z_ref the first cell centre."""
    d = decks.abl(16, 16, 8, steps=1).replace("ks_init.noise_amplitude = 0.5", "ks_init.noise_amplitude = 0.0")
    o = oracle_mod.Oracle(d)
    v = o.get_field("velocity")
    o.InitData()
    umag = np.sqrt(v[0, 0] ** 2 + v[1, 0] ** 2).mean()
    zref = 0.5 * 20.0
    assert abs(o.scalar("utau") - 0.41 * umag / math.log(zref / 0.1)) < 1e-12


def test_divtau_discrete_eigenfunction(oracle_mod):
    """Tensor operator on u = sin(z): div tau_x = mu * (-(2 - 2cos dz)/dz^2) sin(z)."""
    n = 16
    d = box_deck(n=(8, 8, n), hi=(1.0, 1.0, 2 * math.pi), extra="transport.viscosity = 0.3\nturbulence.model = Laminar")
    o = oracle_mod.Oracle(d)
    dz = 2 * math.pi / n
    z = (np.arange(n) + 0.5) * dz
    v = np.zeros(o.layout("velocity_old"))
    v[0] = np.sin(z)[:, None, None]
    o.set_field("velocity_old", v)
    o.update_mueff()
    o.compute_divtau(False)
    dt = o.get_field("diff_term")
    expect = 0.3 * (-(2 - 2 * math.cos(dz)) / dz ** 2) * np.sin(z)[:, None, None]
    assert np.allclose(dt[0], expect, atol=1e-12)
    assert np.abs(dt[1:]).max() < 1e-12


def test_tgv_initial_field_and_decay(oracle_mod):
    """TaylorGreenVortex.cpp:22-54 initial field (KE = 1/8); the early KE
    decay rate approaches the viscous rate -6 nu KE of the single-mode
    Taylor-Green vortex as the grid is refined (numerical dissipation of the
    limited PPM shrinks)."""
    rates = []
    for n in (32, 64):
        o = oracle_mod.Oracle(decks.tgv(n, steps=5))
        assert abs(o.scalar("ke") - 0.125) < 1e-12
        o.InitData()
        assert abs(o.scalar("ke") - 0.125) < 1e-6
        ke0, t0 = o.scalar("ke"), o.scalar("time")
        for _ in range(3):
            o.step()
        rates.append((o.scalar("ke") - ke0) / (o.scalar("time") - t0))
    viscous = -6 * 0.000625 * 0.125
    assert all(r < 0.9 * viscous for r in rates)
    assert abs(rates[1] - viscous) < abs(rates[0] - viscous)
    assert rates[1] > 2.0 * viscous


def test_projection_converges(oracle_mod):
    """Both projections reach the MLMG target max(atol, rtol * r0)."""
    o = oracle_mod.Oracle(decks.tgv(32, steps=2, rtol=1e-11))
    o.InitData()
    o.step()
    assert o.scalar("nodal_res") <= max(1e2 * EPS, 1e-11 * o.scalar("nodal_res0"))
    assert o.scalar("mac_res") <= max(1e2 * EPS, 1e5 * EPS * o.scalar("mac_res0"))
    assert 0 < o.scalar("mac_iters") < 20 and 0 < o.scalar("nodal_iters") < 20


def test_disk_total_thrust(oracle_mod):
    """uniform_ct_ops.H:71-97 + disk_spreading.H:45-105: the spread force of
    a disk integrates to 1/2 U_inf^2 Ct pi R^2 along the disk normal."""
    d = decks.disks(48, 32, 32, steps=2, dcells=8, cts=(0.75,), eps_cells=1.5)
    o = oracle_mod.Oracle(d)
    o.InitData()
    o.step()
    act = o.get_field("actuator_src_term")
    total = -act[0].sum() * 10.0 ** 3  # component along the disk normal (-1, 0, 0)
    R = 40.0
    expect = 0.5 * o.scalar("disk_uinf2:0") * 0.75 * math.pi * R * R
    assert abs(total - expect) / expect < 1e-6
    assert np.abs(act[1:]).max() < 1e-12


def test_disk_spreading_rotation_conventions_agree_for_one_point(oracle_mod):
    """With num_points_t = 1 the reference's rotation of the absolute point
    position (disk_spreading.H:85-86) and rotation about the disk centre agree."""
    fields = []
    for about in (0, 1):
        d = decks.disks(48, 32, 32, steps=2, dcells=8, cts=(0.75,), eps_cells=1.5, about_center=about, nt=1)
        o = oracle_mod.Oracle(d)
        o.InitData()
        o.step()
        fields.append(o.get_field("actuator_src_term"))
    assert np.array_equal(fields[0], fields[1])


def test_noise_initial_field(oracle_mod):
    """Seeded uniform noise: bounded by the amplitude, zero above z_max."""
    o = oracle_mod.Oracle(decks.abl(16, 16, 32, steps=1))
    v = o.get_field("velocity")
    z = (np.arange(32) + 0.5) * 20.0
    w = v[2]
    assert np.abs(w).max() <= 0.5
    assert np.all(w[z > 300] == 0.0)
    assert abs(w[z < 300].mean()) < 0.05


def _aspect2_abl():
    # dz = dx / 2: the 27-point nodal stencil's D^-1 A reaches 3.0, beyond 2 / 0.9
    return decks.abl(32, 32, 16, steps=3).replace("geometry.prob_hi = 640.0 640.0 320.0", "geometry.prob_hi = 640.0 640.0 160.0")


def test_projections_converge_on_anisotropic_cells(oracle_mod):
    """The nodal Jacobi weight drops to 1.35 / lambda_max (0.45 at dz = dx / 2,
    where 0.9 diverges); both projections reach the MLMG target."""
    o = oracle_mod.Oracle(_aspect2_abl())
    o.InitData()
    for _ in range(2):
        o.step()
        assert o.scalar("nodal_res") <= max(1e2 * EPS, 1e5 * EPS * o.scalar("nodal_res0"))
        assert o.scalar("mac_res") <= max(1e2 * EPS, 1e5 * EPS * o.scalar("mac_res0"))
        assert o.scalar("nodal_iters") < 60


def test_maxiter_reports_not_converged(oracle_mod):
    """MLMGOptions runs MLMG in fixed-iteration mode by default (no abort at
    maxiter, MLMGOptions.H:126-128); with do_fixed_iters = 0 a solve that ends
    above the tolerance is KS_ERR_NOT_CONVERGED (3)."""
    o = oracle_mod.Oracle(decks.tgv(16, steps=2) + "\nnodal_proj.maxiter = 1\n")
    o.InitData()
    assert o.scalar("nodal_iters") == 1
    o = oracle_mod.Oracle(decks.tgv(16, steps=2) + "\nnodal_proj.maxiter = 1\nnodal_proj.do_fixed_iters = 0\n")
    with pytest.raises(oracle_mod.OracleError) as e:
        o.InitData()
    assert e.value.code == 3
