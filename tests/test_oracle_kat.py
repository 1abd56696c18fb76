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


def body_force_deck(btype="oscillatory", extra=""):
    return box_deck(n=(8, 8, 8), extra="ICNS.source_terms = BodyForce\nincflo.density = 1.0\nBodyForce.type = %s\n"
                                        "BodyForce.magnitude = 1.0 2.0 3.0\nBodyForce.angular_frequency = 1.0\n%s" % (btype, extra))


def test_body_force_gold(oracle_mod):
    """unit_tests/wind_energy/test_abl_src.cpp:115-160 (parameters of
    abl_test_utils.cpp:40-47): oscillatory BodyForce, magnitude (1, 2, 3),
    angular frequency 1: (1, 2, 3) at t = 0, then (1, 2, 3) cos(0.5 (0.05 +
    t_new)) with the current time 0.05 (BodyForce.cpp:117-169 evaluates at
    the mid-step time)."""
    tol = 1.0e4 * EPS
    o = oracle_mod.Oracle(body_force_deck())
    o.compute_sources()
    src = o.get_field("src_term")
    for n, gold in enumerate((1.0, 2.0, 3.0)):
        assert np.allclose(src[n], gold, rtol=0, atol=tol)
    o.set_scalar("time", 0.05)
    o.set_scalar("new_time", 0.15)
    o.compute_sources()
    src = o.get_field("src_term")
    for n, mag in enumerate((1.0, 2.0, 3.0)):
        assert np.allclose(src[n], mag * math.cos(0.5 * (0.05 + 0.15)), rtol=0, atol=tol)


def test_body_force_types(oracle_mod):
    """uniform_constant (the default) ignores the time; the reference aborts
    on any other name (BodyForce.cpp:47-56) and the file-driven types are
    outside this path."""
    o = oracle_mod.Oracle(body_force_deck("uniform_constant"))
    o.set_scalar("time", 3.0)
    o.set_scalar("new_time", 4.0)
    o.compute_sources()
    src = o.get_field("src_term")
    for n, gold in enumerate((1.0, 2.0, 3.0)):
        assert np.allclose(src[n], gold, rtol=0, atol=1.0e4 * EPS)
    with pytest.raises(oracle_mod.OracleError) as e:
        oracle_mod.Oracle(body_force_deck("constant"))
    assert e.value.code == 1
    with pytest.raises(oracle_mod.OracleError) as e:
        oracle_mod.Oracle(body_force_deck("height_varying"))
    assert e.value.code == 2


def hydrostatic_deck(n=(4, 4, 16)):
    return box_deck(n=n, hi=(1.0, 1.0, 1.0), periodic=(1, 1, 0),
                    extra="zlo.type = slip_wall\nzhi.type = slip_wall\nincflo.density = 1.0\ntransport.viscosity = 0.0\n"
                          "nodal_proj.mg_rtol = 1e-13\nnodal_proj.mg_atol = 1e-14")


def hydrostatic_column(sim, w0=-9.81):
    """unit_tests/projection/test_pressure_offset.cpp:173-203 restated for a
    column closed at both ends: a uniform vertical velocity w0 (the velocity
    gravity F_g = w0 would produce in one unit step) projected with dt = 1 at
    time 1.  The projected velocity vanishes and the pressure carries the
    hydrostatic difference p(bottom) - p(top) = -F_g over the unit column (the
    reference's pressure_outflow top pins p(top) = 0 and checks p(bottom) =
    -F_g to 1e8 eps); gp_z = F_g."""
    v = np.zeros(sim.layout("velocity"))
    v[2] = w0
    for f in ("velocity", "velocity_old"):
        sim.set_field(f, v if f == "velocity" else np.zeros_like(v))
    sim.set_field("gp", np.zeros(sim.layout("gp")))
    sim.ApplyProjection(1.0, 1.0, False)
    p = sim.get_field("p")[0]
    tol = 1.0e8 * EPS
    assert np.abs(sim.get_field("velocity")).max() < tol
    assert abs((p[0].mean() - p[-1].mean()) - (-w0)) < tol
    assert np.abs(p[0] - p[0].mean()).max() < tol  # every bottom node alike
    gp = sim.get_field("gp")
    assert np.allclose(gp[2], w0, rtol=0, atol=tol) and np.abs(gp[:2]).max() < tol


def test_pressure_offset_hydrostatic_column(oracle_mod):
    hydrostatic_column(oracle_mod.Oracle(hydrostatic_deck()))


def rk2_deck():
    return box_deck(n=(8, 8, 16), hi=(1.0, 1.0, 1.0), extra="incflo.density = 2.0\ntransport.viscosity = 0.1\ntime.fixed_dt = 0.5")


def rk2_scalar(shape):
    # init_scalar of unit_tests/equation_systems/test_explicit_diffusion_rk2.cpp:15-31
    nc, nz, ny, nx = shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    f = 1.0 + i * i + 0.2 * (j - 1) * (j - 1) + 0.01 * (k + 1) ** 3
    return np.broadcast_to(f, shape).copy()


@pytest.mark.parametrize("approach", ["old", "correct"])
def test_explicit_diffusion_rk2(oracle_mod, approach):
    """unit_tests/equation_systems/test_explicit_diffusion_rk2.cpp:116-184
    (rho 2, mu 0.1, dt 0.5, 8 x 8 x 16): predictor_rhs with only the explicit
    diffusion term gives u_old + dt D / rho.  old: subtracting dt D does not
    return u_old (error above 10 FP32 eps).  correct: with the diffusion term
    replaced by -2 D, improve_explicit_diffusion (explicit_rk2_post_hoc,
    u += dt/2 diff / rho) returns u_old to 1e4 eps."""
    o = oracle_mod.Oracle(rk2_deck())
    o.set_scalar("dt", 0.5)
    f = rk2_scalar(o.layout("velocity_old"))
    o.set_field("velocity_old", f)
    o.compute_divtau()
    D = o.get_field("diff_term")
    assert np.abs(D).max() > 1.0e4 * EPS
    o.set_field("conv_term", np.zeros_like(D))
    o.set_field("src_term", np.zeros_like(D))
    o.predictor_rhs(1.0)
    u = o.get_field("velocity")
    assert np.allclose(u, f + 0.5 * D / 2.0, rtol=0, atol=1.0e4 * EPS * np.abs(f).max())
    if approach == "old":
        assert np.abs(u - 0.5 * D - f).max() > 10 * np.finfo(np.float32).eps
    else:
        o.set_field("diff_term", -2.0 * D)
        o.improve_explicit_diffusion()
        assert np.abs(o.get_field("velocity") - f).max() < 1.0e4 * EPS


def wall_model_deck(stress="local", fixed_dt=0.1, extra=""):
    # unit_tests/wind_energy/test_abl_bc.cpp:69-170 on the default test mesh (8^3 cells on [0, 8]^3)
    return box_deck(n=(8, 8, 8), hi=(8.0, 8.0, 8.0), periodic=(1, 1, 0),
                    extra=f"zlo.type = wall_model\nzhi.type = slip_wall\nincflo.physics = FreeStream\nincflo.velocity = 5.0 0.0 0.0\n"
                          f"incflo.density = 1.0\ntransport.viscosity = 0.01\nturbulence.model = Laminar\ntime.fixed_dt = {fixed_dt}\n"
                          f"ABL.wall_shear_stress_type = {stress}\nABL.kappa = 0.4\nABL.surface_roughness_z0 = 0.11\n"
                          f"incflo.do_initial_proj = 0\nincflo.initial_iterations = 0\n{extra}")


def wall_model_gold(vval=5.0, dz=1.0, kappa=0.4, z0=0.11):
    utau = kappa * vval / math.log(0.5 * dz / z0)
    return utau, utau ** 2


@pytest.mark.parametrize("stress", ["local", "moeng"])
def test_abl_wall_model_gold(oracle_mod, stress):
    """unit_tests/wind_energy/test_abl_bc.cpp:69-170: uniform u = 5 over a
    wall-model bottom (kappa 0.4, z0 0.11, mu 0.01, dt 0.1): the explicit
    diffusion term of the first layer is -tau_wall / dz with tau_wall =
    u_tau^2, u_tau = kappa U / ln(z_ref / z0), so predictor_rhs with only
    diffusion gives u = 5 - dt tau_wall / dz there (and leaves every other
    cell at 5).  For a uniform field the Moeng stress equals the local one."""
    o = oracle_mod.Oracle(wall_model_deck(stress))
    o.InitData()
    o.set_scalar("dt", 0.1)
    o.pre_advance()
    utau, tau = wall_model_gold()
    assert abs(o.scalar("utau") - utau) < 1.0e4 * EPS
    o.prepare_time_step()
    o.update_mueff()
    o.compute_divtau()
    D = o.get_field("diff_term")
    assert np.allclose(D[0, 0], -tau, rtol=0, atol=1.0e4 * EPS)
    assert np.abs(D[0, 1:]).max() < 1.0e4 * EPS and np.abs(D[1:]).max() < 1.0e4 * EPS
    o.set_field("conv_term", np.zeros_like(D))
    o.set_field("src_term", np.zeros_like(D))
    o.predictor_rhs(1.0)
    u = o.get_field("velocity")
    assert np.allclose(u[0, 0], 5.0 - 0.1 * tau, rtol=0, atol=1.0e4 * EPS)
    assert np.allclose(u[0, 1:], 5.0, rtol=0, atol=1.0e4 * EPS)


def quadratic_velocity(shape, L):
    """Velocity quadratic in z with w = 0 on both walls (z = 0, L)."""
    nc, nz, ny, nx = shape
    z = (np.arange(nz) + 0.5) * (L / nz)
    v = np.zeros(shape)
    v[0] = (0.3 * z * z + 0.7 * z + 1.0)[:, None, None]
    v[1] = (-0.2 * z * z + 0.1 * z)[:, None, None]
    v[2] = (0.05 * z * (L - z))[:, None, None]
    return v


def quadratic_strain_mueff(shape, L, Cs, dx):
    nc, nz, ny, nx = shape
    z = (np.arange(nz) + 0.5) * (L / nz)
    dudz, dvdz, dwdz = 0.6 * z + 0.7, -0.4 * z + 0.1, 0.05 * (L - 2 * z)
    s = np.sqrt(2.0 * dwdz ** 2 + dudz ** 2 + dvdz ** 2)
    return (Cs ** 2 * np.cbrt(dx[0] * dx[1] * dx[2]) ** 2 * s)[:, None, None] * np.ones((nz, ny, nx))


def quadratic_deck(n=(4, 4, 16), L=4.0):
    return box_deck(n=n, hi=(1.0, 1.0, L), periodic=(1, 1, 0),
                    extra="zlo.type = slip_wall\nzhi.type = slip_wall\nturbulence.model = Smagorinsky\nSmagorinsky_coeffs.Cs = 0.16\n"
                          "transport.viscosity = 0.0\nincflo.density = 1.0")


def test_strain_rate_exact_for_quadratics(oracle_mod):
    """unit_tests/fvm/test_fvm_ops.cpp:427-454 (strain rate) and
    test_fvm_operators.cpp:258-341 (gradient) check the FVM operators on
    degree-2 polynomials with wall ghosts holding the wall values; on this
    path the strain rate (fvm::StrainRate, central interior stencils and the
    one-sided wall stencils of stencils.H:166-330) sees the fill-patch ghosts
    (hoextrap (15 q0 - 10 q1 + 3 q2) / 8, which is the wall value of a
    quadratic, and w = 0), so |S| of a quadratic profile is exact in every
    cell, wall cells included."""
    n, L = (4, 4, 16), 4.0
    o = oracle_mod.Oracle(quadratic_deck(n, L))
    shape = o.layout("velocity_old")
    o.set_field("velocity_old", quadratic_velocity(shape, L))
    o.update_mueff()
    dx = (1.0 / n[0], 1.0 / n[1], L / n[2])
    mu = o.get_field("velocity_mueff")[0]
    assert np.allclose(mu, quadratic_strain_mueff(shape, L, 0.16, dx), rtol=1.0e6 * EPS, atol=0)


def disk_orient_deck(extra="", coriolis=""):
    """One uniform-Ct disk in a 16^3 box; `extra` adds keys of the disk."""
    lines = "\n".join("Actuator.T0.%s" % e for e in extra.split(";") if e.strip())
    return f"""
geometry.prob_lo = 0 0 0
geometry.prob_hi = 160 160 160
geometry.is_periodic = 1 1 1
amr.n_cell = 16 16 16
incflo.physics = FreeStream
incflo.velocity = 8.0 0.0 0.0
transport.viscosity = 1e-5
turbulence.model = Laminar
ICNS.source_terms = ActuatorForcing
Actuator.labels = T0
Actuator.type = UniformCtDisk
Actuator.UniformCtDisk.rotor_diameter = 40
Actuator.UniformCtDisk.epsilon = 10
Actuator.UniformCtDisk.thrust_coeff = 0.75
Actuator.UniformCtDisk.num_points_r = 3
Actuator.UniformCtDisk.num_points_t = 4
Actuator.UniformCtDisk.spreading_type = UniformGaussian
Actuator.T0.disk_center = 80 80 80
{lines}
{coriolis}
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = 0
time.cfl = 0.5
time.max_step = 2
"""


def disk_points_deck(center, nr=2, nt=2, diameter=2.0, normal="1 0 0"):
    """One uniform-Ct disk with its sampling disk on the rotor (diameters_to_sample 0),
    in a box holding every centre of the known answers below."""
    return f"""
geometry.prob_lo = -2000 -2000 -2000
geometry.prob_hi = 2000 2000 2000
geometry.is_periodic = 1 1 1
amr.n_cell = 8 8 8
incflo.physics = FreeStream
incflo.velocity = 8.0 0.0 0.0
transport.viscosity = 1e-5
turbulence.model = Laminar
ICNS.source_terms = ActuatorForcing
Actuator.labels = T0
Actuator.type = UniformCtDisk
Actuator.UniformCtDisk.rotor_diameter = {diameter}
Actuator.UniformCtDisk.epsilon = 1
Actuator.UniformCtDisk.thrust_coeff = 0.75
Actuator.UniformCtDisk.num_points_r = {nr}
Actuator.UniformCtDisk.num_points_t = {nt}
Actuator.UniformCtDisk.spreading_type = UniformGaussian
Actuator.UniformCtDisk.diameters_to_sample = 0
Actuator.T0.disk_center = {center[0]} {center[1]} {center[2]}
Actuator.T0.disk_normal = {normal}
incflo.use_godunov = 1
incflo.godunov_type = ppm
time.fixed_dt = 0.1
time.max_step = 1
"""


# unit_tests/wind_energy/actuator/test_disk_functions.cpp:80-116: a disk of
# diameter 2 facing x, 2 x 2 points; the points sit at -+ 0.5 dr and -+ 1.5 dr
# along y (dr = 0.5) from each of these centres, radius-major
DISK_POINT_CENTERS = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1), (-1, 0, 0), (-1, -1, -1), (1000.0, 30.0, 5.0)]


@pytest.mark.parametrize("center", DISK_POINT_CENTERS)
def test_disk_points_known_answers(oracle_mod, center):
    o = oracle_mod.Oracle(disk_points_deck(center))
    dr = 2.0 * 0.5 / 2
    gold = [(0.0, 0.5 * dr, 0.0), (0.0, -0.5 * dr, 0.0), (0.0, 1.5 * dr, 0.0), (0.0, -1.5 * dr, 0.0)]
    eps = 3.0 * EPS
    for p, gp in enumerate(gold):
        for m in range(3):
            x = o.scalar("disk_point:0:%d:%d" % (p, m))
            assert abs(x - (gp[m] + center[m])) <= eps * max(1.0, abs(center[m])), (p, m, x)


# test_disk_functions.cpp:47-78, 118-125 (AreaComputer): the ring sections of a
# polar grid of nr x nt points add up to pi R^2 and their weights to 1
@pytest.mark.parametrize("radius,nr,nt", [(1.0, 3, 1), (1.0, 3, 2), (127.0, 10, 3), (30.0, 5, 30)])
def test_disk_area_weights_known_answers(oracle_mod, radius, nr, nt):
    o = oracle_mod.Oracle(disk_points_deck((0, 0, 0), nr=nr, nt=nt, diameter=2.0 * radius))
    area = math.pi * radius * radius
    w = [o.scalar("disk_weight:0:%d" % p) for p in range(nr * nt)]
    assert abs(sum(w) - 1.0) <= 10.0 * EPS
    assert abs(sum(x * area for x in w) - area) <= 1.0e4 * EPS * area
    # AreaComputer::area_section(i) = R^2 pi / (nr^2 nt) ((i + 1)^2 - i^2)
    for i in range(nr):
        for j in range(nt):
            sec = radius * radius / nr / nr * math.pi / nt * ((i + 1.0) ** 2 - float(i) ** 2)
            assert abs(w[i * nt + j] * area - sec) <= 1.0e2 * EPS * area


DIFFERENT_NORTH = "Coriolis.Forcing.north_vector = 1 0 0\nCoriolis.Forcing.east_vector = 0 -1 0"
_R2 = math.sqrt(0.5)
# (disk keys, Coriolis keys, gold normal, gold sample vector): the cases of
# unit_tests/wind_energy/actuator/test_disk_uniform_ct.cpp:35-166, 218-294
DISK_ORIENT_GOLDS = [
    ("yaw = 90;sample_yaw = 45", "", (1, 0, 0), (_R2, _R2, 0)),
    ("yaw = 270;sample_yaw = -315;sample_tilt = -45", "", (-1, 0, 0), (0.5, 0.5, _R2)),
    ("", DIFFERENT_NORTH, (1, 0, 0), (1, 0, 0)),
    ("yaw = 90;sample_yaw = 45;sample_tilt = -45", DIFFERENT_NORTH, (0, -1, 0), (0.5, -0.5, _R2)),
    ("yaw = 0", "", (0, 1, 0), (0, 1, 0)),
    ("yaw = 180", "", (0, -1, 0), (0, -1, 0)),
    ("yaw = 270", "", (-1, 0, 0), (-1, 0, 0)),
    ("yaw = 90", "", (1, 0, 0), (1, 0, 0)),
    ("sample_yaw = 0", "", (0, 1, 0), (0, 1, 0)),
    ("sample_yaw = 180", "", (0, 1, 0), (0, -1, 0)),
    ("sample_yaw = 270", "", (0, 1, 0), (-1, 0, 0)),
    ("sample_yaw = 90", "", (0, 1, 0), (1, 0, 0)),
]


def check_disk_orientation(sim, normal, sample):
    for m in range(3):
        assert abs(sim.scalar("disk_normal:0:%d" % m) - normal[m]) < 1e4 * EPS
        assert abs(sim.scalar("disk_sample:0:%d" % m) - sample[m]) < 1e4 * EPS


@pytest.mark.parametrize("case", range(len(DISK_ORIENT_GOLDS)))
def test_disk_orientation_golds(oracle_mod, case):
    """Disk normal and sampling vector from yaw / tilt / sample_yaw /
    sample_tilt and the Coriolis north / east vectors
    (ops::base::optional_parameters, disk_ops.cpp:182-264): the reference's
    golds, including a yaw of 0 / 180 / 270 / 90 degrees pointing the normal
    against a wind from north / south / west / east."""
    keys, cor, normal, sample = DISK_ORIENT_GOLDS[case]
    check_disk_orientation(oracle_mod.Oracle(disk_orient_deck(keys, cor)), normal, sample)


@pytest.mark.parametrize("keys", ["yaw = 270;tilt = -90", "disk_normal = 1 0 0;yaw = 10", "sample_normal = 1 0 0;sample_tilt = 10",
                                  "base_position = 80 80 0"])
def test_disk_orientation_errors(oracle_mod, keys):
    """A tilt of -90 degrees points the normal up, which the coplanar vector
    rejects (test_disk_uniform_ct.cpp:93-97); disk_normal with yaw / tilt,
    sample_normal with sample_yaw / sample_tilt and base_position without
    hub_height are parse conflicts (disk_ops.cpp:278-300)."""
    d = disk_orient_deck(keys)
    if "base_position" in keys:
        d = d.replace("Actuator.T0.disk_center = 80 80 80\n", "")
    with pytest.raises(oracle_mod.OracleError) as e:
        oracle_mod.Oracle(d)
    assert e.value.code == 1
