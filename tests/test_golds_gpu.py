"""The reference's unit-test known answers, checked on the CUDA path (C ABI,
cuda:0) as the oracle's copies in test_oracle_kat.py check the restatement:
BodyForce (unit_tests/wind_energy/test_abl_src.cpp:115-160), the hydrostatic
pressure of a projected column (unit_tests/projection/test_pressure_offset.cpp:
173-203), the wall-model stress in the first layer's diffusion term
(unit_tests/wind_energy/test_abl_bc.cpp:69-170), the strain rate of
quadratic profiles at wall cells (unit_tests/fvm/test_fvm_operators.cpp:258-341)
and the disk orientation from yaw / tilt
(unit_tests/wind_energy/actuator/test_disk_uniform_ct.cpp:35-294).
"""
import numpy as np
import pytest

from kynema_sgf_gb300 import decks
from test_oracle_kat import (DISK_ORIENT_GOLDS, EPS, check_disk_orientation, disk_orient_deck, hydrostatic_column, hydrostatic_deck,
                             quadratic_deck, quadratic_strain_mueff, quadratic_velocity, wall_model_deck, wall_model_gold)

pytestmark = pytest.mark.gpu
TOL = 1e-9


def rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("btype", ["uniform_constant", "oscillatory"])
def test_body_force_steps(cuda_dev, oracle_mod, btype):
    """A Taylor-Green vortex driven by a BodyForce: the source term and the
    state agree with the oracle after every step (the oscillatory factor
    cos(omega t) at the mid-step time of each step)."""
    d = decks.tgv(16, steps=4) + ("ICNS.source_terms = BodyForce\nBodyForce.type = %s\nBodyForce.magnitude = 0.1 0.2 0.3\n"
                                  "BodyForce.angular_frequency = 2.0\n" % btype)
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    g.InitData()
    o.InitData()
    for _ in range(3):
        assert g.step() and o.step()
        for f in ("src_term", "velocity", "gp"):
            e = rel(g.get_field(f), o.get_field(f))
            assert e < TOL, (f, e)
    if btype == "oscillatory":  # the source's mean is the force at the last mid-step time
        t = 0.5 * (g.scalar("time") + g.scalar("new_time"))
        src = g.get_field("src_term")
        assert abs(src[2].mean() - 0.3 * np.cos(2.0 * t)) < 1e-12


def test_body_force_type_names(cuda_dev):
    d = decks.tgv(16, steps=4) + "ICNS.source_terms = BodyForce\nBodyForce.magnitude = 0.1 0.2 0.3\n"
    with pytest.raises(cuda_dev.KsError) as e:
        cuda_dev.Incflo(d + "BodyForce.type = constant\n")
    assert e.value.code == 1
    with pytest.raises(cuda_dev.KsError) as e:
        cuda_dev.Incflo(d + "BodyForce.type = height_varying\n")
    assert e.value.code == 2


def test_pressure_offset_hydrostatic_column(cuda_dev):
    g = cuda_dev.Incflo(hydrostatic_deck() + "incflo.do_initial_proj = 0\nincflo.initial_iterations = 0\n")
    g.InitData()
    hydrostatic_column(g)


@pytest.mark.parametrize("stress", ["local", "moeng"])
def test_abl_wall_model_gold(cuda_dev, oracle_mod, stress):
    """One step from u = 5 over the wall model: diff_term (divtau of the Old
    state) is -tau_wall / dz in the first layer and zero elsewhere, u_tau as
    the log law gives it; the whole step agrees with the oracle."""
    d = wall_model_deck(stress)
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    g.InitData()
    o.InitData()
    assert g.step() and o.step()
    utau, tau = wall_model_gold()
    assert abs(g.scalar("utau") - utau) < 1.0e4 * EPS
    D = g.get_field("diff_term")
    assert np.allclose(D[0, 0], -tau, rtol=0, atol=1.0e4 * EPS)
    assert np.abs(D[0, 1:]).max() < 1.0e4 * EPS and np.abs(D[1:]).max() < 1.0e4 * EPS
    for f in ("velocity", "diff_term", "p"):
        a, b = g.get_field(f), o.get_field(f)
        if f == "p":
            a, b = a - a.mean(), b - b.mean()
        assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1.0), f


def test_strain_rate_exact_for_quadratics(cuda_dev):
    n, L = (4, 4, 16), 4.0
    g = cuda_dev.Incflo(quadratic_deck(n, L) + "time.fixed_dt = 0.01\nincflo.do_initial_proj = 0\nincflo.initial_iterations = 0\n")
    g.InitData()
    shape = g.layout("velocity")
    g.set_field("velocity", quadratic_velocity(shape, L))
    assert g.step()  # velocity_mueff is formed from the Old state, the field set above
    dx = (1.0 / n[0], 1.0 / n[1], L / n[2])
    mu = g.get_field("velocity_mueff")[0]
    assert np.allclose(mu, quadratic_strain_mueff(shape, L, 0.16, dx), rtol=1.0e6 * EPS, atol=0)


@pytest.mark.parametrize("case", range(len(DISK_ORIENT_GOLDS)))
def test_disk_orientation_golds(cuda_dev, case):
    keys, cor, normal, sample = DISK_ORIENT_GOLDS[case]
    check_disk_orientation(cuda_dev.Incflo(disk_orient_deck(keys, cor)), normal, sample)


def test_disk_orientation_errors(cuda_dev):
    for keys in ("yaw = 270;tilt = -90", "disk_normal = 1 0 0;yaw = 10", "sample_normal = 1 0 0;sample_tilt = 10"):
        with pytest.raises(cuda_dev.KsError) as e:
            cuda_dev.Incflo(disk_orient_deck(keys))
        assert e.value.code == 1, keys


def test_yawed_disk_steps(cuda_dev, oracle_mod):
    """A disk yawed 80 degrees and tilted 5, sampling upstream along its own
    vector (sample_yaw 60, sample_tilt -10, 1.5 diameters): the sampled U_inf,
    Ct, actuator source and state agree with the oracle after every step."""
    d = disk_orient_deck("yaw = 80;tilt = 5;sample_yaw = 60;sample_tilt = -10;diameters_to_sample = 1.5;ks_spread_about_center = 1",
                         "ks_init.noise_amplitude = 0.2\nks_init.noise_seed = 3")
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    g.InitData()
    o.InitData()
    for _ in range(2):
        assert g.step() and o.step()
        ug, uo = g.scalar("disk_uinf2:0"), o.scalar("disk_uinf2:0")
        assert abs(ug - uo) < 1e-9 * uo
        for f in ("actuator_src_term", "velocity", "p"):
            a, b = g.get_field(f), o.get_field(f)
            if f == "p":
                a, b = a - a.mean(), b - b.mean()
            assert rel(a, b) < TOL, f
