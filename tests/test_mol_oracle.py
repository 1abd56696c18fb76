"""The oracle's MOL predictor-corrector (incflo.use_godunov = false) on the CPU.

The reference holds no known answers for MOL, so these tests pin properties
of the scheme instead: free-stream preservation (periodic and between walls,
which exercises the one-sided wall slopes and the ext_dir faces), agreement
with the Godunov scheme to discretisation error on a smooth flow, second-order
convergence of the step, and the deck checks of src/setup/init.cpp:60-88.
"""
import numpy as np
import pytest

from kynema_sgf_gb300 import decks


def fixed(deck, dt):
    return deck.replace("time.fixed_dt = -1", "time.fixed_dt = %r" % dt)


def run(oracle_mod, deck, steps):
    o = oracle_mod.Oracle(deck)
    o.InitData()
    for _ in range(steps):
        assert o.step()
    return o


def test_free_stream_periodic(oracle_mod):
    d = decks.mol(decks.tgv(16, steps=3, cfl=0.45)).replace(
        "incflo.physics = TaylorGreenVortex", "incflo.physics = FreeStream\nincflo.velocity = 1.5 -0.7 0.3")
    o = run(oracle_mod, d, 2)
    v = o.get_field("velocity")
    assert np.abs(v[0] - 1.5).max() < 1e-13 and np.abs(v[1] + 0.7).max() < 1e-13 and np.abs(v[2] - 0.3).max() < 1e-13
    assert np.abs(o.get_field("conv_term")).max() < 1e-12
    assert np.abs(o.get_field("conv_term_old")).max() < 1e-12


def test_free_stream_between_slip_walls(oracle_mod):
    d = decks.mol(decks.abl(16, 16, 8, steps=3, cfl=0.45))
    d = d.replace("zlo.type = wall_model", "zlo.type = slip_wall").replace("turbulence.model = Smagorinsky", "turbulence.model = Laminar")
    d = d.replace("ICNS.source_terms = GeostrophicForcing CoriolisForcing\n", "")
    d = d.replace("ks_init.loglaw_utop = 8.0", "ks_init.profile = uniform\nincflo.velocity = 6.0 -2.5 0.0")
    d = d.replace("ks_init.noise_amplitude = 0.5", "ks_init.noise_amplitude = 0")
    o = run(oracle_mod, d, 2)
    v = o.get_field("velocity")
    assert np.abs(v[0] - 6.0).max() < 1e-12 and np.abs(v[1] + 2.5).max() < 1e-12 and np.abs(v[2]).max() < 1e-12
    assert np.abs(o.get_field("w_mac")).max() < 1e-12


def test_mol_agrees_with_godunov_on_tgv(oracle_mod):
    base = fixed(decks.tgv(32, steps=10, cfl=0.45), 0.02)
    vg = run(oracle_mod, base, 8).get_field("velocity")
    vm = run(oracle_mod, decks.mol(base), 8).get_field("velocity")
    assert np.linalg.norm(vm - vg) / np.linalg.norm(vg) < 2e-3


def test_second_order_in_space_and_time(oracle_mod):
    """TGV to t = 0.2 at dt proportional to dx: the MOL step (MC slopes,
    Heun time integration) converges at close to second order."""
    vals = {}
    for n in (16, 32, 64):
        d = fixed(decks.mol(decks.tgv(n, steps=1000, cfl=0.45)), 0.1 * 16 / n)
        d = d.replace("time.max_step = 1000", "time.max_step = %d" % (2 * n // 16))
        o = run(oracle_mod, d, 2 * n // 16)
        vals[n] = o.scalar("ke")
    e1 = abs(vals[16] - vals[32])
    e2 = abs(vals[32] - vals[64])
    assert e1 / e2 > 3.0, (vals, e1 / e2)


def test_deck_checks(oracle_mod):
    with pytest.raises(oracle_mod.OracleError) as e:
        oracle_mod.Oracle(decks.mol(decks.tgv(16, cfl=0.5)).replace("time.cfl = 0.5", "time.cfl = 0.6"))
    assert e.value.code == 1 and "0.5" in str(e.value)
    with pytest.raises(oracle_mod.OracleError):
        oracle_mod.Oracle(decks.mol(decks.tgv(16, cfl=0.45)).replace("incflo.diffusion_type = 0", "incflo.diffusion_type = 3"))
    o = oracle_mod.Oracle(decks.tgv(16, cfl=0.45))
    with pytest.raises(oracle_mod.OracleError):
        o.ApplyCorrector()
