"""GPU parity of the MOL predictor-corrector (incflo.use_godunov = false)
against the CPU oracle: whole steps, the operator surface one call at a time
(ApplyPredictor, then ApplyCorrector), wall-bounded ABL with Smagorinsky and
the wall model, and actuator disks.  Tolerance as in test_parity_gpu.py."""
import numpy as np
import pytest

from kynema_sgf_gb300 import decks

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


def pair(cuda_dev, oracle_mod, deck):
    return cuda_dev.Incflo(deck), oracle_mod.Oracle(deck)


@pytest.mark.parametrize("n", [16, 32])
def test_tgv_mol_steps(cuda_dev, oracle_mod, n):
    g, o = pair(cuda_dev, oracle_mod, decks.mol(decks.tgv(n, steps=4, cfl=0.45)) + "ks.mg_warm_start = 0\n")
    g.InitData()
    o.InitData()
    check(g, o, ["velocity", "p", "gp"])
    for _ in range(3):
        assert g.step() and o.step()
        assert abs(g.scalar("dt") - o.scalar("dt")) <= 1e-12 * o.scalar("dt")
        assert abs(g.scalar("nodal_iters") - o.scalar("nodal_iters")) <= 1
        check(g, o, ["velocity", "p", "gp", "u_mac", "v_mac", "w_mac", "conv_term", "conv_term_old", "diff_term"])
    assert abs(g.scalar("ke") - o.scalar("ke")) < 1e-12


def test_abl_mol_steps(cuda_dev, oracle_mod):
    g, o = pair(cuda_dev, oracle_mod, decks.mol(decks.abl(32, 32, 16, steps=4, cfl=0.45)))
    g.InitData()
    o.InitData()
    check(g, o, ["velocity", "p", "gp"])
    for _ in range(3):
        assert g.step() and o.step()
        check(g, o, ["velocity", "p", "gp", "velocity_mueff", "src_term", "diff_term", "conv_term", "conv_term_old",
                     "u_mac", "v_mac", "w_mac"])


def test_mol_operator_surface(cuda_dev, oracle_mod):
    """incflo::advance for MOL called one operator at a time: the predicted
    state after ApplyPredictor and the corrected one after ApplyCorrector."""
    d = decks.mol(decks.abl(32, 32, 16, steps=4, cfl=0.45))
    g, o = pair(cuda_dev, oracle_mod, d)
    g.InitData()
    o.InitData()
    assert abs(g.compute_dt() - o.compute_dt()) < 1e-12 * o.compute_dt()
    g.pre_advance()
    o.pre_advance()
    g.prepare_time_step()
    o.prepare_time_step()
    g.ApplyPredictor(False, 0)
    o.ApplyPredictor(False, 0)
    check(g, o, ["velocity", "p", "gp", "conv_term_old", "diff_term", "u_mac", "w_mac"])
    g.ApplyCorrector()
    o.ApplyCorrector()
    check(g, o, ["velocity", "p", "gp", "conv_term", "velocity_mueff", "src_term", "u_mac", "w_mac"])


def test_mol_disks(cuda_dev, oracle_mod):
    g, o = pair(cuda_dev, oracle_mod, decks.mol(decks.disks(48, 32, 32, steps=4, dcells=8, eps_cells=1.5, cfl=0.45)))
    g.InitData()
    o.InitData()
    for _ in range(3):
        assert g.step() and o.step()
        check(g, o, ["velocity", "p", "actuator_src_term", "src_term"])


def test_mol_rejections(cuda_dev):
    with pytest.raises(cuda_dev.KsError) as e:
        cuda_dev.Incflo(decks.mol(decks.tgv(16, cfl=0.45)).replace("time.cfl = 0.45", "time.cfl = 0.6"))
    assert "0.5" in str(e.value)
    g = cuda_dev.Incflo(decks.mol(decks.tgv(16, steps=2, cfl=0.45)).replace("time.fixed_dt = -1", "time.fixed_dt = 0.01"))
    g.InitData()
    with pytest.raises(cuda_dev.KsError):
        g.adjoint_step()
