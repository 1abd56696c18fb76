"""MAC semicoarsening (mac_proj.do_semicoarsening) in the oracle.

The reference parses do_semicoarsening and max_semicoarsening_level for every
MLMG solve (src/core/MLMGOptions.cpp:24-28).  On cells finer in one direction
the MAC hierarchy halves only that direction until the cells are cubic, then
coarsens all three.  The converged solution is the same as with full
coarsening (the stopping rule does not change); the V-cycle count drops on the
2:1 cells of the ABL benchmark box, where the point smoother leaves errors
smooth in z for the coarse levels.
"""
import numpy as np
import pytest

from kynema_sgf_gb300 import decks


def rel(a, b, name=""):
    if name == "p":
        a = a - a.mean()
        b = b - b.mean()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def levels(o):
    return [tuple(int(o.scalar("mac_level:%d:%d" % (l, d))) for d in range(3)) for l in range(int(o.scalar("mac_levels")))]


def abl_pair(oracle_mod, extra, n=64, dz=10.0):
    base = decks.abl(n, n, n // 2, steps=10, dz=dz) + "ks.mg_warm_start = 0\n"
    a, b = oracle_mod.Oracle(base), oracle_mod.Oracle(base + extra)
    a.InitData()
    b.InitData()
    return a, b


def test_semicoarsening_on_2to1_cells(oracle_mod):
    full, semi = abl_pair(oracle_mod, "mac_proj.do_semicoarsening = true\n")
    for _ in range(2):
        assert full.step() and semi.step()
        # z alone is halved first (20 x 20 x 10 m -> 20 x 20 x 20 m), then all three
        assert levels(semi)[:3] == [(64, 64, 32), (64, 64, 16), (32, 32, 8)]
        assert levels(full)[:2] == [(64, 64, 32), (32, 32, 16)]
        assert full.scalar("mac_iters") >= 30
        assert semi.scalar("mac_iters") <= 10
        for side in (full, semi):
            assert side.scalar("mac_divu_rel") <= 1e-10
        for f, tol in (("velocity", 1e-11), ("p", 1e-10), ("gp", 1e-10), ("u_mac", 1e-10), ("w_mac", 1e-10)):
            assert rel(semi.get_field(f), full.get_field(f), f) < tol, f


@pytest.mark.parametrize("extra,dz", [("mac_proj.do_semicoarsening = true\n", 20.0),
                                      ("mac_proj.do_semicoarsening = true\nmac_proj.max_semicoarsening_level = 0\n", 10.0),
                                      ("mac_proj.max_semicoarsening_level = 3\n", 10.0)])
def test_semicoarsening_is_full_coarsening_when_not_partial(oracle_mod, extra, dz):
    """Cubic cells, a zero semicoarsening depth, or the key off: the hierarchy
    and the result are those of full coarsening (to the rounding of the
    oracle's OpenMP reductions, whose order varies from run to run)."""
    full, other = abl_pair(oracle_mod, extra, n=32, dz=dz)
    for _ in range(2):
        assert full.step() and other.step()
        assert levels(full) == levels(other)
        assert abs(full.scalar("mac_iters") - other.scalar("mac_iters")) <= 1
        for f in ("velocity", "p", "u_mac"):
            assert rel(other.get_field(f), full.get_field(f), f) < 1e-12, f


def test_semicoarsening_depth_limit(oracle_mod):
    """max_semicoarsening_level = 1: level 0 may coarsen partially, every
    later coarsening is full (or none)."""
    d = decks.abl(64, 64, 64, steps=10, dz=5.0) + ("ks.mg_warm_start = 0\nmac_proj.do_semicoarsening = true\n"
                                                  "mac_proj.max_semicoarsening_level = 1\n")
    o = oracle_mod.Oracle(d)
    o.InitData()
    assert o.step()
    # 20 x 20 x 5 m: z halved once (-> 10 m), then full coarsening keeps the 2:1 ratio
    assert levels(o)[:3] == [(64, 64, 64), (64, 64, 32), (32, 32, 16)]
    d2 = d.replace("max_semicoarsening_level = 1", "max_semicoarsening_level = 2")
    o2 = oracle_mod.Oracle(d2)
    o2.InitData()
    assert o2.step()
    assert levels(o2)[:4] == [(64, 64, 64), (64, 64, 32), (64, 64, 16), (32, 32, 8)]
    assert o2.scalar("mac_iters") < o.scalar("mac_iters")


def test_semicoarsening_x_fine_box(oracle_mod):
    """Cells finer in x: x alone is halved first."""
    d = decks.tgv(32, steps=2).replace("amr.n_cell = 32 32 32", "amr.n_cell = 64 32 32") + "mac_proj.do_semicoarsening = true\n"
    assert "amr.n_cell = 64 32 32" in d
    o = oracle_mod.Oracle(d)
    o.InitData()
    assert o.step()
    assert levels(o)[:3] == [(64, 32, 32), (32, 32, 32), (16, 16, 16)]


def test_semicoarsening_mol(oracle_mod):
    """The MOL predictor-corrector projects twice per step; both MAC solves
    take the semicoarsened hierarchy and agree with full coarsening."""
    base = decks.mol(decks.abl(32, 32, 16, steps=10, cfl=0.45, dz=10.0)) + "ks.mg_warm_start = 0\n"
    full, semi = oracle_mod.Oracle(base), oracle_mod.Oracle(base + "mac_proj.do_semicoarsening = true\n")
    full.InitData()
    semi.InitData()
    for _ in range(2):
        assert full.step() and semi.step()
        assert levels(semi)[:2] == [(32, 32, 16), (32, 32, 8)]
        assert semi.scalar("mac_iters") < full.scalar("mac_iters")
        assert semi.scalar("mac_divu_rel") <= 1e-10
        for f in ("velocity", "p", "u_mac"):
            assert rel(semi.get_field(f), full.get_field(f), f) < 1e-10, f
