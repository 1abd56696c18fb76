"""Mixed-precision form (FP32 advection, diffusion operator and multigrid
cycles; FP64 residuals, defect correction, right-hand sides and velocity
update) against the FP64 form on the same deck.

Stated error (ABL deck, 64 x 64 x 32, 40 steps, against the FP64 run):
- velocity relative L2 error <= 1e-6 (the target of the stated error);
- 99 % of the velocity values within 1e-6 of max|u|, and 99.9 % within
  2e-6: the tail is set by where FP32 rounding flips a discontinuous branch
  (below) and moves with the seed; over noise seeds 42, 1, 2, 3 of this deck
  the 99th percentile is 3.5e-7 to 3.7e-7, the 99.9th 5.2e-7 to 1.14e-6;
- velocity max-norm relative error <= 2e-4: the PPM limiter, trace switch
  and Riemann selections are discontinuous, and FP32 rounding flips them at
  isolated cells;
- pressure-gradient max-norm error <= 5e-3;
- both projections reach the FP64 multigrid tolerance on every step (defect
  correction in FP64) and the MAC divergence stays below 1e-10 relative.
"""
import numpy as np
import pytest

from kynema_sgf_gb300 import decks

pytestmark = pytest.mark.gpu
EPS = np.finfo(float).eps


def assert_fp64_tolerance(sim):
    """Both solves stopped by MLMG's rule at the FP64 tolerance: the final
    max-norm FP64 residual is at most the solve's threshold max(atol,
    rtol max(|rhs|, initial residual)) (mac_proj / nodal_proj rtol 1e-11 on
    these decks; a warm-started solve measures against |rhs|, which can exceed
    the initial residual)."""
    for s in ("mac", "nodal"):
        r, tgt = sim.scalar(s + "_res"), sim.scalar(s + "_target")
        assert 0.0 < tgt and r <= tgt, (s, r, tgt)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_mixed_matches_fp64(cuda_dev):
    deck = decks.abl(64, 64, 32, steps=40)
    ref = cuda_dev.Incflo(deck)
    mix = cuda_dev.Incflo(deck + "\nks.precision = mixed\n")
    assert mix.scalar("precision") == 1.0
    ref.InitData()
    mix.InitData()
    for _ in range(40):
        ref.step()
        mix.step()
        assert_fp64_tolerance(mix)
        assert mix.scalar("mac_iters") <= ref.scalar("mac_iters") + 2
        assert mix.scalar("nodal_iters") <= ref.scalar("nodal_iters") + 2
        # post-projection divergence: the MAC projection is exact (its
        # divergence is the FP64 residual) in both forms
        assert mix.scalar("mac_divu_rel") <= 1e-10 and ref.scalar("mac_divu_rel") <= 1e-10
    v, r = mix.get_field("velocity"), ref.get_field("velocity")
    ev = rel(v, r)
    e2 = np.sqrt(((v - r) ** 2).sum() / (r ** 2).sum())
    p99, p999 = np.quantile(np.abs(v - r) / np.abs(r).max(), [0.99, 0.999])
    eg = rel(mix.get_field("gp"), ref.get_field("gp"))
    print("mixed vs fp64 after 40 steps: vel l2 %.3e p99 %.3e p99.9 %.3e linf %.3e gp linf %.3e" % (e2, p99, p999, ev, eg))
    assert e2 <= 1e-6, e2
    assert p99 <= 1e-6, p99
    assert p999 <= 2e-6, p999
    assert ev < 2e-4, ev
    assert eg < 5e-3, eg


def test_mixed_large_levels(cuda_dev):
    """128 x 128 x 32 cells: the levels above 2^18 points run the FP32
    vector-load sweeps (k_nd_xv, k_cc_gsrb4, k_cc_resid4); both solves reach
    the FP64 tolerance within the FP64 form's V-cycle counts + 2 and the
    velocity stays within the stated error after 6 steps."""
    deck = decks.abl(128, 128, 32, steps=6)
    ref = cuda_dev.Incflo(deck)
    mix = cuda_dev.Incflo(deck + "\nks.precision = mixed\n")
    ref.InitData()
    mix.InitData()
    for _ in range(6):
        ref.step()
        mix.step()
        assert_fp64_tolerance(mix)
        assert mix.scalar("mac_iters") <= ref.scalar("mac_iters") + 2
        assert mix.scalar("nodal_iters") <= ref.scalar("nodal_iters") + 2
        assert mix.scalar("mac_divu_rel") <= 1e-10
    v, r = mix.get_field("velocity"), ref.get_field("velocity")
    e2 = np.sqrt(((v - r) ** 2).sum() / (r ** 2).sum())
    assert e2 <= 1e-6, e2


def test_precision_switch_through_abi(cuda_dev):
    sim = cuda_dev.Incflo(decks.tgv(16, steps=2))
    sim.set_precision(1)
    assert sim.scalar("precision") == 1.0
    sim.InitData()
    assert sim.step()
    sim.set_precision(0)
    assert sim.scalar("precision") == 0.0
    with pytest.raises(cuda_dev.KsError):
        sim.set_precision(7)
