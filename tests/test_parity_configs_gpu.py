"""GPU parity on the benchmark configurations themselves (not toy grids).

The CUDA path (C ABI, cuda:0) and the CPU oracle advance the same decks:
- the Taylor-Green vortex exactly as benchmarked: 64^3, Re 1600, CFL 0.5,
  nodal rtol 1e-11, initial projection and 3 pressure iterations, 20 steps;
- the neutral ABL on 128 x 128 x 64 cubic 20 m cells (wall model, slip top,
  Smagorinsky, geostrophic + Coriolis, CFL 0.9), 4 steps (the benchmark box's
  20 x 20 x 10 m cells: test_zzz_named_box_gpu.py);
- the adjoint-check disk deck (128 x 128 x 64, 3 uniform-Ct disks, D = 16
  cells, fixed dt), 3 steps.

After every step both sides must agree on dt (1e-12 relative), on the
V-cycle counts of both projections (within one, both solves started from
zero; with the warm start the GPU may only take fewer), and on all state
fields to max-norm relative 1e-9.  The post-projection divergence is checked
on both sides: the MAC projection is exact, so the divergence of the MAC
velocities is at most 1e-10 relative (|div u_mac| max-norm times min(dx) over
max|u_mac|); the nodal projection is an approximate projection, so the nodal
divergence of the cell velocity is truncation-sized and must agree between
the two sides to 1e-8 relative.
"""
import numpy as np
import pytest

from kynema_sgf_gb300 import decks

pytestmark = pytest.mark.gpu
TOL = 1e-9
DIV_TOL = 1e-10


def rel(a, b, name=""):
    if name == "p":
        a = a - a.mean()
        b = b - b.mean()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def check_fields(g, o, names, tol=TOL):
    for f in names:
        e = rel(g.get_field(f), o.get_field(f), f)
        assert e < tol, "%s rel err %.3e" % (f, e)


def check_step(g, o, warm):
    assert abs(g.scalar("dt") - o.scalar("dt")) <= 1e-12 * o.scalar("dt")
    for s in ("mac_iters", "nodal_iters"):
        if warm:
            assert g.scalar(s) <= o.scalar(s) + 1, s
        else:
            assert abs(g.scalar(s) - o.scalar(s)) <= 1, s
    for side in (g, o):
        assert side.scalar("mac_divu_rel") <= DIV_TOL, side.scalar("mac_divu_rel")
    dg, do = g.scalar("divu"), o.scalar("divu")
    assert abs(dg - do) <= 1e-8 * do, (dg, do)


@pytest.mark.parametrize("warm", [0, 1])
def test_c0_tgv64_20_steps(cuda_dev, oracle_mod, warm):
    d = decks.tgv(64, steps=20) + "ks.mg_warm_start = %d\n" % warm
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    check_fields(g, o, ["velocity"], tol=1e-14)
    g.InitData()
    o.InitData()
    check_fields(g, o, ["velocity", "p", "gp"])
    for _ in range(20):
        assert g.step() and o.step()
        check_step(g, o, warm)
        check_fields(g, o, ["velocity", "p", "gp"])
    check_fields(g, o, ["u_mac", "v_mac", "w_mac", "conv_term", "diff_term"])
    assert not g.step() and not o.step()  # time.max_step = 20 ends the run on both sides
    assert abs(g.scalar("ke") - o.scalar("ke")) < 1e-12 * o.scalar("ke")


def test_abl_128x128x64(cuda_dev, oracle_mod):
    d = decks.abl(128, 128, 64, steps=10) + "ks.mg_warm_start = 0\n"
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    check_fields(g, o, ["velocity"], tol=1e-14)
    g.InitData()
    o.InitData()
    check_fields(g, o, ["velocity", "p", "gp"])
    for _ in range(4):
        assert g.step() and o.step()
        check_step(g, o, 0)
        assert abs(g.scalar("utau") - o.scalar("utau")) < 1e-12 * o.scalar("utau")
        check_fields(g, o, ["velocity", "p", "gp", "velocity_mueff", "src_term", "forces", "diff_term", "conv_term",
                            "u_mac", "v_mac", "w_mac"])


def test_c3_disk_deck_128x128x64(cuda_dev, oracle_mod):
    d, lo, hi, cts = decks.adjoint_c3()
    d += "ks.mg_warm_start = 0\n"
    g, o = cuda_dev.Incflo(d), oracle_mod.Oracle(d)
    g.InitData()
    o.InitData()
    for _ in range(3):
        assert g.step() and o.step()
        check_step(g, o, 0)
        for k in range(len(cts)):
            assert abs(g.scalar("disk_ct:%d" % k) - o.scalar("disk_ct:%d" % k)) < 1e-12
            ug, uo = g.scalar("disk_uinf2:%d" % k), o.scalar("disk_uinf2:%d" % k)
            assert abs(ug - uo) < 1e-9 * uo
        check_fields(g, o, ["velocity", "p", "gp", "actuator_src_term", "src_term", "conv_term"])
