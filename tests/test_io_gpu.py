"""GPU: plot files of a running handle, checkpoint / restart (bitwise
continuation at fixed dt, replication onto a larger domain) and the
interval-driven outputs, through the C ABI."""
import os

import numpy as np
import pytest

from amrex_reader import read_plotfile, read_vismf
from kynema_sgf_gb300 import decks

pytestmark = pytest.mark.gpu


def abl_deck(steps=6, extra=""):
    d = decks.abl(32, 32, 16, steps=steps).replace("time.cfl = 0.9", "time.cfl = 0.9\ntime.fixed_dt = 0.5")
    return d + extra


def test_plotfile_of_a_handle(cuda_dev, tmp_path):
    g = cuda_dev.Incflo(abl_deck())
    g.InitData()
    for _ in range(2):
        g.step()
    g.write_plot_file(tmp_path / "plt00002")
    h, ch, d = read_plotfile(tmp_path / "plt00002")
    assert h["names"] == ["density", "gpx", "gpy", "gpz", "mu_turb", "p", "velocityx", "velocityy", "velocityz", "velocity_mueff"]
    assert h["level_steps"] == [2] and abs(h["time"] - g.scalar("time") - g.scalar("dt")) < 1e-12
    v, gp, mu = g.get_field("velocity"), g.get_field("gp"), g.get_field("velocity_mueff")
    assert np.array_equal(d[6:9], v) and np.array_equal(d[1:4], gp) and np.array_equal(d[9], mu[0])
    assert np.all(d[0] == 1.225)
    assert np.allclose(d[4], mu[0] - 1.8e-5, rtol=0, atol=1e-18)
    assert np.array_equal(d[5], g.get_field("p")[0, :16, :32, :32])  # the node at each cell's low corner


def test_checkpoint_restart_continues_bitwise(cuda_dev, tmp_path):
    a = cuda_dev.Incflo(abl_deck())
    a.InitData()
    for _ in range(2):
        a.step()
    chk = tmp_path / "chk00002"
    a.write_checkpoint_file(chk)
    hv, vel = read_vismf(chk / "Level_0" / "velocity")
    assert hv["ngrow"] == 3 and hv["fab_box"][0] == [-3, -3, -3]
    assert np.array_equal(vel[:, 3:-3, 3:-3, 3:-3], a.get_field("velocity"))
    hp, _ = read_vismf(chk / "Level_0" / "p")
    assert hp["box"] == ([0, 0, 0], [32, 32, 16], [1, 1, 1])
    b = cuda_dev.Incflo(abl_deck(extra="io.restart_file = %s\n" % chk))
    b.InitData()
    assert b.scalar("step") == 2
    for f in ("velocity", "gp", "p"):
        assert np.array_equal(a.get_field(f), b.get_field(f))
    for _ in range(2):
        assert a.step() and b.step()
    for f in ("velocity", "gp", "p"):
        assert np.array_equal(a.get_field(f), b.get_field(f)), f


def test_restart_replicates_onto_a_larger_domain(cuda_dev, tmp_path):
    a = cuda_dev.Incflo(abl_deck())
    a.InitData()
    a.step()
    a.write_checkpoint_file(tmp_path / "chk")
    big = abl_deck(extra="io.restart_file = %s\n" % (tmp_path / "chk"))
    big = big.replace("amr.n_cell = 32 32 16", "amr.n_cell = 64 32 16").replace("geometry.prob_hi = 640.0 640.0 320.0",
                                                                                  "geometry.prob_hi = 1280.0 640.0 320.0")
    b = cuda_dev.Incflo(big)
    b.InitData()
    va, vb = a.get_field("velocity"), b.get_field("velocity")
    assert np.array_equal(vb[:, :, :, :32], va) and np.array_equal(vb[:, :, :, 32:], va)


def test_interval_outputs(cuda_dev, tmp_path):
    cwd = os.getcwd()
    os.chdir(tmp_path)
    try:
        g = cuda_dev.Incflo(abl_deck(steps=5, extra="time.plot_interval = 2\ntime.checkpoint_interval = 4\n"))
        g.InitData()
        g.write_outputs()
        while g.step():
            g.write_outputs()
        g.write_outputs(last=True)
    finally:
        os.chdir(cwd)
    names = sorted(p.name for p in tmp_path.iterdir())
    # SimTime::write_plot_file / write_checkpoint at steps 0 (InitData), 2, 4 and the
    # end-of-run rules at step 5 (5 % 2 != 0, 5 % 4 != 0)
    assert names == ["chk00000", "chk00004", "chk00005", "plt00000", "plt00002", "plt00004", "plt00005"]
