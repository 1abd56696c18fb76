"""GPU parity: the CUDA path (C ABI, cuda:0) against the CPU oracle on the
same decks and seeded inputs.

Tolerance: FP64 on both sides with the same discrete algorithm; differences
come from summation order in reductions, fused multiply-adds and the
solvability shift, amplified by the multigrid stopping test.  Fields are
compared with max-norm relative error <= 1e-9 (pressure after removing its
mean), iteration counts of both Poisson solves must agree within one.
"""
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


def pair(cuda_dev, oracle_mod, deck):
    return cuda_dev.Incflo(deck), oracle_mod.Oracle(deck)


def check_fields(g, o, names, tol=TOL):
    for f in names:
        e = rel(g.get_field(f), o.get_field(f), f)
        assert e < tol, "%s rel err %.3e" % (f, e)


@pytest.mark.parametrize("warm", [0, 1])
@pytest.mark.parametrize("n", [16, 32])
def test_tgv_steps(cuda_dev, oracle_mod, n, warm):
    """warm = 0: both Poisson solves start from zero like the oracle's and the
    V-cycle counts agree within one.  warm = 1 (the default): the solves start
    from the previous potential / the pressure and stop at the same MLMG
    tolerance, so the fields still agree and no solve takes more V-cycles."""
    d = decks.tgv(n, steps=4) + "ks.mg_warm_start = %d\n" % warm
    g, o = pair(cuda_dev, oracle_mod, d)
    check_fields(g, o, ["velocity"], tol=1e-14)
    g.InitData()
    o.InitData()
    check_fields(g, o, ["velocity", "p", "gp"])
    for _ in range(3):
        assert g.step() and o.step()
        assert abs(g.scalar("dt") - o.scalar("dt")) <= 1e-12 * o.scalar("dt")
        for s in ("mac_iters", "nodal_iters"):
            if warm:
                assert g.scalar(s) <= o.scalar(s) + 1
            else:
                assert abs(g.scalar(s) - o.scalar(s)) <= 1
        check_fields(g, o, ["velocity", "p", "gp", "u_mac", "v_mac", "w_mac", "conv_term", "diff_term"])
    assert abs(g.scalar("ke") - o.scalar("ke")) < 1e-12


def test_abl_steps(cuda_dev, oracle_mod):
    g, o = pair(cuda_dev, oracle_mod, decks.abl(32, 32, 16, steps=4))
    check_fields(g, o, ["velocity"], tol=1e-14)
    g.InitData()
    o.InitData()
    assert abs(g.scalar("utau") - o.scalar("utau")) < 1e-13
    check_fields(g, o, ["velocity", "p", "gp"])
    for _ in range(3):
        assert g.step() and o.step()
        check_fields(g, o, ["velocity", "p", "gp", "velocity_mueff", "src_term", "forces", "diff_term", "conv_term",
                            "u_mac", "v_mac", "w_mac"])


def test_disk_steps(cuda_dev, oracle_mod):
    g, o = pair(cuda_dev, oracle_mod, decks.disks(48, 32, 32, steps=4, dcells=8, eps_cells=1.5))
    g.InitData()
    o.InitData()
    for _ in range(3):
        assert g.step() and o.step()
        for k in range(3):
            assert abs(g.scalar("disk_ct:%d" % k) - o.scalar("disk_ct:%d" % k)) < 1e-12
            assert abs(g.scalar("disk_uinf2:%d" % k) - o.scalar("disk_uinf2:%d" % k)) < 1e-9 * o.scalar("disk_uinf2:%d" % k)
        check_fields(g, o, ["velocity", "p", "actuator_src_term", "src_term"])


def test_reference_rotation_convention(cuda_dev, oracle_mod):
    """ks_spread_about_center = 0 reproduces the reference's rotation of the
    absolute force-point position; both sides must agree on it too."""
    d = decks.disks(48, 32, 32, steps=2, dcells=8, eps_cells=1.5, about_center=0, nt=4)
    g, o = pair(cuda_dev, oracle_mod, d)
    g.InitData()
    o.InitData()
    g.step()
    o.step()
    check_fields(g, o, ["actuator_src_term", "velocity"])


def test_operator_surface(cuda_dev, oracle_mod):
    """compute_dt / pre_advance / prepare_time_step / ApplyPredictor /
    ApplyProjection called one by one, as incflo::advance does."""
    d = decks.abl(32, 32, 16, steps=4)
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
    check_fields(g, o, ["velocity", "p", "gp"])
    g.ApplyProjection(g.scalar("new_time"), g.scalar("dt"), False)
    o.ApplyProjection(o.scalar("new_time"), o.scalar("dt"), False)
    check_fields(g, o, ["velocity", "p", "gp"])
    with pytest.raises(cuda_dev.KsError):
        g.ApplyCorrector()
    with pytest.raises(cuda_dev.KsError):
        g.ApplyPredictor(False, 1)


def test_field_roundtrip_host_and_device(cuda_dev):
    import torch
    g = cuda_dev.Incflo(decks.tgv(16, steps=2))
    v = g.get_field("velocity")
    t = torch.empty(v.size, dtype=torch.float64, device="cuda")
    g.get_field("velocity", out=t)
    assert np.array_equal(t.cpu().numpy().reshape(v.shape), v)
    g.set_field("velocity", t * 2)
    assert np.array_equal(g.get_field("velocity"), 2 * v)


def test_invalid_decks_fail_loudly(cuda_dev):
    bad = decks.tgv(16).replace("incflo.godunov_type = ppm", "incflo.godunov_type = weno_z")
    with pytest.raises(cuda_dev.KsError):
        cuda_dev.Incflo(bad)
    with pytest.raises(cuda_dev.KsError):
        cuda_dev.Incflo(decks.tgv(16).replace("time.cfl = 0.5", "time.cfl = 1.5"))


def test_anisotropic_cells(cuda_dev, oracle_mod):
    """dz = dx / 2: both sides reduce the nodal Jacobi weight to 1.35 / 3.0."""
    d = decks.abl(32, 32, 16, steps=3).replace("geometry.prob_hi = 640.0 640.0 320.0", "geometry.prob_hi = 640.0 640.0 160.0")
    g, o = pair(cuda_dev, oracle_mod, d)
    assert abs(g.scalar("nodal_omega") - 0.45) < 1e-12
    g.InitData()
    o.InitData()
    for _ in range(2):
        assert g.step() and o.step()
        check_fields(g, o, ["velocity", "p", "gp"])


def test_maxiter_reports_not_converged(cuda_dev):
    g = cuda_dev.Incflo(decks.tgv(16, steps=2) + "\nnodal_proj.maxiter = 1\nnodal_proj.do_fixed_iters = 0\n")
    with pytest.raises(cuda_dev.KsError) as e:
        g.InitData()
    assert e.value.code == 3


def test_graph_replay_matches_launches(cuda_dev):
    """The coarse V-cycle tails replayed as CUDA graphs run the same kernels
    with the same arguments as launching them one by one: bitwise equal."""
    base = decks.abl(64, 64, 32, steps=4)
    out = {}
    for graphs in (0, 1):
        g = cuda_dev.Incflo(base + "ks.mg_graphs = %d\n" % graphs)
        g.InitData()
        for _ in range(2):
            assert g.step()
        out[graphs] = (g.get_field("velocity"), g.get_field("p"), g.scalar("mac_iters"), g.scalar("nodal_iters"))
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    assert out[0][2:] == out[1][2:]
