"""Reverse mode of the advance (ks_adjoint_* through the C ABI) on the GPU.

Gradients of J = mean 0.5 |u|^2 over the wake box of the last disk with
respect to the disk thrust coefficients are checked against central finite
differences of the FP64 forward run; the bar is 1e-4 relative to the largest
gradient component.

The discrete forward map is piecewise smooth with jumps: the PPM trace
switches from the parabola to the cell value where a transverse velocity
crosses +-small_vel, and the Riemann solver switches states across sonic
points.  With +-0.2 m/s noise around zero transverse velocity (the literal
128 x 128 x 64 check) such a jump lies within 1e-7 of the base point for
every disk: J jumps by about 1e-11 relative, which a central difference with
h = 1e-6 turns into a 1e-3 error.  That check therefore uses h = 1e-8 (J is
resolved to about 1e-15, so roundoff stays below 1e-6 of the gradient); the
same box with a uniform cross-flow (v, w) = (1, 0.5) m/s, where no
transverse velocity crosses zero, is checked with h = 1e-6.
"""
import numpy as np
import pytest

from kynema_sgf_gb300 import decks

pytestmark = pytest.mark.gpu
TOL = 1e-4
SMALL = dict(nx=32, ny=32, nz=16, dcells=4, nr=3, nt=8)


def make(ks, **kw):
    deck, lo, hi, cts = decks.adjoint_c3(**kw)
    sim = ks.Incflo(deck)
    sim.InitData()
    sim.set_objective_box(lo, hi)
    x0 = {f: sim.get_field(f) for f in ("velocity", "gp", "p")}
    return sim, x0, np.array(cts), (deck, lo, hi)


def restore(sim, x0):
    for f, v in x0.items():
        sim.set_field(f, v)


def forward_J(sim, x0, ct, nsteps):
    restore(sim, x0)
    sim.set_disk_ct(ct)
    for _ in range(nsteps):
        assert sim.step()
    return sim.objective()


def adjoint(sim, x0, ct, nsteps, snapshots):
    restore(sim, x0)
    sim.set_disk_ct(ct)
    J = sim.adjoint_run(nsteps, snapshots)
    return J, sim.ct_gradient()


def fd_rel(sim, x0, ct, nsteps, g, h):
    fd = np.array([(forward_J(sim, x0, ct + h * e, nsteps) - forward_J(sim, x0, ct - h * e, nsteps)) / (2 * h)
                   for e in np.eye(len(ct))])
    return np.abs(fd - g).max() / np.abs(g).max()


def test_ct_gradient_small(cuda_dev):
    sim, x0, ct, _ = make(cuda_dev, **SMALL)
    J, g = adjoint(sim, x0, ct, 10, 10)
    assert J == forward_J(sim, x0, ct, 10)
    assert np.all(g < 0)  # more thrust, slower wake
    assert fd_rel(sim, x0, ct, 10, g, 1e-6) < TOL


def test_ct_gradient_c3_crossflow(cuda_dev):
    sim, x0, ct, _ = make(cuda_dev, crossflow=(1.0, 0.5))
    J, g = adjoint(sim, x0, ct, 40, 6)
    assert fd_rel(sim, x0, ct, 40, g, 1e-6) < TOL


def test_ct_gradient_c3(cuda_dev):
    sim, x0, ct, _ = make(cuda_dev)
    assert np.all((ct >= 0.6) & (ct <= 0.9))
    J, g = adjoint(sim, x0, ct, 40, 6)
    assert J == forward_J(sim, x0, ct, 40)
    assert fd_rel(sim, x0, ct, 40, g, 1e-8) < TOL


def test_binomial_matches_store_all(cuda_dev, ks_lib):
    sim, x0, ct, _ = make(cuda_dev, **SMALL)
    J1, g1 = adjoint(sim, x0, ct, 12, 12)
    u1 = sim.get_field("velocity_adjoint")
    p1 = sim.get_field("gp_adjoint")
    assert sim.scalar("adj_forward_steps") == ks_lib.checkpoint_cost(12, 12) == 11
    J2, g2 = adjoint(sim, x0, ct, 12, 3)
    assert sim.scalar("adj_forward_steps") == ks_lib.checkpoint_cost(12, 3)
    assert sim.scalar("adj_reverse_steps") == 12
    assert J1 == J2
    assert np.abs(g1 - g2).max() <= 1e-12 * np.abs(g1).max()
    u2 = sim.get_field("velocity_adjoint")
    assert np.abs(u1 - u2).max() <= 1e-12 * np.abs(u1).max()
    assert np.abs(p1 - sim.get_field("gp_adjoint")).max() <= 1e-12 * np.abs(p1).max()


def test_adjoint_run_final_state(cuda_dev):
    """After adjoint_run(n) the forward state and clock are those of n Evolve steps."""
    sim, x0, ct, _ = make(cuda_dev, **SMALL)
    ref, _, _, _ = make(cuda_dev, **SMALL)
    adjoint(sim, x0, ct, 6, 2)
    for _ in range(6):
        ref.step()
    for name in ("time", "new_time", "step", "dt"):
        assert sim.scalar(name) == ref.scalar(name), name
    for f in ("velocity", "gp", "p"):
        assert np.array_equal(sim.get_field(f), ref.get_field(f)), f


def test_one_step_vjp(cuda_dev):
    """<x_bar^n, dx> = d/dh <w, step(x^n + h dx)> for random w, dx (velocity and gp)."""
    sim, x0, ct, _ = make(cuda_dev, **SMALL)
    for _ in range(5):
        sim.step()
    xs = {f: sim.get_field(f) for f in ("velocity", "gp", "p")}
    rng = np.random.default_rng(5)
    sh = xs["velocity"].shape
    w, w2, du, dg = rng.standard_normal(sh), rng.standard_normal(sh), rng.uniform(-1, 1, sh), rng.uniform(-1, 1, sh)

    def F(h):
        restore(sim, xs)
        sim.set_field("velocity", xs["velocity"] + h * du)
        sim.set_field("gp", xs["gp"] + h * dg)
        sim.step()
        return float((w * sim.get_field("velocity")).sum() + (w2 * sim.get_field("gp")).sum())

    restore(sim, xs)
    sim.adjoint_reset()
    sim.set_field("velocity_adjoint", w)
    sim.set_field("gp_adjoint", w2)
    sim.adjoint_step()
    assert np.array_equal(sim.get_field("velocity"), xs["velocity"])  # forward state left at x^n
    adj = float((sim.get_field("velocity_adjoint") * du).sum() + (sim.get_field("gp_adjoint") * dg).sum())
    h = 1e-7
    assert abs((F(h) - F(-h)) / (2 * h) - adj) <= 1e-6 * abs(adj)


def test_torch_autograd_chain(cuda_dev):
    import torch
    from kynema_sgf_gb300.autograd import AdjointRun, AdvanceStep, box_cells, box_mean_ke

    sim, x0, ct0, (deck, lo, hi) = make(cuda_dev, **SMALL)
    n = (SMALL["nx"], SMALL["ny"], SMALL["nz"])
    cells = box_cells(lo, hi, (0.0, 0.0, 0.0), (10.0, 10.0, 10.0), n)
    dev = torch.device("cuda:0")
    u = torch.tensor(x0["velocity"], device=dev)
    gp = torch.tensor(x0["gp"], device=dev)
    ct = torch.tensor(ct0, dtype=torch.float64, requires_grad=True)
    for _ in range(5):
        u, gp = AdvanceStep.apply(sim, u, gp, ct)
    J = box_mean_ke(u, cells)
    J.backward()
    g_chain = ct.grad.clone()
    J_ref, g_ref = adjoint(sim, x0, ct0, 5, 5)
    assert abs(J.item() - J_ref) <= 1e-14 * abs(J_ref)
    assert torch.allclose(g_chain, torch.tensor(g_ref, dtype=torch.float64), rtol=1e-10, atol=0)
    # the checkpointed node gives the same gradient
    restore(sim, x0)
    ct2 = torch.tensor(ct0, dtype=torch.float64, requires_grad=True)
    J2 = AdjointRun.apply(sim, ct2, 5, 2)
    J2.backward()
    assert J2.item() == J_ref
    assert torch.allclose(ct2.grad, g_chain, rtol=1e-10, atol=0)


def test_forward_J_matches_oracle(cuda_dev, oracle_mod):
    deck, lo, hi, cts = decks.adjoint_c3(**SMALL)
    g = cuda_dev.Incflo(deck)
    o = oracle_mod.Oracle(deck)
    g.InitData()
    o.InitData()
    g.set_objective_box(lo, hi)
    for _ in range(10):
        assert g.step() and o.step()
    from kynema_sgf_gb300.autograd import box_cells
    k, j, i = box_cells(lo, hi, (0.0, 0.0, 0.0), (10.0, 10.0, 10.0), (SMALL["nx"], SMALL["ny"], SMALL["nz"]))
    v = o.get_field("velocity")[:, k, j, i]
    J_oracle = 0.5 * (v * v).sum() / (v.shape[1] * v.shape[2] * v.shape[3])
    assert abs(g.objective() - J_oracle) <= 1e-10 * J_oracle


def test_adjoint_unsupported_decks(cuda_dev):
    sim = cuda_dev.Incflo(decks.abl(32, 32, 16, steps=2))
    with pytest.raises(cuda_dev.KsError) as e:
        sim.adjoint_run(2, 2)
    assert e.value.code == 2
    deck, lo, hi, cts = decks.adjoint_c3(**SMALL)
    adaptive = cuda_dev.Incflo(deck + "\ntime.fixed_dt = -1\ntime.cfl = 0.5\n")
    with pytest.raises(cuda_dev.KsError) as e:
        adaptive.set_objective_box(lo, hi)
    assert e.value.code == 2
    sim = cuda_dev.Incflo(deck)
    with pytest.raises(cuda_dev.KsError) as e:
        sim.adjoint_run(2, 2)  # no objective box
    assert e.value.code == 6
    with pytest.raises(cuda_dev.KsError):
        sim.set_disk_ct([0.7])


FARM = dict(nx=48, ny=48, nz=24, dx=20.0, dz=20.0, dcells=6, ngrid=2, spacing=3.0, dt=1.0, nr=3, nt=8)


def test_abl_farm_ct_gradient(cuda_dev):
    """Wall model, slip top, Smagorinsky, geostrophic + Coriolis, 2 x 2 disks."""
    deck, lo, hi, cts = decks.abl_disks(precision="fp64", **FARM)
    sim = cuda_dev.Incflo(deck)
    sim.InitData()
    sim.set_objective_box(lo, hi)
    x0 = {f: sim.get_field(f) for f in ("velocity", "gp", "p")}
    ct = np.array(cts)
    J, g = adjoint(sim, x0, ct, 10, 4)
    assert J == forward_J(sim, x0, ct, 10)
    assert np.all(g < 0)
    assert fd_rel(sim, x0, ct, 10, g, 1e-6) < TOL


@pytest.mark.parametrize("extra", ["", "\nks.precision = mixed\n"])
def test_abl_farm_one_step_vjp(cuda_dev, extra):
    """Every reverse pass of the ABL step (walls, wall model, Smagorinsky,
    Coriolis, disks) at once; the mixed-precision handle re-linearises in FP64."""
    deck, lo, hi, cts = decks.abl_disks(precision="fp64", **FARM)
    sim = cuda_dev.Incflo(deck + extra)
    sim.InitData()
    for _ in range(3):
        sim.step()
    sim.set_precision(0)
    xs = {f: sim.get_field(f) for f in ("velocity", "gp", "p")}
    rng = np.random.default_rng(5)
    sh = xs["velocity"].shape
    w, w2, du, dg = rng.standard_normal(sh), rng.standard_normal(sh), rng.uniform(-1, 1, sh), rng.uniform(-1, 1, sh)

    def F(h):
        restore(sim, xs)
        sim.set_field("velocity", xs["velocity"] + h * du)
        sim.set_field("gp", xs["gp"] + h * dg)
        sim.step()
        return float((w * sim.get_field("velocity")).sum() + (w2 * sim.get_field("gp")).sum())

    restore(sim, xs)
    sim.adjoint_reset()
    sim.set_field("velocity_adjoint", w)
    sim.set_field("gp_adjoint", w2)
    sim.adjoint_step()
    adj = float((sim.get_field("velocity_adjoint") * du).sum() + (sim.get_field("gp_adjoint") * dg).sum())
    h = 1e-9  # random directions cross the scheme's jumps at larger h
    assert abs((F(h) - F(-h)) / (2 * h) - adj) <= 1e-5 * abs(adj)


def test_mixed_forward_fp64_adjoint(cuda_dev):
    """Mixed-precision forward with the FP64 reverse sweep against FP64 finite differences."""
    deck, lo, hi, cts = decks.abl_disks(precision="mixed", **FARM)
    sim = cuda_dev.Incflo(deck)
    sim.InitData()
    sim.set_objective_box(lo, hi)
    x0 = {f: sim.get_field(f) for f in ("velocity", "gp", "p")}
    ct = np.array(cts)
    J_mixed, g = adjoint(sim, x0, ct, 10, 3)
    sim.set_precision(0)
    J64 = forward_J(sim, x0, ct, 10)
    assert abs(J_mixed - J64) <= 1e-6 * J64
    assert fd_rel(sim, x0, ct, 10, g, 1e-6) < 1e-3
