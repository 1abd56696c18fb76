"""Reverse mode of the advance (ks_adjoint_* through the C ABI) on the GPU.

Gradients of J = mean 0.5 |u|^2 over the wake box of the last disk with
respect to the disk thrust coefficients are checked against central finite
differences of the FP64 forward run; the bar is 1e-4 relative to the largest
gradient component.

The discrete forward map is piecewise smooth with jumps: PPM limiter
cases, the trace switch from the parabola to the cell value where a
transverse velocity crosses +-small_vel, and the Riemann state selection
flip somewhere in the grid as a parameter moves.  On the literal 128 x 128 x
64 deck (+-0.2 m/s noise around zero transverse velocity) these jumps are
about 1e-7 apart in Ct and each moves J by 1e-14 to 1e-11 of its value
(test_ct_gradient_c3_jump_scan locates them): a central difference with
h = 1e-6 sums dozens of them into a 1e-3 error.  That check therefore uses
h = 1e-8 (J is resolved to about 1e-15, so roundoff stays below 1e-6 of the
gradient); the same box with a uniform cross-flow (v, w) = (1, 0.5) m/s,
where no transverse velocity crosses zero, is checked with h = 1e-6.
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


def scan_slopes(F, h, n):
    """Slopes of F over the 2n intervals of [-n h, n h] (F evaluated at the
    2n + 1 points).  The discrete map is piecewise smooth: an interval that
    straddles one of its jumps has an outlying slope, the others agree with
    the derivative on their smooth piece."""
    vals = [F(k * h) for k in range(-n, n + 1)]
    return np.diff(vals) / h, vals


def smooth_slope(slopes, atol):
    """The finite-difference derivative with the jumps set aside: the mean of
    the largest group of slopes that agree with one another within atol (the
    intervals on smooth pieces give the same slope; each interval holding a
    jump gives its own), and the group's size."""
    best = []
    for a in slopes:
        grp = [b for b in slopes if abs(b - a) <= atol]
        if len(grp) > len(best):
            best = grp
    return float(np.mean(best)), len(best)


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


def test_ct_gradient_c3_jump_scan(cuda_dev):
    """The literal C3 deck (128 x 128 x 64, 3 disks, 40 steps): J(Ct_k + s)
    scanned in ten intervals.

    Fine scan, steps of 2e-9: most intervals share one slope up to the
    rounding of J (one unit in the last place of J over the step), and that
    slope agrees with the adjoint dJ/dCt_k to 1e-5; the few intervals off it
    hold a jump of the discrete map (a PPM limiter / trace-switch / Riemann
    branch flipping somewhere in the 40 steps), each below 1e-12 of J.

    Coarse scan of disk 0, steps of 2e-7 (the range of the h = 1e-6 central
    difference): nearly every interval holds such jumps, so the slopes scatter
    by up to 1e-3 of the gradient and so does the central difference, which
    is why the gradient check of this deck uses h = 1e-8.  The jumps are not
    the multigrid stopping test: the same scan with every solve run for a
    fixed 16 V-cycles gives the same slopes."""
    sim, x0, ct, _ = make(cuda_dev)
    J0, g = adjoint(sim, x0, ct, 40, 6)
    gmax = np.abs(g).max()
    for k in range(len(ct)):
        e = np.eye(len(ct))[k]
        h = 2e-9
        slopes, vals = scan_slopes(lambda s: forward_J(sim, x0, ct + s * e, 40), h, 5)
        assert vals[5] == J0
        quantum = np.spacing(J0) / h  # one unit in the last place of J, as a slope
        fd, n_smooth = smooth_slope(slopes, 2.5 * quantum)
        assert n_smooth >= 4, (k, slopes)
        assert abs(fd - g[k]) <= 1e-5 * gmax, (k, fd, g[k])
        jumps = (slopes - fd) * h
        assert np.abs(jumps).max() <= 1e-12 * J0, (k, jumps)
        print("disk %d: dJ/dCt %.10f, smooth slope %.10f (%d of 10 intervals), %d with a jump (largest %.1e of J)"
              % (k, g[k], fd, n_smooth, int((np.abs(slopes - fd) > 2.5 * quantum).sum()), np.abs(jumps).max() / J0))
    h = 2e-7
    slopes, vals = scan_slopes(lambda s: forward_J(sim, x0, ct + s * np.eye(len(ct))[0], 40), h, 5)
    dev = np.abs(slopes - g[0])
    assert (dev > 10 * np.spacing(J0) / h).sum() >= 5, slopes  # jumps in most intervals
    assert np.abs((slopes - g[0]) * h).max() <= 1e-10 * J0
    central = (vals[-1] - vals[0]) / (2 * 5 * h)  # = g + (sum of the jumps) / 2e-6
    print("disk 0, steps of 2e-7: slopes off the gradient by up to %.1e of it; central difference at h = 1e-6 off by %.1e"
          % (dev.max() / gmax, abs(central - g[0]) / gmax))


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
    # the perturbation lives in a 16 x 16 x 8 block on the wall-model bottom
    # under the disks: a direction through every cell crosses one of the
    # scheme's branch jumps in most intervals of 1e-9
    mask = np.zeros(sh[1:])
    mask[:8, 8:24, 8:24] = 1.0
    du, dg = du * mask, dg * mask

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
    # compare with the slope the smooth intervals of a scan share (up to the
    # rounding of F), setting aside intervals that hold a jump
    slopes, vals = scan_slopes(F, 1e-9, 4)
    fd, n_smooth = smooth_slope(slopes, 2.5 * np.spacing(abs(vals[4])) / 1e-9)
    assert n_smooth >= 3 and abs(fd - adj) <= 1e-5 * abs(adj), (slopes, adj)


def test_mixed_forward_fp64_adjoint(cuda_dev):
    """Mixed-precision forward and its reverse sweep (the reverse of each FP32
    Godunov / diffusion pass evaluated in FP32, every adjoint array and every
    accumulation FP64) against the FP64 handle's adjoint of the FP64 forward
    (1e-4 of the gradient) and against FP64 finite differences."""
    deck, lo, hi, cts = decks.abl_disks(precision="mixed", **FARM)
    sim = cuda_dev.Incflo(deck)
    sim.InitData()
    sim.set_objective_box(lo, hi)
    x0 = {f: sim.get_field(f) for f in ("velocity", "gp", "p")}
    ct = np.array(cts)
    J_mixed, g = adjoint(sim, x0, ct, 10, 3)
    sim.set_precision(0)
    J64, g64 = adjoint(sim, x0, ct, 10, 3)
    assert abs(J_mixed - J64) <= 1e-6 * J64
    assert np.abs(g - g64).max() <= 1e-4 * np.abs(g64).max(), (g, g64)
    assert fd_rel(sim, x0, ct, 10, g, 1e-6) < 1e-3
