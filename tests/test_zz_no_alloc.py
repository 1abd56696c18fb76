"""Allocation-free diffusion entry point, ks_divtau_noalloc.

Callers that cannot allocate device memory where they need the viscous term
(hosts whose device memory is owned by another allocator, plug-in code inside
an application that owns every allocation, loops that must not trigger an
allocation) call ks_divtau_noalloc, which keeps its face-flux scratch in a
static device array instead of calling cudaMalloc.
This test calls it through the C ABI, twice in a row on the same inputs, and
compares each result with the diffusion term the regular advance computed
(field "diff_term" after one step), within the parity tolerance of the GPU
tests.  It lives in a file of its own, collected last.
"""
import ctypes

import numpy as np
import pytest

from kynema_sgf_gb300 import decks

pytestmark = pytest.mark.gpu
TOL = 1e-9
KS_ERR_ARG = 6


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _check(cuda_dev, deck, dims, h, z_periodic, wall_model=0):
    import torch
    sim = cuda_dev.Incflo(deck)
    sim.InitData()
    assert sim.step()
    # after a step: diff_term = divtau(velocity_old) with velocity_mueff (and,
    # under the wall model, the wall gradient the step formed from velocity_old)
    vel = torch.from_numpy(sim.get_field("velocity_old").ravel().copy()).cuda()
    mu = torch.from_numpy(sim.get_field("velocity_mueff").ravel().copy()).cuda()
    wg = torch.from_numpy(sim.get_field("wall_grad").ravel().copy()).cuda() if wall_model else None
    ref = sim.get_field("diff_term").ravel()
    lib = cuda_dev.load_library()
    out = torch.empty_like(vel)
    nx, ny, nz = dims
    for _ in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.ks_divtau_noalloc(_ptr(vel), _ptr(mu), _ptr(wg) if wall_model else None, _ptr(out), nx, ny, nz, h[0], h[1], h[2],
                                   z_periodic, wall_model, None)
        torch.cuda.synchronize()
        assert rc == 0
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        err = np.abs(got - ref).max() / np.abs(ref).max()
        assert err < TOL, "no-alloc divtau differs from the advance's diff_term: %.3e" % err


def test_noalloc_divtau_periodic(cuda_dev):
    n = 32
    h = 2 * np.pi / n
    _check(cuda_dev, decks.tgv(n, steps=2), (n, n, n), (h, h, h), 1)


def test_noalloc_divtau_slip_walls(cuda_dev):
    deck = decks.abl(32, 32, 16, steps=2).replace("zlo.type = wall_model", "zlo.type = slip_wall")
    _check(cuda_dev, deck, (32, 32, 16), (20.0, 20.0, 20.0), 0)


def test_noalloc_divtau_wall_model(cuda_dev):
    """The ABL deck as benchmarked: Moeng wall model at z-lo (wall gradient
    2 x nx*ny from the handle), slip wall at z-hi, Smagorinsky viscosity."""
    _check(cuda_dev, decks.abl(32, 32, 16, steps=2), (32, 32, 16), (20.0, 20.0, 20.0), 0, wall_model=1)


def test_noalloc_rejects_oversize(cuda_dev):
    import torch
    lib = cuda_dev.load_library()
    t = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = lib.ks_divtau_noalloc(_ptr(t), _ptr(t), None, _ptr(t), 128, 64, 64, 1.0, 1.0, 1.0, 1, 0, None)
    assert rc == KS_ERR_ARG
