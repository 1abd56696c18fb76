"""Binomial checkpoint schedule of the reverse sweep (host-only, no GPU).

ks_checkpoint_cost is the fewest forward steps, beyond the one each reverse
step recomputes, that reverse n steps with c checkpoint slots (the first
holding the initial state).  It must equal the revolve bound of Griewank and
Walther (ACM TOMS 26 (2000) 19-45): t n - C(c + t, t - 1) with t the least
integer such that C(c + t, t) >= n."""
from math import comb

import pytest


def revolve_bound(n, c):
    t = 0
    while comb(c + t, t) < n:
        t += 1
    return t * n - comb(c + t, t - 1) if t > 0 else 0


def test_cost_equals_revolve_bound(ks_lib):
    for n in range(1, 90):
        for c in range(1, 14):
            assert ks_lib.checkpoint_cost(n, c) == revolve_bound(n, c), (n, c)


def test_store_all_and_single_slot(ks_lib):
    assert ks_lib.checkpoint_cost(40, 40) == 39  # one forward sweep
    assert ks_lib.checkpoint_cost(40, 100) == 39
    assert ks_lib.checkpoint_cost(40, 1) == 40 * 39 // 2  # recompute from the start for every step
    assert ks_lib.checkpoint_cost(1, 1) == 0


def test_c4_schedule_is_cheap(ks_lib):
    # 200 steps with 12 slots: under three extra forward sweeps (495 steps)
    assert ks_lib.checkpoint_cost(200, 12) == 495


def test_invalid_arguments(ks_lib):
    with pytest.raises(ks_lib.KsError):
        ks_lib.checkpoint_cost(0, 3)
    with pytest.raises(ks_lib.KsError):
        ks_lib.checkpoint_cost(10, 0)
