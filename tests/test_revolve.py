"""The binomial (revolve) checkpoint schedule and the budget planner of the
adjoint (host arithmetic of libgbstencil.so; no GPU).

Reversing l steps from a stored state with k free snapshot slots (k + 1
stored states) takes, at best, t = r*l - C(k+r+1, k+2) forward steps, where
r is the least integer with C(k+r+1, k+1) >= l (Griewank and Walther, ACM
TOMS 26(1), 2000): the schedule must reach exactly that count and never
hold more than k snapshots."""
import ctypes
from math import comb

import numpy as np
import pytest

from gbstencil import capi


def optimal(l, k):
    if l <= 1:
        return 0
    r = 1
    while comb(k + 1 + r, k + 1) < l:
        r += 1
    return r * l - comb(k + 1 + r, k + 2)


@pytest.mark.parametrize("k", range(0, 7))
def test_revolve_reaches_the_binomial_minimum(k):
    for l in range(1, 80):
        steps, peak = ctypes.c_longlong(-1), ctypes.c_int(-1)
        capi.check(capi.lib().gbs_revolve_cost(l, k, ctypes.byref(steps), ctypes.byref(peak)))
        assert steps.value == optimal(l, k), (l, k, steps.value)
        assert 0 <= peak.value <= k


def test_revolve_with_many_slots_is_one_sweep():
    steps = ctypes.c_longlong(-1)
    capi.check(capi.lib().gbs_revolve_cost(32, 31, ctypes.byref(steps), None))
    assert steps.value == 31


def _plan(name, dtype, n, T, budget):
    d, _ = capi.make_desc(name, dtype, n, T, "fma")
    c, s, b = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_size_t(0)
    st = capi.lib().gbs_adjoint_plan_budget(ctypes.byref(d), int(budget), ctypes.byref(c), ctypes.byref(s),
                                            ctypes.byref(b))
    return st, c.value, s.value, b.value, d


@pytest.mark.parametrize("name,dtype,n,T,budget", [
    ("gradient2d", np.float64, 4096, 512, 16 * 10**9),   # the gradient2d configuration: 16 GB
    ("j2d5pt", np.float32, 2048, 1024, 2 * 10**9),
    ("j2d5pt", np.float32, 2048, 1024, 400 * 10**6),    # forces the binomial schedule
])
def test_budget_plan_fits_and_matches_the_workspace(name, dtype, n, T, budget):
    st, C, slots, nbytes, d = _plan(name, dtype, n, T, budget)
    assert st == capi.GBS_OK
    assert 1 <= C <= T and 0 <= slots and nbytes <= budget
    ws = ctypes.c_size_t(0)
    capi.check(capi.lib().gbs_adjoint_workspace_slots(ctypes.byref(d), C, slots, ctypes.byref(ws)))
    assert ws.value == nbytes


def test_budget_plan_recomputes_more_when_memory_shrinks():
    L = capi.lib()
    costs = []
    for budget in (4 * 10**9, 1 * 10**9, 400 * 10**6, 200 * 10**6):
        st, C, slots, nbytes, d = _plan("j2d5pt", np.float32, 2048, 1024, budget)
        assert st == capi.GBS_OK
        ncp = -(-1024 // C)
        total = 0
        if slots >= 2 * C:
            total = 1024 - ncp
        else:
            for j in range(ncp):
                s = ctypes.c_longlong(0)
                capi.check(L.gbs_revolve_cost(min(C, 1024 - j * C), slots, ctypes.byref(s), None))
                total += s.value
        costs.append(total)
    assert costs == sorted(costs)
    st, *_ = _plan("j2d5pt", np.float32, 2048, 1024, 10 * 10**6)   # below a few planes: nothing fits
    assert st == capi.GBS_ERR_NOMEM


def test_revolve_matches_exhaustive_search():
    """Against a dynamic program over every split point: the fewest forward
    steps to reverse l steps with k free snapshot slots."""
    from functools import lru_cache

    @lru_cache(None)
    def best(l, k):
        if l <= 1:
            return 0
        if k == 0:
            return l * (l - 1) // 2
        return min(m + best(l - m, k - 1) + best(m, k) for m in range(1, l))

    for k in range(0, 5):
        for l in range(1, 70):
            steps = ctypes.c_longlong(-1)
            capi.check(capi.lib().gbs_revolve_cost(l, k, ctypes.byref(steps), None))
            assert steps.value == best(l, k), (l, k)
