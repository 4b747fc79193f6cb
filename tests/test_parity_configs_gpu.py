"""Parity at the benchmark configurations, in the mode the benchmark times.

The small-grid parity tests cover every stencil, degree and remainder; these
run the timed path itself (FMA mode, the device-buffer entry point
gbs_run_device, the tuned or the named fused degree, one-wave stream
blocks) at the sizes the benchmark runs, and compare plane T%2 with the CPU
oracle in the same precision. Bound: normwise max|gpu - cpu| / max|cpu|
<= 1e-5 (float) / 1e-12 (double).

* star2d1r fp32, 4096^2, T=100 (the 2-D configuration, in full), at the
  tuned degree and at the largest one built;
* the 3-D suite (star3d2r and box3d1r, fp32 and fp64) at 512^3 with T=8 (the
  full grid, fewer steps) and at 128^3 with T=1000 (all the steps);
* star2d1r, j2d5pt and box2d1r fp32 at 16384^2, T=16, at degrees 7 and 5
  (the degrees the artifact-size report runs).

Inputs as the benchmark makes them: every cell U[0,1) from a seed, the
coefficients U[0,1) normalised to sum 1 (times the divisor where the source
divides)."""
import numpy as np
import pytest
import torch

import pyoracle as po
from gbstencil import capi
from gbstencil.grid import DeviceGrid

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float32): 1e-5, np.dtype(np.float64): 1e-12}


def coefficients(name, dtype, seed):
    s = capi.info(name)
    c = np.random.default_rng(seed).random(s["nterms"])
    c = c / c.sum()
    if s["divisor"]:
        c = c * s["divisor"]
    return c.astype(dtype)


def initial(name, n, dtype, seed):
    shape, nn = po.grid_shape(name, n)
    rng = np.random.default_rng(seed)
    A = np.empty(shape, dtype)
    A[0] = rng.random(shape[1:], dtype=np.float64 if dtype == np.float64 else np.float32)
    A[1] = A[0]
    return A, nn


def run_both(name, dtype, n, T, bt, seed):
    """(engine result, oracle result, plan) of one timed-mode run"""
    dtype = np.dtype(dtype)
    A, nn = initial(name, n, dtype, seed)
    c = coefficients(name, dtype, 1000 + seed)
    g = DeviceGrid(name, dtype, nn)
    g.upload(A)
    g.run(T, "fma", bt, 0, coef=c)
    capi.sync(torch.cuda.current_stream().cuda_stream)
    plan = capi.plan(g.desc(T, "fma", bt, 0, coef=c)[0])
    got = g.download()
    del g
    torch.cuda.empty_cache()
    po.run(name, A, nn, T, coef=c)
    return got, A, plan


def check(name, dtype, n, T, bt, seed=1):
    got, want, plan = run_both(name, dtype, n, T, bt, seed)
    t = T % 2
    err = po.normwise_error(got, want, T)
    r = capi.info(name)["rad"]
    inner = tuple(slice(r, -r) for _ in range(got.ndim - 1))
    assert np.isfinite(got[t][inner]).all()
    assert err <= TOL[np.dtype(dtype)], (name, np.dtype(dtype).name, n, T, plan.bt, err)
    if bt:
        assert plan.bt == bt
    return err, plan


@pytest.mark.parametrize("bt", [0, 8])
def test_star2d1r_4096_t100(bt):
    check("star2d1r", np.float32, 4096, 100, bt)


SUITE = [("star3d2r", np.float32), ("star3d2r", np.float64), ("box3d1r", np.float32), ("box3d1r", np.float64)]


@pytest.mark.parametrize("name,dtype", SUITE, ids=lambda v: getattr(v, "__name__", str(v)))
def test_suite3d_512_reduced_steps(name, dtype):
    check(name, dtype, 512, 8, 0)


@pytest.mark.parametrize("name,dtype", SUITE, ids=lambda v: getattr(v, "__name__", str(v)))
def test_suite3d_128_all_steps(name, dtype):
    check(name, dtype, 128, 1000, 0)


@pytest.mark.parametrize("name,bt", [("star2d1r", 7), ("j2d5pt", 7), ("box2d1r", 5)])
def test_2d_16384_t16(name, bt):
    check(name, np.float32, 16384, 16, bt)
