"""Per-stencil error of the engine against the CPU oracle in the same
precision (the artifact's -c comparison) and against a higher-precision
oracle (float stencils: the double oracle on the same inputs and float
coefficients widened exactly; double stencils: the long-double oracle).

Inputs are the artifact's own (init_grid, common.h:44-56: values in
[0, 1000], and the source literals), the fused degree the engine uses at the
configuration sizes (4096^2 in 2-D, 256^3 in 3-D), both fp modes. The bound
checked is the parity bound against the same-precision oracle (exact mode:
bit for bit; FMA mode: normwise 1e-5 float / 1e-12 double); the
higher-precision error is recorded, not bounded (it is the rounding error of
the stencil itself in that precision, which the artifact's CPU path has
too). With GBS_ERROR_REPORT=<path> the table is written there as JSON."""
import json
import os

import numpy as np
import pytest

import pyoracle as po
from gbstencil import capi

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float32): 1e-5, np.dtype(np.float64): 1e-12}
# grid and steps per dimension: the long-double oracle is software quad
# precision on some hosts, so the grids stay small
SIZE = {2: (384, 48), 3: (48, 12)}
NAMES = capi.NAMES
ROWS = []


def config_bt(name, dtype, mode):
    s = capi.info(name)
    n = 4096 if s["dim"] == 2 else 256
    d, _ = capi.make_desc(name, dtype, n, 100, mode)
    return capi.plan(d).bt


@pytest.mark.parametrize("mode", ["exact", "fma"])
@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("name", NAMES)
def test_error_against_oracles(name, dt, mode):
    s = capi.info(name)
    if mode == "exact" and not s.get("exact", True):
        pytest.skip("no exact form (3d125pt)")
    n, T = SIZE[s["dim"]]
    bt = config_bt(name, dt, mode)
    A0 = po.init_grid(name, n, dt)
    gpu = A0.copy()
    d, _ = capi.make_desc(name, dt, n, T, fp_mode=mode, bt=bt)
    capi.run_host(d, gpu)
    same = A0.copy()
    po.run(name, same, n, T)
    hi_t = np.float64 if np.dtype(dt) == np.float32 else np.longdouble
    hi = A0.astype(hi_t)
    po.run(name, hi, n, T, coef=po.reference_coefficients(name, dt).astype(hi_t))
    e_same = po.normwise_error(gpu, same, T)
    t = T % 2
    den = float(np.abs(hi[t]).max()) or 1.0
    e_hi = float(np.abs(gpu[t].astype(hi_t) - hi[t]).max()) / den
    e_cpu_hi = float(np.abs(same[t].astype(hi_t) - hi[t]).max()) / den
    ROWS.append({"stencil": name, "dtype": np.dtype(dt).name, "mode": mode, "bt": bt, "n": n, "T": T,
                 "vs_same_precision": e_same, "vs_higher_precision": e_hi,
                 "cpu_vs_higher_precision": e_cpu_hi})
    if mode == "exact":
        assert np.array_equal(gpu[t], same[t])
    else:
        assert e_same <= TOL[np.dtype(dt)], e_same
    path = os.environ.get("GBS_ERROR_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(ROWS, f, indent=1)
