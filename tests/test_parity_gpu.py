"""Parity of the CUDA engine with the CPU oracle (and, through the golden
fixtures, with the AN5D artifact's own CPU path).

Exact mode must be bit-identical. FMA mode must agree within the normwise
tolerance max|gpu - cpu| / max|cpu| <= 1e-5 (float) / 1e-12 (double) over the
result plane T%2. Every launch goes through the C ABI (gbs_run)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import pyoracle as po
from gbstencil import capi

pytestmark = pytest.mark.gpu

TOL = {np.dtype(np.float32): 1e-5, np.dtype(np.float64): 1e-12}
GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_outputs.json").read_text())["cases"]
DT = {"float": np.float32, "double": np.float64}
NAMES_2D = [s["name"] for s in capi.TABLE if s["dim"] == 2]
NAMES_3D = [s["name"] for s in capi.TABLE if s["dim"] == 3]


def has_exact(name):
    """3d125pt has no exact form in the engine (its float build sums groups
    in float and combines them in double)."""
    return capi.info(name).get("exact", True)


def max_class(name, dt, mode):
    """Largest fused degree the build instantiates (mirrors csrc/inst.cu);
    0 when the mode is not built for the stencil."""
    s = capi.info(name)
    if mode == "exact" and not has_exact(name):
        return 0
    if s.get("groups") or s["dim"] == 3:  # degrees limited by shared memory: ask the planner
        import ctypes
        top = 0
        for bt in range(1, 9):
            d, _ = capi.make_desc(name, dt, 64, 2 * bt, mode, bt=bt)
            if capi.lib().gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) != capi.GBS_OK:
                break
            top = bt
        return top
    if np.dtype(dt) == np.float64:
        return 2
    if s["kind"] == "gradient":
        return 2
    cap = 8 if mode == "fma" else 4
    if s["form"] == "assoc":
        return cap if s["rad"] == 1 else (4 if s["rad"] == 2 else 2)
    return cap if s["rad"] <= 2 else 4


def random_grid(name, n, dt, seed):
    """Uniform [0,1) cells, halos identical in both planes."""
    shape, nn = po.grid_shape(name, n)
    rng = np.random.default_rng(seed)
    A = np.empty(shape, dt)
    A[0] = rng.random(shape[1:])
    A[1] = A[0]
    return A, nn


def compare(name, A0, nn, T, dt, mode, bt, sl=0, coef=None):
    ref = A0.copy()
    po.run(name, ref, nn, T, coef=coef)
    gpu = A0.copy()
    d, keep = capi.make_desc(name, dt, nn, T, fp_mode=mode, bt=bt, sl=sl, coef=coef)
    capi.run_host(d, gpu)
    t = T % 2
    r = po.BY_NAME[name][1]["rad"]
    # the halo of both planes is never written
    inner = tuple(slice(r, -r) for _ in nn)
    for pl in (0, 1):
        m = np.ones(A0.shape[1:], bool)
        m[inner] = False
        assert np.array_equal(gpu[pl][m], A0[pl][m]), "halo modified"
    if mode == "exact":
        bad = np.argwhere(gpu[t].view(np.uint8 if False else gpu.dtype) != ref[t])
        assert np.array_equal(gpu[t], ref[t]), (
            f"{len(bad)} cells differ, first {bad[:3].tolist()}, "
            f"normwise {po.normwise_error(gpu, ref, T):.3e}")
    else:
        err = po.normwise_error(gpu, ref, T)
        assert err <= TOL[np.dtype(dt)], err
    return gpu, ref


CASES_2D = [  # (n, T, sl)
    (23, 1, 0), (23, 2, 0), (23, 7, 0), (70, 9, 0), (130, 5, 7), ((37, 150), 6, 0),
    ((300, 41), 11, 13), (257, 16, 0),
]


@pytest.mark.parametrize("mode", ["exact", "fma"])
@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("name", NAMES_2D)
def test_parity_2d(name, dt, mode):
    mc = max_class(name, dt, mode)
    seed = 0
    for n, T, sl in CASES_2D:
        for bt in sorted({1, 2, mc, max(1, mc // 2), 3 if mc >= 3 else 1}):
            if bt > mc:
                continue
            seed += 1
            A0, nn = random_grid(name, n, dt, seed)
            compare(name, A0, nn, T, dt, mode, bt, sl=sl)


@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("name", NAMES_2D)
def test_parity_2d_reference_init(name, dt):
    """The artifact's own init_grid values (0..1000) and source literals."""
    n, T = 200, 12
    A0 = po.init_grid(name, n, dt)
    compare(name, A0, [n, n], T, dt, "exact", max_class(name, dt, "exact"))
    compare(name, A0, [n, n], T, dt, "fma", max_class(name, dt, "fma"))


@pytest.mark.parametrize("name", ["star2d1r", "j2d5pt", "box2d2r"])
def test_parity_2d_random_coefficients(name):
    rng = np.random.default_rng(5)
    nt = capi.info(name)["nterms"]
    c = rng.random(nt)
    c = (c / c.sum()).astype(np.float32)
    if capi.info(name)["divisor"]:
        c = c * np.float32(capi.info(name)["divisor"])
    A0, nn = random_grid(name, 150, np.float32, 9)
    compare(name, A0, nn, 20, np.float32, "exact", 4, coef=c)


@pytest.mark.parametrize("case", GOLDEN,
                         ids=lambda c: f"{c['stencil']}-{c['dtype']}-{c['compsize']}-{c['timestep']}")
def test_exact_mode_matches_artifact_golden(case):
    """Bit-identical to the artifact's own CPU path (committed digests). A
    stencil without an exact form: FMA mode within tolerance of the oracle,
    whose result carries the artifact's digest."""
    name, dt = case["stencil"], DT[case["dtype"]]
    n, T = case["compsize"], case["timestep"]
    A = po.init_grid(name, n, dt)
    if not has_exact(name):
        ref = A.copy()
        po.run(name, ref, n, T)
        assert hashlib.sha256(np.ascontiguousarray(ref[T % 2]).tobytes()).hexdigest() == case["sha256"]
        d, _ = capi.make_desc(name, dt, n, T, fp_mode="fma")
        capi.run_host(d, A)
        assert po.normwise_error(A, ref, T) <= TOL[np.dtype(dt)]
        return
    d, _ = capi.make_desc(name, dt, n, T, fp_mode="exact")
    capi.run_host(d, A)
    assert hashlib.sha256(np.ascontiguousarray(A[T % 2]).tobytes()).hexdigest() == case["sha256"]


CASES_3D = [  # (n, T, sl)
    (11, 1, 0), (11, 2, 0), (20, 3, 0), ((13, 40, 150), 4, 0), (70, 3, 9), ((37, 9, 300), 5, 0),
]


@pytest.mark.parametrize("mode", ["exact", "fma"])
@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("name", NAMES_3D)
def test_parity_3d(name, dt, mode):
    mc = max_class(name, dt, mode)
    if mc == 0:  # not built: refused, not computed
        d, _ = capi.make_desc(name, dt, 11, 2, fp_mode=mode)
        A = np.zeros(po.grid_shape(name, 11)[0], dt)
        with pytest.raises(capi.GbsError) as e:
            capi.run_host(d, A)
        assert e.value.status == capi.GBS_ERR_UNSUPPORTED
        return
    seed = 100
    for n, T, sl in CASES_3D:
        for bt in sorted({1, mc, min(2, mc), max(1, mc // 2)}):
            seed += 1
            A0, nn = random_grid(name, n, dt, seed)
            compare(name, A0, nn, T, dt, mode, bt, sl=sl)


@pytest.mark.parametrize("dt", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("name", NAMES_3D)
def test_parity_3d_reference_init(name, dt):
    n, T = 40, 5
    A0 = po.init_grid(name, n, dt)
    if has_exact(name):
        compare(name, A0, [n, n, n], T, dt, "exact", max_class(name, dt, "exact"))
    compare(name, A0, [n, n, n], T, dt, "fma", max_class(name, dt, "fma"))


@pytest.mark.parametrize("name,dt", [("box3d1r", np.float64), ("star3d2r", np.float32), ("j3d27pt", np.float32)])
def test_parity_3d_block_shapes(name, dt):
    """Every built tile height gives the same bits (the arithmetic of a cell
    does not depend on the tiling) and the oracle's result within tolerance."""
    import ctypes
    outs = []
    for bs1 in (64, 32):
        d, _ = capi.make_desc(name, dt, 70, 5, "fma", bt=1, bs1=bs1)
        if capi.lib().gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) != capi.GBS_OK:
            continue
        A0, nn = random_grid(name, [70, 45, 150], dt, 400)
        ref = A0.copy()
        po.run(name, ref, nn, 5)
        gpu = A0.copy()
        d, _ = capi.make_desc(name, dt, nn, 5, fp_mode="fma", bt=1, bs1=bs1)
        capi.run_host(d, gpu)
        assert po.normwise_error(gpu, ref, 5) <= TOL[np.dtype(dt)]
        outs.append(gpu)
    assert len(outs) == 2 and np.array_equal(outs[0][1], outs[1][1])
