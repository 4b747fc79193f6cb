"""The batched persistent launch (one CUDA-graph-captured kernel over many
uneven grids) gives every grid the same result as the single-grid engine
and the CPU oracle: bit-identical in exact mode, within 1e-5 in FMA mode."""
import numpy as np
import pytest
import torch

import pyoracle as po
from gbstencil import capi
from gbstencil.grid import DeviceGrid

pytestmark = pytest.mark.gpu

MIX = ["star2d1r", "star2d2r", "star2d3r", "star2d4r", "box2d1r", "box2d2r", "box2d3r", "box2d4r",
       "j2d5pt", "j2d9pt", "j2d9pt-gol", "gradient2d"]


def make_batch(seed, count, nmax, tmax):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(count):
        name = MIX[i % len(MIX)] if i < len(MIX) else MIX[rng.integers(len(MIX))]
        n = [int(rng.integers(3, nmax)), int(rng.integers(3, nmax))]
        T = int(rng.integers(0, tmax))
        specs.append((name, n, T))
    return specs


@pytest.mark.parametrize("sched", ["persistent", "layered", "streams"])
@pytest.mark.parametrize("mode", ["exact", "fma"])
def test_batch_matches_oracle(mode, sched):
    specs = make_batch(7, 40, 300, 23)
    grids, hosts, entries = [], [], []
    for i, (name, n, T) in enumerate(specs):
        shape, nn = po.grid_shape(name, n)
        rng = np.random.default_rng(100 + i)
        A = np.empty(shape, np.float32)
        A[0] = rng.random(shape[1:], dtype=np.float32)
        A[1] = A[0]
        g = DeviceGrid(name, np.float32, n)
        g.upload(A)
        coef = None
        if i % 3 == 1 and capi.info(name)["kind"] == "linear":
            c = rng.random(capi.info(name)["nterms"])
            coef = (c / c.sum() * (capi.info(name)["divisor"] or 1)).astype(np.float32)
        grids.append(g)
        hosts.append((A, coef))
        entries.append((g, T, coef))
    b = capi.Batch(entries, fp_mode=mode, mode=sched)
    st = b.stats()
    assert st.grids == len(specs)
    # algorithmic HBM bytes: every time block of a grid reads and writes its
    # interior once, so between one pass per step and one pass per run
    upd = sum(int(np.prod(n)) * T for name, n, T in specs)
    assert st.cell_updates == upd
    assert sum(8 * int(np.prod(n)) for name, n, T in specs if T > 0) <= st.hbm_bytes <= 8 * upd
    s = torch.cuda.current_stream()
    b.run(s.cuda_stream)
    capi.sync(s.cuda_stream)
    for (name, n, T), g, (A, coef) in zip(specs, grids, hosts):
        ref = A.copy()
        po.run(name, ref, n, T, coef=coef)
        out = g.download()
        if mode == "exact":
            assert np.array_equal(out[T % 2], ref[T % 2]), (name, n, T)
        else:
            assert po.normwise_error(out, ref, T) <= 1e-5, (name, n, T)
    # the plan replays: a second run continues from the current state
    b.run(s.cuda_stream)
    capi.sync(s.cuda_stream)
    b.close()


def test_batch_replay_matches_two_runs():
    """Two replays of a plan equal one single-grid run of 2T steps (the
    counters are reset inside the graph)."""
    name, n, T = "box2d1r", [200, 333], 9
    A = po.init_grid(name, 1, np.float32)  # shape placeholder
    shape, nn = po.grid_shape(name, n)
    rng = np.random.default_rng(3)
    A = np.empty(shape, np.float32)
    A[0] = rng.random(shape[1:], dtype=np.float32)
    A[1] = A[0]
    g = DeviceGrid(name, np.float32, n)
    g.upload(A)
    b = capi.Batch([(g, T, None)], fp_mode="exact")
    s = torch.cuda.current_stream()
    b.run(s.cuda_stream)
    capi.sync(s.cuda_stream)
    mid = g.download()
    if T % 2:  # the next run starts from plane 0: bring u_T there, as a caller would
        g.upload(np.stack([mid[1], mid[1]]))
    else:
        g.upload(np.stack([mid[0], mid[0]]))
    b.run(s.cuda_stream)
    capi.sync(s.cuda_stream)
    out = g.download()
    ref = A.copy()
    po.run(name, ref, nn, 2 * T)
    assert np.array_equal(out[T % 2], ref[(2 * T) % 2])
    b.close()


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_batch_3d_streams_matches_oracle(dtype):
    """Uneven 3-D grids (j3d27pt as in the batched adjoint configuration,
    with other 3-D stencils mixed in) in one graph launch of the streams
    schedule: each grid as its own time loop, within the FMA tolerance of
    the oracle."""
    specs = [("j3d27pt", [19, 23, 40], 7), ("j3d27pt", [24, 24, 24], 10), ("j3d27pt", [31, 17, 66], 5),
             ("star3d2r", [20, 30, 41], 6), ("box3d1r", [33, 12, 25], 9), ("star3d1r", [16, 16, 16], 0)]
    tol = 1e-5 if dtype == np.float32 else 1e-12
    grids, hosts, entries = [], [], []
    for i, (name, n, T) in enumerate(specs):
        shape, nn = po.grid_shape(name, n)
        rng = np.random.default_rng(300 + i)
        A = np.empty(shape, dtype)
        A[0] = rng.random(shape[1:])
        A[1] = A[0]
        g = DeviceGrid(name, dtype, n)
        g.upload(A)
        grids.append(g)
        hosts.append(A)
        entries.append((g, T, None))
    b = capi.Batch(entries, fp_mode="fma", mode="streams")
    assert b.stats().grids == len(specs)
    s = torch.cuda.current_stream()
    b.run(s.cuda_stream)
    capi.sync(s.cuda_stream)
    for (name, n, T), g, A in zip(specs, grids, hosts):
        ref = A.copy()
        po.run(name, ref, n, T)
        assert po.normwise_error(g.download(), ref, T) <= tol, (name, n, T)
    b.close()


def test_batch_work_item_schedules_refuse_3d_and_double():
    g3 = DeviceGrid("j3d27pt", np.float32, [12, 12, 12])
    for sched in ("persistent", "layered"):
        with pytest.raises(capi.GbsError) as e:
            capi.Batch([(g3, 2, None)], fp_mode="fma", mode=sched)
        assert e.value.status == capi.GBS_ERR_UNSUPPORTED
    g2 = DeviceGrid("star2d1r", np.float64, [40, 40])
    with pytest.raises(capi.GbsError) as e:
        capi.Batch([(g2, 2, None)], fp_mode="fma", mode="persistent")
    assert e.value.status == capi.GBS_ERR_UNSUPPORTED
