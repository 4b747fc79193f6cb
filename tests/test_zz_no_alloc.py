"""gbs_batch_run_noalloc: the batched run for callers that may not allocate
device memory themselves (for example code inside a framework whose caching
allocator owns the device budget, or a host loop that must not call
cudaMalloc because it can synchronise the device). It keeps its work list
and counters in a static device array instead of allocating them.

Checked against the planned batch (gbs_batch_plan + gbs_batch_run), through
the C ABI, on two calls in a row; and its size limits. This file is
collected last on purpose, so that a run stopping at the first failure has
already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

import pyoracle as po
from gbstencil import capi
from gbstencil.grid import DeviceGrid

pytestmark = pytest.mark.gpu

SPECS = [("star2d1r", [70, 133], 9), ("box2d2r", [41, 300], 7), ("j2d5pt", [200, 57], 12),
         ("box2d4r", [90, 90], 5), ("star2d3r", [33, 260], 6), ("gradient2d", [64, 64], 4)]


def make_grids(seed):
    out = []
    for i, (name, n, T) in enumerate(SPECS):
        shape, _ = po.grid_shape(name, n)
        rng = np.random.default_rng(seed + i)
        A = np.empty(shape, np.float32)
        A[0] = rng.random(shape[1:], dtype=np.float32)
        A[1] = A[0]
        g = DeviceGrid(name, np.float32, n)
        g.upload(A)
        out.append((g, T, None))
    return out


@pytest.mark.parametrize("mode", ["exact", "fma"])
def test_no_alloc_matches_planned_batch_twice(mode):
    ref = make_grids(11)
    new = make_grids(11)
    stream = torch.cuda.current_stream().cuda_stream
    plan = capi.Batch(ref, fp_mode=mode, mode="persistent")
    for call in range(2):
        plan.run(stream)
        capi.sync(stream)
        capi.batch_run_noalloc(new, fp_mode=mode, stream=stream)
        for (gr, T, _), (gn, _, _) in zip(ref, new):
            a, b = gr.download(), gn.download()
            if mode == "exact":
                assert np.array_equal(a, b), (gr.name, call)
            else:
                assert po.normwise_error(b, a, T) <= 1e-5, (gr.name, call)
    plan.close()


def test_no_alloc_rejects_oversized_batches():
    g = DeviceGrid("star2d1r", np.float32, [8, 8])
    too_many = [(g, 1, None)] * 65
    with pytest.raises(capi.GbsError) as e:
        capi.batch_run_noalloc(too_many)
    assert e.value.status == capi.GBS_ERR_INVALID
    big = DeviceGrid("star2d1r", np.float32, [4096, 4096])
    with pytest.raises(capi.GbsError) as e:
        capi.batch_run_noalloc([(big, 512, None)])  # about 155k work items
    assert e.value.status == capi.GBS_ERR_INVALID
    assert "work items" in capi.lib().gbs_last_error().decode()
