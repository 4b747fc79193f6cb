"""gbs_batch_run_noalloc: the batched run for callers that may not allocate
device memory themselves (for example code inside a framework whose caching
allocator owns the device budget, or a host loop that must not call
cudaMalloc because it can synchronise the device). It keeps its work list
and counters in a static device array instead of allocating them.

Checked through the C ABI, on two calls in a row, against the planned batch
(gbs_batch_plan + gbs_batch_run: the same kernel on the same work items, so
bit for bit in both fp modes) and against the CPU oracle (exact mode bit for
bit, FMA mode within the normwise 1e-5 float tolerance); and its size
limits. This file is
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


def initial_grids(seed):
    out = []
    for i, (name, n, T) in enumerate(SPECS):
        shape, _ = po.grid_shape(name, n)
        rng = np.random.default_rng(seed + i)
        A = np.empty(shape, np.float32)
        A[0] = rng.random(shape[1:], dtype=np.float32)
        A[1] = A[0]
        out.append(A)
    return out


def make_grids(hosts):
    out = []
    for (name, n, T), A in zip(SPECS, hosts):
        g = DeviceGrid(name, np.float32, n)
        g.upload(A)
        out.append((g, T, None))
    return out


@pytest.mark.parametrize("mode", ["exact", "fma"])
def test_no_alloc_matches_planned_batch_and_oracle_twice(mode):
    hosts = initial_grids(11)
    ref = make_grids(hosts)
    new = make_grids(hosts)
    # the oracle after one and after two calls (each call advances T steps)
    expect = []
    cpu = [A.copy() for A in hosts]
    for call in range(2):
        for (name, n, T), A in zip(SPECS, cpu):
            po.run(name, A, n, T)
            if T % 2:  # the next call starts from plane 0: hand it u_T
                A[0] = A[1]
        expect.append([A.copy() for A in cpu])
    stream = torch.cuda.current_stream().cuda_stream
    plan = capi.Batch(ref, fp_mode=mode, mode="persistent")
    for call in range(2):
        plan.run(stream)
        capi.sync(stream)
        capi.batch_run_noalloc(new, fp_mode=mode, stream=stream)
        for gi, ((gr, T, _), (gn, _, _)) in enumerate(zip(ref, new)):
            a, b = gr.download(), gn.download()
            assert np.array_equal(a[T % 2], b[T % 2]), (gr.name, call)
            want = expect[call][gi]
            if mode == "exact":
                assert np.array_equal(b[T % 2], want[T % 2]), (gr.name, call)
            else:
                assert po.normwise_error(b, want, T) <= 1e-5, (gr.name, call)
            if T % 2:  # mirror the oracle's hand-over on the device grids
                for g in (gr, gn):
                    g.plane(0).copy_(g.plane(1))
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


def test_no_alloc_refuses_a_capturing_stream():
    """The call copies its tables in and waits on its stream, so it cannot be
    captured: on a capturing stream it returns GBS_ERR_INVALID and issues
    nothing, and the capture stays valid."""
    g = DeviceGrid("star2d1r", np.float32, [8, 8])
    x = torch.zeros(4, device="cuda")
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    status = None
    with torch.cuda.graph(graph, stream=s):
        x.add_(1.0)
        try:
            capi.batch_run_noalloc([(g, 1, None)], stream=s.cuda_stream)
        except capi.GbsError as e:
            status = e.status
    assert status == capi.GBS_ERR_INVALID
    assert "captured" in capi.lib().gbs_last_error().decode()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(x, torch.ones(4, device="cuda"))
