"""Autotuner: the tuning table (CPU) and gbs_tune on the device (GPU)."""
import ctypes

import numpy as np
import pytest

from gbstencil import capi, tune


@pytest.fixture
def fresh_table(tmp_path):
    """An empty table for the test; the shipped one is restored afterwards."""
    capi.lib()
    saved = tmp_path / "saved.txt"
    tune.save(saved)
    tune.clear()
    yield tmp_path
    tune.clear()
    tune.load(saved)


def test_table_set_lookup_save_load(fresh_table):
    assert tune.entries() == 0
    assert tune.lookup("star2d1r", np.float32, 4096) == (0, 0)
    tune.record("star2d1r", np.float32, 4096, bt=3, sl=256, ms_per_step=0.01)
    assert tune.lookup("star2d1r", np.float32, 4096) == (3, 256)
    # same size class (floor(log2(cells)) = 24): same entry
    assert tune.lookup("star2d1r", np.float32, [4096, 4097]) == (3, 256)
    # nearby class: the bt carries over, the stream length does not
    assert tune.lookup("star2d1r", np.float32, 2048) == (3, 0)
    # more than 3 classes away, other dtype or mode: no entry
    assert tune.lookup("star2d1r", np.float32, 256) == (0, 0)
    assert tune.lookup("star2d1r", np.float64, 4096) == (0, 0)
    assert tune.lookup("star2d1r", np.float32, 4096, "exact") == (0, 0)
    # the time loop's plan resolves bt = 0 through the table
    d, _ = capi.make_desc("star2d1r", np.float32, 4096, 100, "fma")
    p = capi.plan(d)
    assert p.bt == 3 and p.sl == 256
    path = fresh_table / "t.txt"
    tune.save(path)
    text = path.read_text()
    assert "star2d1r f32 fma 24 3 256" in text
    tune.clear()
    assert tune.lookup("star2d1r", np.float32, 4096) == (0, 0)
    tune.load(path)
    assert tune.lookup("star2d1r", np.float32, 4096) == (3, 256)


def test_table_rejects_bad_entries(fresh_table):
    bad = fresh_table / "bad.txt"
    bad.write_text("star2d1r f32 fma 24 3\n")
    with pytest.raises(capi.GbsError):
        tune.load(bad)
    bad.write_text("nosuch f32 fma 24 3 0 1.0\n")
    with pytest.raises(capi.GbsError):
        tune.load(bad)
    with pytest.raises(capi.GbsError):
        tune.record("star2d1r", np.float32, 4096, bt=99)
    ok = fresh_table / "ok.txt"
    ok.write_text("# comment\n\nj2d5pt f32 exact 22 2 0 0.5  # trailing comment\n")
    tune.load(ok)
    assert tune.lookup("j2d5pt", np.float32, 2048, "exact") == (2, 0)


def test_shipped_table_is_consistent():
    """Every entry of the shipped table names a built kernel degree."""
    if not tune.DEFAULT_TABLE.exists():
        pytest.skip("no shipped table")
    for line in tune.DEFAULT_TABLE.read_text().splitlines():
        line = line.split("#")[0].split()
        if not line:
            continue
        if len(line) == 7:
            name, dt, mode, cls, bt, sl, ms = line
            bs1 = 0
        else:
            name, dt, mode, cls, bt, sl, bs1, ms = line
        s = capi.info(name)
        assert 1 <= int(bt) <= 16 and int(sl) >= 0 and int(bs1) >= 0 and float(ms) > 0
        d, _ = capi.make_desc(name, np.float32 if dt == "f32" else np.float64, 64, 1, mode, bt=int(bt),
                              bs1=int(bs1))
        assert capi.lib().gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_OK, (s, line)


@pytest.mark.gpu
@pytest.mark.parametrize("name,dtype,n", [("star2d1r", np.float32, 1024), ("j2d5pt", np.float64, 768),
                                          ("star3d1r", np.float32, 96), ("box3d1r", np.float32, 80)])
def test_tune_times_candidates(fresh_table, name, dtype, n):
    best, cands = tune.tune(name, dtype, n, "fma")
    timed = [c for c in cands if c["ms_per_step"] > 0]
    assert timed and best == cands[0] and best["ms_per_step"] == min(c["ms_per_step"] for c in timed)
    assert all(c["redundancy"] >= 1.0 and c["model_ms_per_step"] > 0 for c in cands)
    assert tune.lookup(name, dtype, n) == (best["bt"], best["sl"])
    # the tuned configuration runs and matches an explicit run of the same (bt, sl)
    import torch
    from gbstencil.grid import DeviceGrid
    a, b = DeviceGrid(name, dtype, n), DeviceGrid(name, dtype, n)
    a.fill_uniform(1)
    b.fill_uniform(1)
    a.run(6, "fma")
    b.run(6, "fma", bt=best["bt"], sl=best["sl"], bs1=best["bs1"])
    torch.cuda.synchronize()
    capi.sync(0)
    assert torch.equal(a.plane(0), b.plane(0))


def test_model_prefers_fusion_when_memory_bound():
    """The model's memory term shrinks with bt; its time per step is positive
    and finite for every degree the planner accepts (host arithmetic; without
    a GPU the peak rates fall back to fixed GB300 figures)."""
    times = []
    for bt in (1, 2, 4):
        d, _ = capi.make_desc("star2d1r", np.float32, 4096, 8 * bt, "fma", bt=bt)
        ms = ctypes.c_double(0.0)
        assert capi.lib().gbs_tune_model(ctypes.byref(d), ctypes.byref(ms)) == capi.GBS_OK
        assert 0 < ms.value < 1e3
        times.append(ms.value)
    assert times[0] > times[1] > times[2]


def test_block_shape_choices():
    """bs1 selects the 3-D tile height among the built shapes (gbs_plan
    reports it); other heights, 2-D warps per CTA other than 4 and tile
    widths other than one warp of 16-byte vectors are refused (host
    arithmetic)."""
    L = capi.lib()
    heights = set()
    for bs1 in (0, 64, 32):
        d, _ = capi.make_desc("box3d1r", np.float64, 256, 10, "fma", bt=1, bs1=bs1)
        pi = capi.PlanInfo()
        assert L.gbs_plan(ctypes.byref(d), ctypes.byref(pi)) == capi.GBS_OK
        assert bs1 == 0 or pi.bs1 == bs1
        assert pi.bs2 == 64
        heights.add(pi.bs1)
    assert heights == {64, 32}
    d, _ = capi.make_desc("box3d1r", np.float64, 256, 10, "fma", bt=1, bs1=48)
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_ERR_UNSUPPORTED
    d, _ = capi.make_desc("star2d1r", np.float32, 256, 10, "fma", bs1=8)
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_ERR_UNSUPPORTED
    d, _ = capi.make_desc("star2d1r", np.float32, 256, 10, "fma")
    d.bs2 = 64
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_ERR_UNSUPPORTED
    d.bs2 = 128
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_OK


def test_table_records_block_shape(fresh_table):
    d, _ = capi.make_desc("star3d2r", np.float32, 256, 0, "fma", bs1=32)
    capi.check(capi.lib().gbs_tune_set(ctypes.byref(d), 1, 0, ctypes.c_double(0.5)))
    d0, _ = capi.make_desc("star3d2r", np.float32, 256, 10, "fma")
    assert capi.plan(d0).bs1 == 32          # bs1 = 0 resolves through the table
    path = fresh_table / "t.txt"
    tune.save(path)
    assert "star3d2r f32 fma 24 1 0 32 0.5" in path.read_text()
