"""Benchmark of the stencil time loop on GB300 (one JSON line on stdout).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload suite3d|star2d1r|batched|adjoint] [--fp-mode fma|exact]

A step is one full time loop (T timesteps) over each grid of the workload:

* suite3d (default): star3d2r and box3d1r, fp32 and fp64, 512^3 interior,
  T=1000, each at the fused degree the planner picks.
* star2d1r: star2d1r fp32, 4096^2 interior, T=100.
* batched: 512 independent fp32 2-D grids, sides log-uniform in [128, 4096]
  per axis, stencil uniform over star2d1r-4r, box2d1r-4r, j2d5pt, j2d9pt,
  T uniform in [16, 512], normalised random coefficients per grid, all
  advanced by ONE CUDA-graph launch (--batch-mode: layered, the default and
  the fastest, persistent or streams); the line also reports the same work
  done by per-grid plain launches, one grid after another.
* adjoint: the gradient of the time loop (gbs_adjoint_forward/backward):
  j2d5pt f32 2048^2 T=1024 (checkpoints every 32, gradients of u_0 and the
  coefficients), gradient2d f64 4096^2 T=512, j3d27pt f32 384^3 T=256 and
  eight j3d27pt grids of 192^3..384^3 (gradients of u_0); the line reports
  each backward against the plain forward loop.

Inputs are synthetic: every cell (halo included) i.i.d. U[0,1) from a fixed
seed, coefficients U[0,1) normalised to sum 1. ``value`` is GCells/s
(interior cell updates per second) with the grids resident in HBM; ``e2e`` is
the same metric through the C ABI's host-buffer entry point gbs_run (pinned
host grids copied in and out inside the timed region). The L2 is flushed
(a 512 MB write) between timed steps.

``--impl reference`` times the artifact's CPU path (the OpenMP restatement
in oracle/, which is bit-identical to it) on the host cores, on a bounded
sample of each grid (fewer timesteps), and reports the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (ROOT, ROOT / "oracle", ROOT / "an5d-artifact_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

import numpy as np  # noqa: E402

METRIC = "GCells/s per stencil fp32/fp64 & % roofline; batched and adjoint vs plain"

WORKLOADS = {
    "suite3d": [("star3d2r", np.float32, 512, 1000), ("star3d2r", np.float64, 512, 1000),
                ("box3d1r", np.float32, 512, 1000), ("box3d1r", np.float64, 512, 1000)],
    "star2d1r": [("star2d1r", np.float32, 4096, 100)],
    # the fp32 3-D grids of the fused-degree sweep (use with --bt)
    "sweep3d": [("star3d2r", np.float32, 512, 100), ("box3d1r", np.float32, 512, 100),
                ("j3d27pt", np.float32, 512, 100)],
}


BATCH_MIX = ["star2d1r", "star2d2r", "star2d3r", "star2d4r", "box2d1r", "box2d2r", "box2d3r", "box2d4r",
             "j2d5pt", "j2d9pt"]


# DRAM bytes (read + write) per interior cell per launch of the dominant
# kernels, from ncu captures of small cases (dram__bytes_read.sum +
# dram__bytes_write.sum over the interior cells of that case), scaled to a
# full launch by its interior cells (a launch reads and writes each plane
# once, so traffic grows in proportion). Keyed by (stencil, dtype, bt); the
# value names the capture, whose summary is under profiles/.
NCU_DRAM_BYTES_PER_CELL = {
    ("box3d1r", "float64", 1): (15.01, "profiles/stencil3d_stream_box3d1r_f64_n256.md (256^3 capture)"),
    ("star3d2r", "float32", 1): (9.01, "profiles/stencil3d_tile_star3d2r_f32_n320.md (320^3 capture)"),
}


def select_work(args):
    """The workload's grids, narrowed by --only and resized by --n / --T
    (used for small profiling cases of one kernel)."""
    work = list(WORKLOADS[args.workload])
    if args.only:
        keep = {tuple(x.split(":")) for x in args.only.split(",")}
        work = [w for w in work if (w[0], np.dtype(w[1]).name) in keep]
        if not work:
            raise SystemExit(f"--only {args.only!r} selects no grid of workload {args.workload}")
    if args.n:
        work = [(a, b, args.n, d) for a, b, c, d in work]
    if args.T:
        work = [(a, b, c, args.T) for a, b, c, d in work]
    return work


def rank_specs(count, rank, world, tmax=512):
    """The batched grids of one rank: rank 0 of a single-GPU run gets the
    standard seeded set; under N ranks each rank gets its own seeded set of
    the same size (weak scaling, no data shared between ranks)."""
    return batched_specs(count, seed=20250101 + (rank if world > 1 else 0), tmax=tmax)


def max_over_ranks(ms: float, world: int, device=None) -> float:
    """The slowest rank's time (all ranks take part; world 1: ms itself)."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def batched_specs(count=512, seed=20250101, tmax=512):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = [int(round(np.exp(rng.uniform(np.log(128), np.log(4096))))) for _ in range(2)]
        name = BATCH_MIX[int(rng.integers(len(BATCH_MIX)))]
        T = int(rng.integers(16, tmax + 1))
        out.append((name, n, T))
    return out


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def random_coefficients(name, dtype, seed):
    from gbstencil import capi
    s = capi.info(name)
    rng = np.random.default_rng(seed)
    c = rng.random(s["nterms"])
    c = c / c.sum()
    if s["divisor"]:
        c = c * s["divisor"]
    return c.astype(dtype)


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for n, v in zip(names, s[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# our engine
# ---------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch
    from gbstencil import capi
    from gbstencil.grid import DeviceGrid

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    work = select_work(args)
    grids, coefs, plans = [], [], []
    for i, (name, dt, n, T) in enumerate(work):
        g = DeviceGrid(name, dt, n, device=dev)
        g.fill_uniform(seed=20250101 + i)
        c = random_coefficients(name, dt, 1000 + i)
        d, keep = g.desc(T, args.fp_mode, args.bt, 0, coef=c, bs1=args.bs1)
        plans.append(capi.plan(d))
        grids.append(g)
        coefs.append(c)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    cells = sum(int(np.prod(g.n)) * T for g, (_, _, _, T) in zip(grids, work))

    def step():
        for g, c, (_, _, _, T) in zip(grids, coefs, work):
            g.run(T, args.fp_mode, args.bt, 0, coef=c, bs1=args.bs1)

    for _ in range(args.warmup):
        step()
    capi.sync(stream.cuda_stream)
    torch.cuda.synchronize()

    # device-resident timing, per grid (for the per-stencil breakdown)
    per_grid_ms = [0.0] * len(grids)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in grids]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            for gi, (g, c, (_, _, _, T)) in enumerate(zip(grids, coefs, work)):
                ev[gi][0].record(stream)
                g.run(T, args.fp_mode, args.bt, 0, coef=c, bs1=args.bs1)
                ev[gi][1].record(stream)
            torch.cuda.synchronize()
            for gi in range(len(grids)):
                per_grid_ms[gi] += ev[gi][0].elapsed_time(ev[gi][1])
    capi.sync(stream.cuda_stream)
    total_ms = max_over_ranks(sum(per_grid_ms), world, dev)
    ms_per_step = total_ms / args.steps
    value = cells * world / (ms_per_step * 1e-3) / 1e9

    # end to end through gbs_run with pinned host grids
    e2e_ms, h2d, d2h = 0.0, 0, 0
    hosts = []
    for g in grids:
        h = torch.empty((2,) + tuple(g.dimsize), dtype=g.buf.dtype).pin_memory()
        h.copy_(torch.from_numpy(g.download()))
        hosts.append(h)
    def e2e_step():
        nonlocal h2d, d2h
        for g, h, c, (_, _, _, T) in zip(grids, hosts, coefs, work):
            d, keep = capi.make_desc(g.name, g.dtype, g.n, T, args.fp_mode, bt=args.bt, bs1=args.bs1, coef=c)
            capi.run_host(d, h.numpy())
    e2e_samples = []
    if not args.no_e2e:
        e2e_step()  # allocates gbs_run's device buffer once
        torch.cuda.synchronize()
        for _ in range(max(1, min(args.steps, args.e2e_steps))):
            t0 = time.perf_counter()
            e2e_step()
            e2e_samples.append(round((time.perf_counter() - t0) * 1e3, 3))
        e2e_ms = statistics.median(e2e_samples)
    h2d = sum(int(h.numel()) * h.element_size() for h in hosts)
    d2h = h2d
    del hosts

    # each grid's kernel (the same degree and tiling) on a reduced number of
    # steps, against the CPU oracle in the same precision
    errs, err_note = [None] * len(grids), None
    if not args.no_check:
        import pyoracle as po
        for i, (g, c, p) in enumerate(zip(grids, coefs, plans)):
            Tc = 2 * p.bt if p.bt > 1 else 4
            g.fill_uniform(seed=20250101 + i)
            A = g.download()
            g.run(Tc, args.fp_mode, p.bt, 0, coef=c, bs1=p.bs1 if args.bs1 else 0)
            capi.sync(stream.cuda_stream)
            got = g.download()
            po.run(g.name, A, g.n, Tc, coef=c)
            errs[i] = float(f"{po.normwise_error(got, A, Tc):.3e}")
            del A, got
        err_note = ("max_err_vs_oracle: normwise max|gpu-cpu|/max|cpu| over plane T%2 after T = 2*bt steps "
                    "(4 when bt = 1) of the timed kernel at the full grid size, against the CPU oracle in the "
                    "same precision; bound 1e-5 (float), 1e-12 (double)")

    # roofline of each grid: Roofline(bt) = min(B_HBM*bt/(2S), P_FP/FPP) cell
    # updates per second; the binding roof is the smaller term
    hbm, peak_kind = load_peaks()
    fp_peak = {np.dtype(np.float32): capi.measure_fp_peak(np.float32),
               np.dtype(np.float64): capi.measure_fp_peak(np.float64)}
    per = []
    for i, (nm, d_, n_, T_) in enumerate(work):
        ms = per_grid_ms[i] / args.steps
        gc = int(np.prod(grids[i].n)) * T_ / (ms * 1e-3) / 1e9
        s_ = capi.info(nm)
        Sb = np.dtype(d_).itemsize
        bt = plans[i].bt
        roof_hbm = hbm * 1e9 * bt / (2 * Sb) / 1e9
        roof_fp = fp_peak[np.dtype(d_)] * 1e9 / s_["fpp"] / 1e9
        roof = min(roof_hbm, roof_fp)
        roof1 = min(hbm * 1e9 / (2 * Sb) / 1e9, roof_fp)
        per.append({"stencil": nm, "dtype": np.dtype(d_).name, "n": n_, "T": T_, "bt": bt,
                    "launches": plans[i].launches, "ms": round(ms, 4), "gcells_s": round(gc, 2),
                    "bound": ("hbm" if roof_hbm <= roof_fp else ("fp64" if Sb == 8 else "fp32")),
                    "roofline_gcells_s": round(roof, 1), "frac_roofline": round(gc / roof, 4),
                    "roofline_bt1_gcells_s": round(roof1, 1), "max_err_vs_oracle": errs[i]})

    # the dominant kernel (largest device time), against its binding roof
    gi = int(np.argmax(per_grid_ms))
    name, dt, n, T = work[gi]
    p = plans[gi]
    S = np.dtype(dt).itemsize
    ncell = int(np.prod(grids[gi].n))
    launch_ms = per_grid_ms[gi] / args.steps / max(1, p.launches)
    # algorithmic work per launch: each cell read and written once (bytes),
    # fpp flops per cell update, bt updates per cell (flops)
    alg_bytes = 2 * S * ncell
    hbm_achieved = alg_bytes / (launch_ms * 1e-3) / 1e9
    fpp = capi.info(name)["fpp"]
    fp_achieved = fpp * p.bt * ncell / (launch_ms * 1e-3) / 1e9
    per_cell = NCU_DRAM_BYTES_PER_CELL.get((name, np.dtype(dt).name, p.bt))
    traffic = None if per_cell is None else int(per_cell[0] * ncell)
    hbm_block = {"bound": "hbm", "achieved": round(hbm_achieved, 1), "peak": hbm, "unit": "GB/s",
                 "frac": round(hbm_achieved / hbm, 4), "traffic": traffic,
                 "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback 6.8 TB/s"}
    fp_block = {"bound": "fp64" if S == 8 else "fp32", "achieved": round(fp_achieved, 1),
                "peak": round(fp_peak[np.dtype(dt)], 1), "unit": "GFLOP/s",
                "frac": round(fp_achieved / fp_peak[np.dtype(dt)], 4), "traffic": traffic,
                "flops_per_cell_update": fpp,
                "peak_source": "measured on this GPU by gbs_measure_fp_peak (an FMA loop, 2 flops per FMA); "
                               "MEASURED_PEAKS.json has no FP32/FP64 figure"}
    binding = fp_block if per[gi]["bound"] != "hbm" else hbm_block
    roofline = dict(binding)
    roofline["kernel"] = f"{name} {np.dtype(dt).name} bt={p.bt}, {p.launches} launches of {ncell} cells"
    roofline["traffic_source"] = (f"dram__bytes_read.sum + dram__bytes_write.sum per interior cell from "
                                  f"{per_cell[1]}, times the cells of one launch" if per_cell else
                                  "no capture of this kernel")
    roofline["secondary"] = hbm_block if binding is fp_block else fp_block
    # the aggregate split by element type (the same timed runs)
    by_dtype = {}
    for i, (nm, d_, n_, T_) in enumerate(work):
        k = np.dtype(d_).name
        c, m = by_dtype.get(k, (0, 0.0))
        by_dtype[k] = (c + int(np.prod(grids[i].n)) * T_, m + per_grid_ms[i] / args.steps)
    value_by_dtype = {k: round(c / (m * 1e-3) / 1e9, 3) for k, (c, m) in by_dtype.items()}
    total_ms = sum(m for _, m in by_dtype.values())
    time_share = {k: round(m / total_ms, 4) for k, (c, m) in by_dtype.items()}
    launches = sum(p.launches for p in plans) * args.steps
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GCells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "+".join(sorted({np.dtype(w[1]).name.replace("float", "f") for w in work})),
        "data": "synthetic U[0,1) grids and normalised U[0,1) coefficients, seeded",
        "config": {"workload": args.workload, "grids": [f"{w[0]} {np.dtype(w[1]).name} {w[2]}^{capi.info(w[0])['dim']} T={w[3]}" for w in work],
                   "fp_mode": args.fp_mode, "l2": "flushed between timed steps (512 MB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "value_by_dtype": value_by_dtype,
        "time_share_by_dtype": time_share,
        "per_stencil": per,
        "e2e": None if args.no_e2e else {
            "value": round(cells * world / (e2e_ms * 1e-3) / 1e9, 3), "unit": "GCells/s",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "samples_ms": e2e_samples},
        "err_check": err_note,
        "roofline": roofline,
        "fp_peak_gflops": {k.name: round(v, 1) for k, v in fp_peak.items()},
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    return line


# ---------------------------------------------------------------------------
# CPU path (the artifact's OpenMP loop, restated bit for bit in oracle/)
# ---------------------------------------------------------------------------
def cpu_sample(work, budget_s=12.0, threads=None):
    import pyoracle as po
    if threads:
        po.set_threads(threads)
    cells, secs, parts = 0, 0.0, []
    per_budget = budget_s / len(work)
    for i, (name, dt, n, T) in enumerate(work):
        shape, nn = po.grid_shape(name, n)
        A = np.empty(shape, dt)
        rng = np.random.default_rng(20250101 + i)
        A[0] = rng.random(A.shape[1:], dtype=np.float64 if dt == np.float64 else np.float32)
        A[1] = A[0]
        c = random_coefficients(name, dt, 1000 + i)
        # one step to size the sample, then as many steps as fit the budget
        ms1 = po.timed_run(name, A, n, 1, coef=c)
        Ts = int(max(1, min(T, per_budget * 1e3 / max(ms1, 1e-3))))
        ms = po.timed_run(name, A, n, Ts, coef=c)
        ncell = int(np.prod(nn))
        cells += ncell * Ts
        secs += ms * 1e-3
        parts.append(f"{name} {np.dtype(dt).name} {'x'.join(map(str, nn))} T={Ts}")
    return cells / secs / 1e9, "; ".join(parts)


def batched_cpu_work(args, count=16):
    """A bounded sample of the batched workload for the CPU legs: its first
    ``count`` grids (fp32), each at its own stencil and size."""
    specs = batched_specs(args.batch_grids, tmax=args.batch_tmax)[:count]
    return [(name, np.float32, n, T) for name, n, T in specs]


def cpu_work(args):
    if args.workload == "batched":
        return batched_cpu_work(args)
    if args.workload == "adjoint":
        # the forward loop of each adjoint case (the artifact has no adjoint)
        return [(name, dt, n[0], T) for name, dt, n, T, *_ in ADJOINT_CASES[:3]]
    return select_work(args)


def run_reference(args, rank, world):
    import pyoracle as po
    work = cpu_work(args)
    threads = po.max_threads()
    vals = []
    for _ in range(args.warmup):
        cpu_sample(work, budget_s=args.cpu_budget or 2.0)
    sample = ""
    for _ in range(args.steps):
        v, sample = cpu_sample(work, budget_s=args.cpu_budget or max(2.0, 60.0 / max(1, args.steps)))
        vals.append(v)
    value = statistics.median(vals)
    return {
        "metric": METRIC, "value": round(value, 4), "unit": "GCells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "impl": "reference",
        "dtype": "+".join(sorted({np.dtype(w[1]).name.replace("float", "f") for w in work})),
        "data": "synthetic U[0,1) grids and normalised U[0,1) coefficients, seeded",
        "config": {"workload": args.workload, "grids": [f"{w[0]} {np.dtype(w[1]).name} {w[2]} T={w[3]}" for w in work]},
        "cpu_baseline": {"value": round(value, 4), "unit": "GCells/s", "cores": threads, "kind": "port",
                         "sample": sample + ("; the first 16 grids of the batched workload"
                                             if args.workload == "batched" else "")},
        "e2e": {"value": round(value, 4), "unit": "GCells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_batched(args, rank, world):
    import torch
    from gbstencil import capi
    from gbstencil.grid import DeviceGrid

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    specs = rank_specs(args.batch_grids, rank, world, tmax=args.batch_tmax)
    grids, entries = [], []
    for i, (name, n, T) in enumerate(specs):
        g = DeviceGrid(name, np.float32, n, device=dev)
        g.fill_uniform(seed=7 + i)
        c = random_coefficients(name, np.float32, 3000 + i)
        grids.append(g)
        entries.append((g, T, c))
    stream = torch.cuda.current_stream(dev)
    batch = capi.Batch(entries, fp_mode=args.fp_mode, mode=args.batch_mode)
    st = batch.stats()
    cells = st.cell_updates
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(args.warmup):
        batch.run(stream.cuda_stream)
    capi.sync(stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms = 0.0
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0.record(stream)
            batch.run(stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
    capi.sync(stream.cuda_stream)
    ms = max_over_ranks(ms, world, dev)
    ms_step = ms / args.steps
    value = cells * world / (ms_step * 1e-3) / 1e9

    # the same work as per-grid plain launches, one grid after another
    def plain():
        for g, T, c in entries:
            g.run(T, args.fp_mode, args.bt, 0, coef=c, bs1=args.bs1)
    plain()
    capi.sync(stream.cuda_stream)
    torch.cuda.synchronize()
    flush.fill_(1.0)
    e0.record(stream)
    plain()
    e1.record(stream)
    torch.cuda.synchronize()
    capi.sync(stream.cuda_stream)
    plain_ms = e0.elapsed_time(e1)
    plain_launches = 0
    for g, T, c in entries:
        d, _ = g.desc(T, args.fp_mode, 0, 0, coef=c)
        plain_launches += capi.plan(d).launches

    # end to end: pinned host grids in, one batched replay, grids out
    hosts = []
    for g in grids:
        h = torch.empty((2,) + tuple(g.dimsize), dtype=torch.float32).pin_memory()
        h.copy_(torch.from_numpy(g.download()))
        hosts.append(h)
    def e2e_step():
        for g, h in zip(grids, hosts):
            g.upload(h.numpy(), stream=stream.cuda_stream)
        batch.run(stream.cuda_stream)
        for g, h in zip(grids, hosts):
            g.download(h.numpy(), stream=stream.cuda_stream)
        torch.cuda.synchronize()
    e2e_step()
    t0 = time.perf_counter()
    e2e_step()
    e2e_ms = (time.perf_counter() - t0) * 1e3
    capi.sync(stream.cuda_stream)
    hbytes = sum(int(h.numel()) * 4 for h in hosts)
    hbm, peak_kind = load_peaks()
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GCells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: 512 seeded grids, U[0,1) cells, normalised U[0,1) coefficients",
        "config": {"workload": "batched", "grids": len(specs), "cell_updates": cells,
                   "sides": "log-uniform [128, 4096] per axis", "T": "uniform [16, 512]",
                   "stencils": BATCH_MIX, "fp_mode": args.fp_mode, "items": st.items, "ctas": st.ctas,
                   "batch_mode": args.batch_mode, "graph_kernels": st.kernels,
                   "l2": "flushed between timed steps (512 MB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "batched_vs_plain": {"plain_gcells_s": round(cells / (plain_ms * 1e-3) / 1e9, 3),
                             "plain_ms": round(plain_ms, 3), "plain_launches": plain_launches,
                             "batched_launches": 1, "ratio": round(plain_ms / ms_step, 3)},
        "e2e": {"value": round(cells * world / (e2e_ms * 1e-3) / 1e9, 3), "unit": "GCells/s",
                "h2d_bytes_per_step": hbytes, "d2h_bytes_per_step": hbytes},
        "roofline": {"bound": "hbm", "achieved": round(st.hbm_bytes / (ms_step * 1e-3) / 1e9, 1), "peak": hbm,
                     "unit": "GB/s", "frac": round(st.hbm_bytes / (ms_step * 1e-3) / 1e9 / hbm, 4),
                     "traffic": None, "kernel": f"the whole {args.batch_mode} graph",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "note": "achieved: algorithmic HBM bytes of the batch (each fused launch of a grid "
                             "reads and writes its interior once, at the degrees the schedule runs) per "
                             "second; the mix has FP32-bound grids (box2d3r/4r), so the HBM roof is "
                             "not reachable for all of it"},
        "clocks": clk.summary(),
        "gpu_launches": args.steps * st.kernels,
    }
    batch.close()
    return line


# The adjoint cases: (stencil, dtype, interior, T, checkpoint interval (or
# a workspace budget in bytes, as "16GB"), loss, coefficient gradients wanted)
ADJOINT_CASES = [
    ("j2d5pt", np.float32, [2048, 2048], 1024, 32, "half_sq_err", True),
    ("gradient2d", np.float64, [4096, 4096], 512, "16GB", "mean_sq", False),
    ("j3d27pt", np.float32, [384, 384, 384], 256, 16, "half_sq", False),
] + [("j3d27pt", np.float32, [n, n, n], 256, 16, "half_sq", False)
     for n in (192, 224, 256, 288, 320, 336, 352, 384)]
# the uneven j3d27pt instances, also run as one batch
BATCH_ADJOINT = [c for c in ADJOINT_CASES[3:]]


def run_adjoint(args, rank, world):
    """Forward with checkpoints + backward (gbs_adjoint_*) per case, against
    the plain forward loop at the tuned degree."""
    import torch
    from gbstencil import capi
    from gbstencil.adjoint import Checkpointed
    from gbstencil.grid import DeviceGrid

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    cases, tot_cells, tot_bwd, tot_e2e, h2d, d2h, launches = [], 0, 0.0, 0.0, 0, 0, 0
    gen = torch.Generator(device=dev)
    todo = list(ADJOINT_CASES)
    clk = ClockSampler(dev.index).__enter__()  # clocks over every timed run below
    if args.only:  # e.g. j2d5pt:float32 (small profiling cases)
        keep = {tuple(x.split(":")) for x in args.only.split(",")}
        todo = [c for c in todo if (c[0], np.dtype(c[1]).name) in keep][:1]
    if args.T:
        todo = [(a, b, c, args.T, e if isinstance(e, str) else min(e, args.T), f, g) for a, b, c, d, e, f, g in todo]
    for ci, (name, dt, n, T, C, loss, want_coef) in enumerate(todo):
        tdt = torch.float32 if dt == np.float32 else torch.float64
        s = capi.info(name)
        shape = [x + 2 * s["rad"] for x in n]
        gen.manual_seed(20250101 + ci)
        u0 = torch.rand(shape, generator=gen, dtype=tdt, device=dev)
        target = torch.rand(shape, generator=gen, dtype=tdt, device=dev)
        cells = int(np.prod(n)) * T

        def lam_of(uT):
            if loss == "half_sq_err":
                return uT - target          # d/du 0.5 |u - target|^2
            if loss == "mean_sq":
                return 2.0 * uT / uT.numel()
            return uT.clone()               # d/du 0.5 |u|^2

        # plain forward at the tuned degree
        g = DeviceGrid(name, dt, n, device=dev)
        g.plane(0).copy_(u0)
        g.plane(1).copy_(u0)
        fwd = []
        for k in range(args.warmup + args.steps):
            flush.fill_(1.0)
            e0.record(stream)
            g.run(T)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= args.warmup:
                fwd.append(e0.elapsed_time(e1))
        capi.sync(stream.cuda_stream)
        plain = capi.plan(g.desc(T)[0])
        del g
        ckw = dict(checkpoint_every=C) if not isinstance(C, str) else dict(budget_bytes=int(float(C[:-2]) * 1e9))
        run = Checkpointed(name, u0, T, **ckw)
        lam = lam_of(run.u_T)
        C, slots, ws_bytes = run.checkpoint_every, run.slots, run.workspace_bytes
        bwd, ck = [], []
        for k in range(args.warmup + args.steps):
            flush.fill_(1.0)
            e0.record(stream)
            run = Checkpointed(name, u0, T, C, slots=slots)
            e1.record(stream)
            torch.cuda.synchronize()
            ck_ms = e0.elapsed_time(e1)
            flush.fill_(1.0)
            e0.record(stream)
            gu, gc = run.backward(lam, want_coef=want_coef)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= args.warmup:
                bwd.append(e0.elapsed_time(e1))
                ck.append(ck_ms)
        capi.sync(stream.cuda_stream)
        if not args.no_e2e:
            # end to end: host u_0 in, forward with checkpoints, backward, host gradient out
            hu0 = u0.cpu().pin_memory()
            hgrad = torch.empty_like(hu0).pin_memory()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            du0 = hu0.to(dev, non_blocking=True)
            run = Checkpointed(name, du0, T, C, slots=slots)
            gu, gc = run.backward(lam_of(run.u_T), want_coef=want_coef)
            hgrad.copy_(gu, non_blocking=True)
            torch.cuda.synchronize()
            tot_e2e += (time.perf_counter() - t0) * 1e3
            h2d += hu0.numel() * hu0.element_size()
            d2h += hgrad.numel() * hgrad.element_size()
        del run
        torch.cuda.empty_cache()
        f_ms, b_ms, c_ms = statistics.median(fwd), statistics.median(bwd), statistics.median(ck)
        # kernel launches per backward step: gradient2d recompute + pre-pass +
        # gather; 2-D linear (<= 32 terms) the fused step (+ recompute for
        # coefficients); 3-D linear halo + transposed step (+ recompute and
        # product kernel for coefficients)
        if s["kind"] == "gradient":
            per_step = 3
        elif s["dim"] == 2 and s["nterms"] <= 32:
            per_step = 2 if want_coef else 1
        else:
            per_step = 4 if want_coef else 2
        launches += (T * per_step + plain.launches) * args.steps
        tot_cells += cells
        tot_bwd += b_ms
        cases.append({"stencil": name, "dtype": np.dtype(dt).name, "n": n, "T": T, "checkpoint_every": C,
                      "stash_slots": slots, "schedule": "two-level" if slots >= 2 * C else "binomial",
                      "workspace_bytes": ws_bytes,
                      "loss": loss, "coef_grad": want_coef, "forward_ms": round(f_ms, 3),
                      "forward_bt": plain.bt, "forward_checkpointed_ms": round(c_ms, 3),
                      "backward_ms": round(b_ms, 3), "backward_vs_forward": round(b_ms / f_ms, 3),
                      "backward_gcells_s": round(cells / (b_ms * 1e-3) / 1e9, 2)})
    # the uneven instances as one batch (gbs_adjoint_forward_batch /
    # gbs_adjoint_backward_batch) against the same instances one at a time
    batch = None
    bnames = [(c[0], c[2], c[3], c[4]) for c in BATCH_ADJOINT]
    if not args.only and not args.T:
        from gbstencil.adjoint import backward_batch, forward_batch
        u0s, lams = [], []
        for i, (name, n, T, C) in enumerate(bnames):
            gen.manual_seed(777 + i)
            shape = [x + 2 * capi.info(name)["rad"] for x in n]
            u0s.append(torch.rand(shape, generator=gen, dtype=torch.float32, device=dev))
        fw, bw = [], []
        for k in range(args.warmup + args.steps):
            flush.fill_(1.0)
            e0.record(stream)
            runs = forward_batch([(nm, u) for (nm, _, _, _), u in zip(bnames, u0s)], bnames[0][2], bnames[0][3])
            e1.record(stream)
            torch.cuda.synchronize()
            f_ms = e0.elapsed_time(e1)
            lams = [r.u_T.clone() for r in runs]
            flush.fill_(1.0)
            e0.record(stream)
            backward_batch(runs, lams)
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= args.warmup:
                fw.append(f_ms)
                bw.append(e0.elapsed_time(e1))
            del runs
        capi.sync(stream.cuda_stream)
        one = {(c["stencil"], tuple(c["n"])): c for c in cases}
        sum_b = sum(one[(nm, tuple(n))]["backward_ms"] for nm, n, _, _ in bnames if (nm, tuple(n)) in one)
        sum_f = sum(one[(nm, tuple(n))]["forward_checkpointed_ms"] for nm, n, _, _ in bnames
                    if (nm, tuple(n)) in one)
        batch = {"instances": [f"{nm} {'x'.join(map(str, n))} T={T}" for nm, n, T, _ in bnames],
                 "forward_checkpointed_ms": round(statistics.median(fw), 3),
                 "backward_ms": round(statistics.median(bw), 3),
                 "one_at_a_time_forward_checkpointed_ms": round(sum_f, 3),
                 "one_at_a_time_backward_ms": round(sum_b, 3),
                 "backward_speedup": round(sum_b / statistics.median(bw), 3)}
        torch.cuda.empty_cache()
    clk.__exit__(None, None, None)
    tot_bwd = max_over_ranks(tot_bwd, world, dev)
    value = tot_cells * world / (tot_bwd * 1e-3) / 1e9
    hbm, peak_kind = load_peaks()
    # dominant case (largest backward time): algorithmic bytes per cell step
    # 2S (linear, dL/du0 only), 6S (with coefficients), 10S (gradient2d:
    # recompute 2S, pre-pass 3S, gather 5S)
    dom = max(cases, key=lambda c: c["backward_ms"])
    S = np.dtype(dom["dtype"]).itemsize
    per_cell = 10 * S if dom["stencil"] == "gradient2d" else (6 * S if dom["coef_grad"] else 2 * S)
    dcells = int(np.prod(dom["n"])) * dom["T"]
    achieved = per_cell * dcells / (dom["backward_ms"] * 1e-3) / 1e9
    return {
        "metric": METRIC, "value": round(value, 3), "unit": "GCells/s (backward cell-steps)", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot_bwd, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic U[0,1) initial grids and targets, seeded",
        "config": {"workload": "adjoint", "cases": [f"{c['stencil']} {c['dtype']} {'x'.join(map(str, c['n']))} "
                                                     f"T={c['T']} C={c['checkpoint_every']}" for c in cases],
                   "l2": "flushed between timed runs (512 MB write)", "parallelism": "replicas" if world > 1 else "single GPU"},
        "adjoint": cases,
        "adjoint_batch": batch,
        "e2e": None if args.no_e2e else {
            "value": round(tot_cells / (tot_e2e * 1e-3) / 1e9, 3), "unit": "GCells/s (forward+backward, host buffers)",
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": None,
                     "kernel": f"backward of {dom['stencil']} {dom['dtype']} {'x'.join(map(str, dom['n']))}",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"},
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }


def launch_ranks(argv, n):
    """Runs this script as n ranks (one process per GPU) under
    torch.distributed.run on this node and returns its exit status; rank 0
    prints the line."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py")]
    # the ranks' arguments travel in the environment: torch.distributed.run
    # would read abbreviations such as --n as its own options
    env = dict(os.environ, GBS_BENCH_ARGV=json.dumps(list(argv)))
    return subprocess.run(cmd, env=env).returncode


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="suite3d", choices=sorted(WORKLOADS) + ["batched", "adjoint"])
    ap.add_argument("--fp-mode", default="fma", choices=["fma", "exact"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--only", default="", help="grids of the workload to keep, e.g. box3d1r:float64")
    ap.add_argument("--n", type=int, default=0, help="interior side length override")
    ap.add_argument("--T", type=int, default=0, help="timestep override")
    ap.add_argument("--bt", type=int, default=0, help="fused degree of every grid (0: the tuned one)")
    ap.add_argument("--bs1", type=int, default=0, help="3-D tile rows of every grid (0: the tuned shape)")
    ap.add_argument("--batch-grids", type=int, default=512, help="batched workload: number of grids")
    ap.add_argument("--batch-tmax", type=int, default=512, help="batched workload: largest T")
    ap.add_argument("--batch-mode", default="layered", choices=["persistent", "layered", "streams"],
                    help="batched workload: scheduling of the work items")
    ap.add_argument("--e2e-steps", type=int, default=3, help="timed host-buffer samples (at most --steps)")
    ap.add_argument("--no-check", action="store_true", help="skip the per-grid error check against the oracle")
    ap.add_argument("--cpu-budget", type=float, default=0.0,
                    help="seconds of CPU work per CPU-baseline sample (0: the default)")
    ap.add_argument("--dist-backend", default="nccl", help="process-group backend of N > 1 ranks")
    if argv is None and os.environ.get("GBS_BENCH_ARGV") and "WORLD_SIZE" in os.environ:
        argv = json.loads(os.environ["GBS_BENCH_ARGV"])
    args = ap.parse_args(argv)
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        # one process per GPU: re-run this script as args.gpus ranks
        return launch_ranks(sys.argv[1:] if argv is None else list(argv), args.gpus)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}", file=sys.stderr)
        return 2
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, world)))
        return 0
    if world > 1:
        import torch
        if args.dist_backend == "nccl" and int(os.environ.get("LOCAL_RANK", 0)) >= torch.cuda.device_count():
            print(f"bench.py: rank {rank} has no GPU of its own ({torch.cuda.device_count()} visible)",
                  file=sys.stderr)
            return 2
        torch.distributed.init_process_group(args.dist_backend)
    if args.workload == "batched":
        line = run_batched(args, rank, world)
    elif args.workload == "adjoint":
        line = run_adjoint(args, rank, world)
    else:
        line = run_ours(args, rank, world)
    if rank == 0:
        if not args.no_cpu:
            import pyoracle as po
            v, sample = cpu_sample(cpu_work(args), budget_s=args.cpu_budget or 12.0)
            line["cpu_baseline"] = {"value": round(v, 4), "unit": "GCells/s", "cores": po.max_threads(),
                                    "kind": "port", "sample": sample}
        print(json.dumps(line))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
