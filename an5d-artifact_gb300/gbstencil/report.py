"""The artifact's result tables, produced with this engine.

    python -m gbstencil.report run    --prec float  --out gb300      # compiled/run.sh
    python -m gbstencil.report sconf  --out gb300                    # run_sconf.sh
    python -m gbstencil.report regcap --caps 0,32,64,96 --out gb300  # all.sh REGNUM loop
    python -m gbstencil.report sweep  -t 100 --out gb300             # make.sh --bt, 1..8

``run`` writes ``<out>/<prec>_run.csv`` in the format of compiled/run.sh
(compiled/run.sh:14,35,58): ``Stencil,bS1,bS2,bT,sl,Model,Measured`` with one
row per stencil, bS2 empty for 2-D, Model and Measured in GFLOP/s
(BENCH_FPP flops per cell update, as common.h's calc_gflops counts them).
Sizes and repetitions follow the artifact (-s 16384 for 2-D, 512 for 3-D,
-t 1000, -n 5: one warm-up run, then the average of n runs), each run
through gbs_run on a host grid, which times the device loop only, as
kernel_stencil does. bS1/bS2/bT/sl are the configuration the engine runs:
2-D bS1 = threads per CTA (one 32*V-column strip per warp), 3-D bS1 x bS2 =
tile rows x tile columns; Model is the autotuner's roofline model for it.

``sconf`` repeats run_sconf.sh's fixed configuration (make_sconf.sh: bt=4,
bs1=128 for 2-D, 32x32 with sl=512 for 3-D) for its seven stencils, in float
and double, with bt clamped to the largest fused degree the build has.

``sweep`` times every fused degree bt = 1 .. --bt-max that the build has
for each stencil of --stencils (default star3d2r,box3d1r) in float and
double at -s (3-D: --s3), the degree sweep of the artifact's make.sh --bt
option; the grid stays on the device and each of -n runs is timed with CUDA
events. It writes ``<out>/sweep.csv``: Stencil, Precision, bT, bS1, bS2,
sl, redundancy (computed cells per output cell), Model and Measured GCells/s,
and Measured as a share of Roofline(bt) = min(HBM * bt / (2 * element
bytes), FP peak / flops per cell) with the measured peaks.

``regcap`` runs ``run`` once per register cap (0 = none), each with the
library built by ``python -m gbstencil.build --regcap=N``, and writes
``<out>/<prec>_regcap.csv`` with a RegCap column.
"""
from __future__ import annotations

import argparse
import csv
import ctypes
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

from . import capi

SCONF_STENCILS = ["j2d5pt", "j2d9pt-gol", "j2d9pt", "gradient2d", "star3d1r", "star3d2r", "j3d27pt"]
PREC = {"float": np.float32, "double": np.float64}


def host_grid(name, dtype, n, seed):
    """Both planes equal, every cell U[0,1) from a fixed seed."""
    shape, _ = grid_shape(name, n)
    rng = np.random.default_rng(seed)
    A = np.empty(shape, dtype)
    A[0] = rng.random(shape[1:], dtype=np.float64 if dtype == np.float64 else np.float32)
    A[1] = A[0]
    return A


def grid_shape(name, n):
    s = capi.info(name)
    return (2,) + (n + 2 * s["rad"],) * s["dim"], [n] * s["dim"]


def measure(name, dtype, n, T, reps, bt=0, sl=0, fp_mode="fma"):
    """(config dict, model GFLOP/s, measured GFLOP/s averaged over reps)."""
    s = capi.info(name)
    d, keep = capi.make_desc(name, dtype, n, T, fp_mode, bt=bt, sl=sl)
    p = capi.plan(d)
    model_ms = ctypes.c_double(0.0)
    capi.check(capi.lib().gbs_tune_model(ctypes.byref(d), ctypes.byref(model_ms)))
    flops = float(T) * float(n) ** s["dim"] * s["fpp"]
    A = host_grid(name, dtype, n, 1)
    capi.run_host(d, A)  # warm-up, as the harness's [Device warm-up]
    total = 0.0
    for r in range(reps):
        A = host_grid(name, dtype, n, 2 + r)
        total += capi.run_host(d, A)
    ms = total / reps
    cfg = {"bS1": 128 if s["dim"] == 2 else p.bs1, "bS2": "" if s["dim"] == 2 else p.bs2, "bT": p.bt, "sl": p.sl}
    return cfg, flops / (model_ms.value * T) / 1e6, flops / ms / 1e6


def fmt(x):
    return f"{x:,.0f}"


def cmd_run(args):
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    names = args.stencils.split(",") if args.stencils else capi.NAMES
    path = out / f"{args.prec}_run.csv"
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["Stencil", "bS1", "bS2", "bT", "sl", "Model", "Measured"])
        for name in names:
            s = capi.info(name)
            n = args.s2 if s["dim"] == 2 else args.s3
            cfg, model, meas = measure(name, PREC[args.prec], n, args.t, args.n, fp_mode=args.mode)
            w.writerow([name, cfg["bS1"], cfg["bS2"], cfg["bT"], cfg["sl"], fmt(model), f"{meas:.4f}"])
            f.flush()
            print(f"{name:11s} {args.prec:6s} n={n} T={args.t} bT={cfg['bT']} sl={cfg['sl']} "
                  f"model {model:10.1f} measured {meas:10.1f} GFLOP/s", flush=True)
    return path


def cmd_sconf(args):
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    path = out / "sconf.csv"
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["Stencil", "Precision", "bS1", "bS2", "bT", "sl", "Measured GFLOP/s", "GCells/s", "Note"])
        for name in SCONF_STENCILS:
            s = capi.info(name)
            n = args.s2 if s["dim"] == 2 else args.s3
            for prec in ("float", "double"):
                dt = PREC[prec]
                top = max_degree(name, dt, args.mode)
                bt = min(4, top)
                sl = 512 if s["dim"] == 3 else 0
                cfg, _, meas = measure(name, dt, n, args.t, args.n, bt=bt, sl=sl, fp_mode=args.mode)
                note = "" if bt == 4 else f"bt clamped to {bt} (largest fused degree built)"
                w.writerow([name, prec, cfg["bS1"], cfg["bS2"], cfg["bT"], cfg["sl"], f"{meas:.4f}",
                            f"{meas / s['fpp']:.3f}", note])
                f.flush()
                print(f"{name:11s} {prec:6s} bT={cfg['bT']} sl={cfg['sl']} {meas:10.1f} GFLOP/s {note}", flush=True)
    return path


def max_degree(name, dtype, mode):
    """Largest bt gbs_plan accepts for this stencil, dtype and mode."""
    top = 1
    for bt in range(1, 17):
        d, _ = capi.make_desc(name, dtype, 64, 2 * bt, mode, bt=bt)
        if capi.lib().gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) != capi.GBS_OK:
            break
        top = bt
    return top


def copy_bandwidth(nbytes=2 << 30, reps=5):
    """Device-to-device copy bandwidth (bytes read + written per second) of
    the current GPU, the HBM roof of the sweep's Roofline(bt)."""
    import torch
    src = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda").fill_(1.0)
    dst = torch.empty_like(src)
    dst.copy_(src)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        dst.copy_(src)
    e1.record()
    e1.synchronize()
    bw = 2.0 * nbytes * reps / (e0.elapsed_time(e1) * 1e-3)
    del src, dst
    torch.cuda.empty_cache()
    return bw


def cmd_sweep(args):
    import torch
    from .grid import DeviceGrid
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    names = args.stencils.split(",") if args.stencils else ["star3d2r", "box3d1r"]
    hbm = copy_bandwidth()
    path = out / "sweep.csv"
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["Stencil", "Precision", "bT", "bS1", "bS2", "sl", "Redundancy", "Model GCells/s",
                    "Measured GCells/s", "Roofline(bt) GCells/s", "% of Roofline(bt)"])
        for name in names:
            s = capi.info(name)
            n = args.s2 if s["dim"] == 2 else args.s3
            cells = float(n) ** s["dim"] * args.t
            for prec in ("float", "double"):
                dt = PREC[prec]
                fp = capi.measure_fp_peak(dt) * 1e9
                g = DeviceGrid(name, dt, [n] * s["dim"])
                g.fill_uniform(1)
                for bt in range(1, min(args.bt_max, max_degree(name, dt, args.mode)) + 1):
                    d, _ = g.desc(args.t, args.mode, bt=bt)
                    p = capi.plan(d)
                    model_ms = ctypes.c_double(0.0)
                    capi.check(capi.lib().gbs_tune_model(ctypes.byref(d), ctypes.byref(model_ms)))
                    g.run(args.t, args.mode, bt=bt)  # warm-up
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    for _ in range(args.n):
                        g.run(args.t, args.mode, bt=bt)
                    e1.record()
                    e1.synchronize()
                    meas = cells * args.n / (e0.elapsed_time(e1) * 1e-3) / 1e9
                    model = cells / (model_ms.value * args.t * 1e-3) / 1e9
                    roof = min(hbm * bt / (2 * np.dtype(dt).itemsize), fp / s["fpp"]) / 1e9
                    w.writerow([name, prec, p.bt, p.bs1, p.bs2, p.sl, f"{p.redundancy:.3f}", f"{model:.1f}",
                                f"{meas:.1f}", f"{roof:.1f}", f"{100 * meas / roof:.1f}"])
                    f.flush()
                    print(f"{name:9s} {prec:6s} bT={p.bt} bS1={p.bs1} sl={p.sl} red {p.redundancy:.2f} "
                          f"measured {meas:8.1f} GCells/s ({100 * meas / roof:5.1f}% of Roofline(bt) "
                          f"{roof:.0f})", flush=True)
                del g
                torch.cuda.empty_cache()
    return path


def cmd_regcap(args):
    from . import build as gb
    out = Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    rows = []
    for cap in [int(c) for c in args.caps.split(",")]:
        lib = gb.build(regcap=cap)
        sub = out / f"regcap{cap}"
        env = dict(os.environ, GBS_LIB=str(lib))
        cmd = [sys.executable, "-m", "gbstencil.report", "run", "--prec", args.prec, "--out", str(sub),
               "-t", str(args.t), "-n", str(args.n), "--s2", str(args.s2), "--s3", str(args.s3),
               "--mode", args.mode] + (["--stencils", args.stencils] if args.stencils else [])
        subprocess.run(cmd, check=True, env=env, cwd=Path(__file__).resolve().parent.parent)
        with open(sub / f"{args.prec}_run.csv") as f:
            for r in list(csv.reader(f))[1:]:
                rows.append([cap] + r)
    path = out / f"{args.prec}_regcap.csv"
    with open(path, "w", newline="") as f:
        w = csv.writer(f)
        w.writerow(["RegCap", "Stencil", "bS1", "bS2", "bT", "sl", "Model", "Measured"])
        w.writerows(rows)
    return path


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("what", choices=["run", "sconf", "regcap", "sweep"])
    ap.add_argument("--prec", default="float", choices=list(PREC))
    ap.add_argument("--out", default="gb300")
    ap.add_argument("--stencils", default="")
    ap.add_argument("--mode", default="fma", choices=["fma", "exact"])
    ap.add_argument("-t", type=int, default=1000)
    ap.add_argument("-n", type=int, default=5)
    ap.add_argument("--s2", type=int, default=16384, help="2-D compute size (-s)")
    ap.add_argument("--s3", type=int, default=512, help="3-D compute size (-s)")
    ap.add_argument("--caps", default="0,32,64,96")
    ap.add_argument("--bt-max", type=int, default=8, help="sweep: largest fused degree")
    args = ap.parse_args(argv)
    path = {"run": cmd_run, "sconf": cmd_sconf, "regcap": cmd_regcap, "sweep": cmd_sweep}[args.what](args)
    print(path)


if __name__ == "__main__":
    main()
