"""Autotuner front end (gbs_tune and the engine's tuning table).

    from gbstencil import tune
    best, cands = tune.tune("box3d1r", np.float32, 512, "fma")   # times on the GPU
    tune.save("my_table.txt")

The engine resolves bt = 0 / sl = 0 through its table; ``capi.lib()`` loads
the table shipped with the package (``tuning_gb300.txt``, measured on GB300)
when the library is first loaded. Regenerate that table with
``python -m gbstencil.tune --out gbstencil/tuning_gb300.txt`` on the GPU.
"""
from __future__ import annotations

import argparse
import ctypes
from pathlib import Path

import numpy as np

from . import capi

DEFAULT_TABLE = Path(__file__).resolve().parent / "tuning_gb300.txt"


class Candidate(ctypes.Structure):
    _fields_ = [("bt", ctypes.c_int), ("sl", ctypes.c_int), ("redundancy", ctypes.c_double),
                ("model_ms_per_step", ctypes.c_double), ("ms_per_step", ctypes.c_double), ("bs1", ctypes.c_int)]


def tune(name: str, dtype, n, fp_mode="fma", max_cands: int = 64):
    """Times the candidates for one (stencil, dtype, size, mode); returns
    (best, all candidates fastest first) as dicts. Records the best."""
    d, _ = capi.make_desc(name, dtype, n, 0, fp_mode)
    buf = (Candidate * max_cands)()
    nc = ctypes.c_int(0)
    capi.check(capi.lib().gbs_tune(ctypes.byref(d), ctypes.cast(buf, ctypes.c_void_p), max_cands, ctypes.byref(nc)))
    out = [{"bt": c.bt, "sl": c.sl, "bs1": c.bs1, "redundancy": c.redundancy,
            "model_ms_per_step": c.model_ms_per_step, "ms_per_step": c.ms_per_step}
           for c in buf[:min(nc.value, max_cands)]]
    return out[0], out


def lookup(name: str, dtype, n, fp_mode="fma"):
    """(bt, sl) the table gives for this size; bt 0 when it has no entry."""
    d, _ = capi.make_desc(name, dtype, n, 0, fp_mode)
    bt, sl = ctypes.c_int(0), ctypes.c_int(0)
    capi.check(capi.lib().gbs_tune_lookup(ctypes.byref(d), ctypes.byref(bt), ctypes.byref(sl)))
    return bt.value, sl.value


def record(name: str, dtype, n, bt: int, sl: int = 0, fp_mode="fma", ms_per_step: float = 0.0):
    d, _ = capi.make_desc(name, dtype, n, 0, fp_mode)
    capi.check(capi.lib().gbs_tune_set(ctypes.byref(d), int(bt), int(sl), float(ms_per_step)))


def load(path):
    capi.check(capi.lib().gbs_tune_load(str(path).encode()))


def save(path):
    capi.check(capi.lib().gbs_tune_save(str(path).encode()))


def clear():
    capi.lib().gbs_tune_clear()


def entries() -> int:
    return capi.lib().gbs_tune_entries()


# Sizes the shipped table covers: every stencil at the artifact's benchmark
# sizes (compiled/run.sh: 2-D 16384^2, 3-D 512^3) and at the sizes of the
# single-grid workloads (2-D 4096^2 and 2048^2, 3-D 384^3 and 256^3).
TABLE_SIZES = {2: [4096, 16384, 2048, 1024], 3: [512, 384, 256]}


def main():
    ap = argparse.ArgumentParser(description="tune every stencil and write a table")
    ap.add_argument("--out", default=str(DEFAULT_TABLE))
    ap.add_argument("--stencils", default="", help="comma-separated subset")
    ap.add_argument("--dtypes", default="float32,float64")
    ap.add_argument("--modes", default="fma,exact")
    ap.add_argument("--sizes", default="", help="comma-separated interior sides (default: the table's sizes)")
    ap.add_argument("--log", default="", help="also write every candidate's timing (JSON lines)")
    ap.add_argument("--fresh", action="store_true",
                    help="start from an empty table (default: re-tune into the shipped one)")
    args = ap.parse_args()
    import json
    names = args.stencils.split(",") if args.stencils else capi.NAMES
    capi.lib()
    if args.fresh:
        clear()
    log = open(args.log, "w") if args.log else None
    for name in names:
        s = capi.info(name)
        for dt in args.dtypes.split(","):
            for mode in args.modes.split(","):
                sizes = [int(x) for x in args.sizes.split(",")] if args.sizes else TABLE_SIZES[s["dim"]]
                for n in sizes:
                    best, cands = tune(name, np.dtype(dt), n, mode)
                    print(f"{name:11s} {dt:8s} {mode:5s} n={n:6d} bt={best['bt']} sl={best['sl']} "
                          f"bs1={best['bs1']} {best['ms_per_step']:.4f} ms/step ({len(cands)} candidates)",
                          flush=True)
                    if log:
                        log.write(json.dumps({"stencil": name, "dtype": dt, "mode": mode, "n": n,
                                              "candidates": cands}) + "\n")
                        log.flush()
    save(args.out)


if __name__ == "__main__":
    main()
