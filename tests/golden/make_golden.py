"""Generates tests/golden/reference_outputs.json from the AN5D artifact itself.

For every in-scope stencil and element type it builds the grid with the
artifact's own ``init_grid`` (common.h:44-56) and advances it with the
artifact's own ``kernel_stencil(A, compsize, T, scop=false)`` (its OpenMP CPU
branch, e.g. star2d1r.c:26-37), both taken from the shared libraries that
``make -C oracle ref`` builds from the unmodified sources. It records a
SHA-256 of the result plane (plane T%2, every cell, halo included, raw bytes)
and a few sampled cells.

Run here, where the artifact's sources exist:

    make -C oracle ref && python tests/golden/make_golden.py

The fixtures then pin the CPU oracle and the engine's exact mode bit for bit
on any machine, without the artifact present.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT / "oracle"))
import pyoracle as po  # noqa: E402

# sizes small enough for the pure-CPU checks, odd so that no tile divides them
CASES_2D = [(23, 1), (23, 2), (23, 7), (70, 5)]
CASES_3D = [(11, 1), (11, 2), (11, 5), (20, 3)]


def digest(A: np.ndarray, T: int) -> str:
    return hashlib.sha256(np.ascontiguousarray(A[T % 2]).tobytes()).hexdigest()


def samples(A: np.ndarray, T: int):
    P = A[T % 2].reshape(-1)
    idx = np.linspace(0, P.size - 1, 7).astype(np.int64)
    return [[int(i), float(P[i])] for i in idx]


def main():
    if not po.ref_available():
        raise SystemExit("oracle/_ref is missing: run `make -C oracle ref` first")
    out = []
    for s in po.STENCILS:
        name = s["name"]
        cases = CASES_2D if s["dim"] == 2 else CASES_3D
        for dt, tname in ((np.float32, "float"), (np.float64, "double")):
            for n, T in cases:
                A = po.ref_init_grid(name, n, dt)
                po.ref_run(name, A, n, T, scop=False)
                out.append({"stencil": name, "dtype": tname, "compsize": n, "timestep": T,
                            "sha256": digest(A, T), "samples": samples(A, T)})
    path = Path(__file__).with_name("reference_outputs.json")
    path.write_text(json.dumps({"generator": "tests/golden/make_golden.py",
                                "source": "AN5D artifact init_grid + kernel_stencil(scop=false)",
                                "cases": out}, indent=0) + "\n")
    print(f"wrote {len(out)} cases to {path}")


if __name__ == "__main__":
    main()
