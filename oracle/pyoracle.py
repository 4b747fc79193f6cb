"""ctypes view of the CPU oracle (``liboracle.so``) and of the reference's own
CPU path built under ``_ref/``.

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg, as the oracle. The engine never calls
it.
"""
from __future__ import annotations

import ctypes
import json
import os
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
TABLE = HERE.parent / "an5d-artifact_gb300" / "gbstencil" / "stencils.json"
_LIB = None
_REF = {}

STENCILS = json.loads(TABLE.read_text())["stencils"]
BY_NAME = {s["name"]: (i, s) for i, s in enumerate(STENCILS)}
TCODE = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.longdouble): 2}


def lib():
    global _LIB
    if _LIB is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            raise RuntimeError(f"{path} is missing: run `make -C oracle`")
        _LIB = ctypes.CDLL(str(path))
        _LIB.oracle_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_double, ctypes.c_double]
        _LIB.oracle_init_grid_f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _LIB.oracle_init_grid_d.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _LIB.oracle_set_threads.argtypes = [ctypes.c_int]
        _LIB.oracle_max_threads.restype = ctypes.c_int
    return _LIB


def set_threads(n: int):
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return lib().oracle_max_threads()


def reference_coefficients(name: str, dtype) -> np.ndarray:
    """The source literals converted to the element type (a float literal in
    a double expression is widened exactly, e.g. ``0.1873f``)."""
    _, s = BY_NAME[name]
    if s["kind"] == "gradient":
        return np.array([np.float32(s["numerator"])], dtype=dtype)
    if s.get("groups"):  # double literals (3d125pt)
        return np.array([t["value"] for t in s["terms"]], dtype=dtype)
    return np.array([np.float32(t["value"]) for t in s["terms"]], dtype=dtype)


def reference_divisor(name: str) -> float:
    _, s = BY_NAME[name]
    return float(s["divisor"] or 0)


def reference_eps(name: str) -> float:
    _, s = BY_NAME[name]
    return float(np.float32(s.get("eps", 0.0)))


def grid_shape(name: str, n):
    _, s = BY_NAME[name]
    dim, r = s["dim"], s["rad"]
    if np.isscalar(n):
        n = [int(n)] * dim
    return (2,) + tuple(int(x) + 2 * r for x in n), list(n)


def init_grid(name: str, compsize: int, dtype) -> np.ndarray:
    """Both planes as common.h's init_grid sets them (cubic grid)."""
    shape, _ = grid_shape(name, compsize)
    _, s = BY_NAME[name]
    A = np.empty(shape, dtype=dtype)
    fn = lib().oracle_init_grid_f if A.dtype == np.float32 else lib().oracle_init_grid_d
    fn(A.ctypes.data, int(compsize), s["dim"], s["rad"])
    return A


def run(name: str, A: np.ndarray, n, timestep: int, coef=None, divisor=None, eps=None):
    """Advance ``A`` (shape (2, d0, d1[, d2]), C order) in place by
    ``timestep`` steps; the result is in plane ``timestep % 2``."""
    sid, s = BY_NAME[name]
    assert A.flags.c_contiguous
    if np.isscalar(n):
        n = [int(n)] * s["dim"]
    nn = (ctypes.c_int * 3)(*(list(n) + [0] * (3 - len(n))))
    coef_ptr = None
    if coef is None and s.get("groups"):
        coef_ptr = 0  # the grouped form's double literals, as the source writes them
    elif coef is None:
        coef = reference_coefficients(name, A.dtype)
    if coef_ptr is None:
        coef = np.ascontiguousarray(coef, dtype=A.dtype)
        coef_ptr = coef.ctypes.data
    if divisor is None:
        divisor = reference_divisor(name)
    if eps is None:
        eps = reference_eps(name)
    lib().oracle_run(sid, TCODE[A.dtype], A.ctypes.data, nn, int(timestep),
                     coef_ptr or None, float(divisor), float(eps))
    return A


def timed_run(name, A, n, timestep, **kw) -> float:
    t0 = time.perf_counter()
    run(name, A, n, timestep, **kw)
    return (time.perf_counter() - t0) * 1e3


# --------------------------------------------------------------------------
# The reference's own CPU path (built from its sources by `make ref`).
# --------------------------------------------------------------------------
def ref_available() -> bool:
    return (HERE / "_ref" / "star2d1r_float.so").exists()


def ref_lib(name: str, dtype):
    key = (name, np.dtype(dtype))
    if key not in _REF:
        tname = "float" if np.dtype(dtype) == np.float32 else "double"
        path = HERE / "_ref" / f"{name}_{tname}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        L = ctypes.CDLL(str(path))
        L.kernel_stencil.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_bool]
        L.kernel_stencil.restype = ctypes.c_double
        L.init_grid.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _REF[key] = L
    return _REF[key]


def ref_init_grid(name: str, compsize: int, dtype) -> np.ndarray:
    shape, _ = grid_shape(name, compsize)
    A = np.empty(shape, dtype=dtype)
    ref_lib(name, dtype).init_grid(A.ctypes.data, int(compsize))
    return A


def ref_run(name: str, A: np.ndarray, compsize: int, timestep: int, scop=False) -> float:
    """kernel_stencil(A, compsize, timestep, scop) of the reference itself."""
    return ref_lib(name, A.dtype).kernel_stencil(A.ctypes.data, int(compsize), int(timestep), bool(scop))


def check_result(A: np.ndarray, B: np.ndarray, timestep: int):
    """(max |A-B|, rms) over plane timestep%2, as check_result
    (common.h:58-79) reports them."""
    t = timestep % 2
    e = np.abs(A[t].astype(np.float64) - B[t].astype(np.float64))
    return float(e.max()), float(np.sqrt(np.mean(e.astype(np.longdouble) ** 2)))


def normwise_error(A: np.ndarray, B: np.ndarray, timestep: int) -> float:
    """max |A-B| / max |B| over plane timestep%2 (the parity metric)."""
    t = timestep % 2
    a = A[t].astype(np.float64)
    b = B[t].astype(np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))
