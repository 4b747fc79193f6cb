"""ctypes binding of the C ABI declared in include/gbstencil.h.

This is the Python mirror of the artifact's drop-in boundary: the same
``kernel_stencil(A1, compsize, timestep, scop)`` call (common.h:42), backed by
``gbs_run`` of ``libgbstencil.so``. Loading fails loudly when the library is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import json
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
# GBS_LIB selects another build of the engine (e.g. a register-capped variant)
LIB_PATH = Path(os.environ["GBS_LIB"]) if os.environ.get("GBS_LIB") else PKG / "_lib" / "libgbstencil.so"
TABLE = json.loads((PKG / "stencils.json").read_text())["stencils"]
NAMES = [s["name"] for s in TABLE]

GBS_OK, GBS_ERR_INVALID, GBS_ERR_UNSUPPORTED, GBS_ERR_CUDA, GBS_ERR_NOMEM, GBS_ERR_TIMEOUT, GBS_ERR_NODEVICE = range(7)
STATUS_NAMES = {0: "GBS_OK", 1: "GBS_ERR_INVALID", 2: "GBS_ERR_UNSUPPORTED", 3: "GBS_ERR_CUDA",
                4: "GBS_ERR_NOMEM", 5: "GBS_ERR_TIMEOUT", 6: "GBS_ERR_NODEVICE"}
GBS_F32, GBS_F64 = 0, 1
GBS_FP_EXACT, GBS_FP_FMA = 0, 1
FP_MODES = {"exact": GBS_FP_EXACT, "fma": GBS_FP_FMA}


class GbsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Desc(ctypes.Structure):
    _fields_ = [("stencil", ctypes.c_int), ("dtype", ctypes.c_int), ("n", ctypes.c_int * 3),
                ("timestep", ctypes.c_int), ("fp_mode", ctypes.c_int), ("bt", ctypes.c_int),
                ("bs1", ctypes.c_int), ("bs2", ctypes.c_int), ("sl", ctypes.c_int),
                ("coef", ctypes.c_void_p), ("divisor", ctypes.c_double), ("eps", ctypes.c_double)]


class Layout(ctypes.Structure):
    _fields_ = [("pitch", ctypes.c_size_t), ("shift", ctypes.c_size_t), ("rows", ctypes.c_size_t),
                ("plane", ctypes.c_size_t), ("bytes", ctypes.c_size_t), ("dimsize", ctypes.c_int * 3),
                ("dim", ctypes.c_int), ("rad", ctypes.c_int)]


class PlanInfo(ctypes.Structure):
    _fields_ = [("bt", ctypes.c_int), ("bs1", ctypes.c_int), ("bs2", ctypes.c_int), ("sl", ctypes.c_int),
                ("launches", ctypes.c_int), ("ctas", ctypes.c_int), ("valid_w", ctypes.c_int),
                ("redundancy", ctypes.c_double)]


class BatchGrid(ctypes.Structure):
    _fields_ = [("stencil", ctypes.c_int), ("n", ctypes.c_int * 3), ("timestep", ctypes.c_int),
                ("dev_A", ctypes.c_void_p), ("coef", ctypes.c_void_p), ("divisor", ctypes.c_double)]


class BatchStats(ctypes.Structure):
    _fields_ = [("grids", ctypes.c_int), ("items", ctypes.c_int), ("ctas", ctypes.c_int),
                ("plain_launches", ctypes.c_int), ("cell_updates", ctypes.c_longlong),
                ("kernels", ctypes.c_int), ("mode", ctypes.c_int), ("hbm_bytes", ctypes.c_longlong)]


_lib = None

# every entry point the header declares: (name, restype, argtypes)
SIGNATURES = [
    ("gbs_num_stencils", ctypes.c_int, []),
    ("gbs_stencil_name", ctypes.c_char_p, [ctypes.c_int]),
    ("gbs_stencil_id", ctypes.c_int, [ctypes.c_char_p]),
    ("gbs_stencil_info", ctypes.c_int, [ctypes.c_int] + [ctypes.POINTER(ctypes.c_int)] * 4),
    ("gbs_run", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]),
    ("gbs_run_device", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_void_p]),
    ("gbs_get_layout", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.POINTER(Layout)]),
    ("gbs_plan", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.POINTER(PlanInfo)]),
    ("gbs_upload", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gbs_download", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gbs_sync", ctypes.c_int, [ctypes.c_void_p]),
    ("gbs_batch_plan", ctypes.c_int, [ctypes.POINTER(BatchGrid), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    ("gbs_batch_run", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("gbs_batch_info", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BatchStats)]),
    ("gbs_batch_destroy", None, [ctypes.c_void_p]),
    ("gbs_batch_run_noalloc", ctypes.c_int, [ctypes.POINTER(BatchGrid), ctypes.c_int, ctypes.c_int,
                                             ctypes.c_void_p]),
    ("gbs_adjoint_workspace", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_int, ctypes.POINTER(ctypes.c_size_t)]),
    ("gbs_adjoint_forward", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p]),
    ("gbs_adjoint_backward", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    ("gbs_adjoint_workspace_slots", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_int, ctypes.c_int,
                                                   ctypes.POINTER(ctypes.c_size_t)]),
    ("gbs_adjoint_backward_slots", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    ("gbs_adjoint_plan_budget", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_size_t, ctypes.POINTER(ctypes.c_int),
                                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_size_t)]),
    ("gbs_revolve_cost", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong),
                                        ctypes.POINTER(ctypes.c_int)]),
    ("gbs_adjoint_forward_batch", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                                 ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]),
    ("gbs_adjoint_backward_batch", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                                  ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                                  ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]),
    ("gbs_measure_fp_peak", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("gbs_tune", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    ("gbs_tune_set", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.c_int, ctypes.c_int, ctypes.c_double]),
    ("gbs_tune_model", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.POINTER(ctypes.c_double)]),
    ("gbs_tune_lookup", ctypes.c_int, [ctypes.POINTER(Desc), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    ("gbs_tune_load", ctypes.c_int, [ctypes.c_char_p]),
    ("gbs_tune_save", ctypes.c_int, [ctypes.c_char_p]),
    ("gbs_tune_entries", ctypes.c_int, []),
    ("gbs_tune_clear", None, []),
    ("gbs_check_division", ctypes.c_int, [ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_longlong,
                                          ctypes.POINTER(ctypes.c_longlong)]),
    ("gbs_last_error", ctypes.c_char_p, []),
    ("gbs_release_cache", None, []),
]


def lib():
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: the CUDA engine is not built "
                               "(run __graft_entry__.build() or python -m gbstencil.build)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        # the tuning table measured on GB300 that ships with the package
        table = Path(__file__).resolve().parent / "tuning_gb300.txt"
        if table.exists():
            check_with(L, L.gbs_tune_load(str(table).encode()))
        _lib = L
    return _lib


def check_with(L, status: int):
    if status != GBS_OK:
        raise GbsError(status, L.gbs_last_error().decode())


def check(status: int):
    if status != GBS_OK:
        raise GbsError(status, lib().gbs_last_error().decode())


def stencil_id(name: str) -> int:
    if name not in NAMES:
        raise ValueError(f"unknown stencil {name!r}")
    return NAMES.index(name)


def info(name: str) -> dict:
    return TABLE[stencil_id(name)]


def make_desc(name: str, dtype, n, timestep: int, fp_mode="exact", bt=0, sl=0, bs1=0,
              coef=None, divisor=0.0, eps=0.0):
    """Builds a gbs_desc. ``coef`` (if given) must stay alive while the
    descriptor is used; the returned tuple keeps a reference."""
    s = info(name)
    dt = np.dtype(dtype)
    if dt not in (np.float32, np.float64):
        raise ValueError("dtype must be float32 or float64")
    if np.isscalar(n):
        n = [int(n)] * s["dim"]
    n = list(n) + [1] * (3 - len(n))
    d = Desc()
    d.stencil = stencil_id(name)
    d.dtype = GBS_F32 if dt == np.float32 else GBS_F64
    for a in range(3):
        d.n[a] = int(n[a])
    d.timestep = int(timestep)
    d.fp_mode = FP_MODES[fp_mode] if isinstance(fp_mode, str) else int(fp_mode)
    d.bt, d.sl, d.bs1 = int(bt), int(sl), int(bs1)
    keep = None
    if coef is not None:
        keep = np.ascontiguousarray(coef, dtype=dt)
        d.coef = keep.ctypes.data
    d.divisor = float(divisor)
    d.eps = float(eps)
    return d, keep


def layout(desc: Desc) -> Layout:
    out = Layout()
    check(lib().gbs_get_layout(ctypes.byref(desc), ctypes.byref(out)))
    return out


def plan(desc: Desc) -> PlanInfo:
    out = PlanInfo()
    check(lib().gbs_plan(ctypes.byref(desc), ctypes.byref(out)))
    return out


def run_host(desc: Desc, A: np.ndarray) -> float:
    """gbs_run on a dense host grid (both planes); returns the device ms."""
    if not A.flags.c_contiguous:
        raise ValueError("A must be C-contiguous")
    ms = ctypes.c_double(0.0)
    check(lib().gbs_run(ctypes.byref(desc), A.ctypes.data, ctypes.byref(ms)))
    return ms.value


def run_device(desc: Desc, dev_ptr: int, stream: int = 0):
    check(lib().gbs_run_device(ctypes.byref(desc), ctypes.c_void_p(dev_ptr), ctypes.c_void_p(stream)))


def upload(desc: Desc, host_ptr: int, dev_ptr: int, stream: int = 0):
    check(lib().gbs_upload(ctypes.byref(desc), ctypes.c_void_p(host_ptr), ctypes.c_void_p(dev_ptr),
                           ctypes.c_void_p(stream)))


def download(desc: Desc, dev_ptr: int, host_ptr: int, stream: int = 0):
    check(lib().gbs_download(ctypes.byref(desc), ctypes.c_void_p(dev_ptr), ctypes.c_void_p(host_ptr),
                             ctypes.c_void_p(stream)))


def sync(stream: int = 0):
    check(lib().gbs_sync(ctypes.c_void_p(stream)))


class Batch:
    """A planned batched launch (gbs_batch_plan) over device grids."""

    MODES = {"persistent": 0, "layered": 1, "streams": 2}

    def __init__(self, grids, fp_mode="fma", mode="persistent"):
        """grids: list of (DeviceGrid-like with .name, .n, .dtype, .buf, timestep, coef or None),
        all of one dtype."""
        dts = {np.dtype(getattr(g, "dtype", np.float32)) for g, _, _ in grids}
        if len(dts) != 1:
            raise ValueError("a batch holds grids of one dtype")
        dt = dts.pop()
        self._keep = []
        arr = _batch_grids(grids, dt, self._keep)
        h = ctypes.c_void_p()
        check(lib().gbs_batch_plan(arr, len(grids), GBS_F32 if dt == np.float32 else GBS_F64,
                                   FP_MODES[fp_mode], self.MODES[mode], ctypes.byref(h)))
        self.handle = h

    def run(self, stream: int = 0):
        check(lib().gbs_batch_run(self.handle, ctypes.c_void_p(stream)))

    def stats(self) -> BatchStats:
        st = BatchStats()
        check(lib().gbs_batch_info(self.handle, ctypes.byref(st)))
        return st

    def close(self):
        if self.handle:
            lib().gbs_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _batch_grids(grids, dtype, keep):
    """gbs_batch_grid entries for (grid, timestep, coef or None) tuples;
    coefficient arrays are appended to ``keep``."""
    arr = (BatchGrid * len(grids))()
    for i, (g, T, coef) in enumerate(grids):
        arr[i].stencil = stencil_id(g.name)
        for a in range(3):
            arr[i].n[a] = int(g.n[a]) if a < len(g.n) else 1
        arr[i].timestep = int(T)
        arr[i].dev_A = g.buf.data_ptr()
        if coef is not None:
            c = np.ascontiguousarray(coef, dtype=dtype)
            keep.append(c)
            arr[i].coef = c.ctypes.data
        arr[i].divisor = 0.0
    return arr


def batch_run_noalloc(grids, fp_mode="fma", stream: int = 0):
    """gbs_batch_run_noalloc over (DeviceGrid, timestep, coef or None)
    entries: the batched run that allocates no memory itself."""
    keep = []
    arr = _batch_grids(grids, np.float32, keep)
    check(lib().gbs_batch_run_noalloc(arr, len(grids), FP_MODES[fp_mode], ctypes.c_void_p(stream)))


def measure_fp_peak(dtype) -> float:
    """Measured FMA throughput of the current device, GFLOP/s."""
    g = ctypes.c_double(0.0)
    dt = GBS_F32 if np.dtype(dtype) == np.float32 else GBS_F64
    check(lib().gbs_measure_fp_peak(dt, ctypes.byref(g)))
    return g.value


def check_division(dtype, divisor: float, samples: int = 0, checked: bool = True) -> int:
    """Inputs on which the engine's constant-divisor division differs from
    IEEE division (see gbs_check_division)."""
    m = ctypes.c_longlong(-1)
    dt = GBS_F32 if np.dtype(dtype) == np.float32 else GBS_F64
    check(lib().gbs_check_division(dt, float(divisor), int(bool(checked)), int(samples), ctypes.byref(m)))
    return m.value


def kernel_stencil(A1: np.ndarray, compsize: int, timestep: int, scop: bool = True, *,
                   stencil: str, fp_mode="exact", bt=0, sl=0, coef=None) -> float:
    """Mirror of the artifact's ``double kernel_stencil(SB_TYPE *A1, int
    compsize, int timestep, bool scop)`` (common.h:42) for ``scop == True``:
    advances the two-plane grid ``A1`` in place and returns the device time of
    the time loop in ms. ``scop == False`` selects the artifact's OpenMP CPU
    comparison path, which belongs to the caller's harness, not to this
    engine."""
    if not scop:
        raise NotImplementedError("scop=False is the harness's CPU comparison path; "
                                  "the engine implements the scop (device) branch only")
    d, keep = make_desc(stencil, A1.dtype, compsize, timestep, fp_mode, bt, sl, coef=coef)
    return run_host(d, A1)
