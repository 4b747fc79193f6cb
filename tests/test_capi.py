"""The C-ABI library: exports, catalogue, layout, planning and error
behaviour. None of these calls touches a GPU."""
import ctypes
import json
import re
from pathlib import Path

import numpy as np
import pytest

from gbstencil import capi

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(gbs_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    decl = declared_functions()
    assert "gbs_run" in decl and "gbs_run_device" in decl
    missing = [n for n in decl if not hasattr(L, n)]
    assert not missing, missing


def test_binding_covers_declarations():
    bound = {s[0] for s in capi.SIGNATURES}
    assert set(declared_functions()) <= bound | {"gbs_batch_plan_size"}, set(declared_functions()) - bound


def test_catalogue_matches_table():
    L = capi.lib()
    table = json.loads((ROOT / "an5d-artifact_gb300" / "gbstencil" / "stencils.json").read_text())["stencils"]
    assert L.gbs_num_stencils() == len(table) == 22
    for i, s in enumerate(table):
        assert L.gbs_stencil_name(i).decode() == s["name"]
        assert L.gbs_stencil_id(s["name"].encode()) == i
        dim, rad, nt, fpp = (ctypes.c_int() for _ in range(4))
        capi.check(L.gbs_stencil_info(i, ctypes.byref(dim), ctypes.byref(rad), ctypes.byref(nt), ctypes.byref(fpp)))
        assert (dim.value, rad.value, fpp.value) == (s["dim"], s["rad"], s["fpp"])
    assert L.gbs_stencil_id(b"3d125pt") == 21
    assert L.gbs_stencil_id(b"3d999pt") == -1


@pytest.mark.parametrize("name,dt,n", [("star2d1r", np.float32, 4096), ("star2d4r", np.float64, 77),
                                       ("star3d2r", np.float32, 512), ("box3d1r", np.float64, 33)])
def test_layout_invariants(name, dt, n):
    d, _ = capi.make_desc(name, dt, n, 10)
    L = capi.layout(d)
    s = capi.info(name)
    es = np.dtype(dt).itemsize
    V = 16 // es
    assert L.dimsize[0] == n + 2 * s["rad"]
    assert (L.pitch * es) % 128 == 0
    assert (L.shift + s["rad"]) % V == 0, "first interior column 16-byte aligned"
    assert L.pitch >= L.shift + L.dimsize[s["dim"] - 1] + 32 * V
    assert L.bytes == 2 * L.plane * es
    assert L.rows * L.pitch == L.plane


@pytest.mark.parametrize("T", [0, 1, 2, 3, 7, 8, 9, 100, 101])
@pytest.mark.parametrize("bt", [1, 2, 4, 8])
def test_plan_final_plane_parity(T, bt):
    """Launch j reads plane j%2; the result must land in plane T%2, so the
    number of launches must have the parity of T."""
    d, _ = capi.make_desc("star2d1r", np.float32, 64, T, fp_mode="fma", bt=bt)
    p = capi.plan(d)
    assert p.launches % 2 == T % 2
    assert p.launches >= -(-T // bt)
    assert p.launches <= -(-T // bt) + 1


def test_invalid_descriptors_return_status():
    L = capi.lib()
    d, _ = capi.make_desc("star2d1r", np.float32, 64, 10)
    d.stencil = 99
    assert L.gbs_get_layout(ctypes.byref(d), ctypes.byref(capi.Layout())) == capi.GBS_ERR_INVALID
    assert "unknown stencil" in L.gbs_last_error().decode()
    d, _ = capi.make_desc("star2d1r", np.float32, 64, 10)
    d.n[0] = 0
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_ERR_INVALID
    d, _ = capi.make_desc("star2d1r", np.float32, 64, -1)
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_ERR_INVALID
    d, _ = capi.make_desc("star2d1r", np.float32, 64, 10, fp_mode=7)
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_ERR_INVALID
    d, _ = capi.make_desc("box2d4r", np.float32, 64, 10, bt=8)
    assert L.gbs_plan(ctypes.byref(d), ctypes.byref(capi.PlanInfo())) == capi.GBS_ERR_UNSUPPORTED
    assert L.gbs_run(None, None, None) == capi.GBS_ERR_INVALID


def test_python_mirror_rejects_cpu_branch():
    A = np.zeros((2, 10, 10), np.float32)
    with pytest.raises(NotImplementedError):
        capi.kernel_stencil(A, 8, 1, False, stencil="star2d1r")
