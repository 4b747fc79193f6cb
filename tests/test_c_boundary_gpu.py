"""The C boundary exercised from C: tests/c/capi_from_c.c includes
include/gbstencil.h, links libgbstencil.so and calls gbs_run (the
kernel_stencil drop-in, common.h:42) and the device-buffer path directly,
with no Python between the caller and the engine. The CPU oracle supplies
the expected grid through a file."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import pyoracle as po

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
LIB = ROOT / "an5d-artifact_gb300" / "gbstencil" / "_lib"
CUDA = Path("/usr/local/cuda")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    if not shutil.which("gcc"):
        pytest.skip("needs gcc")
    out = tmp_path_factory.mktemp("cabi") / "capi_from_c"
    r = subprocess.run(["gcc", "-O2", "-std=c11", f"-I{ROOT / 'include'}", f"-I{CUDA / 'include'}",
                        str(ROOT / "tests" / "c" / "capi_from_c.c"), f"-L{LIB}", "-lgbstencil",
                        f"-L{CUDA / 'lib64'}", "-lcudart", f"-Wl,-rpath,{LIB}", f"-Wl,-rpath,{CUDA / 'lib64'}",
                        "-lm", "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.parametrize("name,dt,n,T,mode,bt", [
    ("star2d1r", "float", 257, 13, "exact", 4),
    ("star2d1r", "float", 1000, 20, "fma", 0),
    ("j2d5pt", "double", 130, 7, "exact", 2),
    ("gradient2d", "float", 96, 9, "fma", 2),
    ("box3d1r", "double", 40, 5, "fma", 1),
    ("j3d27pt", "float", 37, 6, "exact", 2),
])
def test_c_caller(exe, tmp_path, name, dt, n, T, mode, bt):
    dtype = np.float32 if dt == "float" else np.float64
    A = po.init_grid(name, n, dtype)
    want = A.copy()
    po.run(name, want, n, T)
    A.tofile(tmp_path / "in.bin")
    want.tofile(tmp_path / "want.bin")
    r = subprocess.run([str(exe), name, dt, str(n), str(T), mode, str(bt), str(tmp_path / "in.bin"),
                        str(tmp_path / "want.bin")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(": ok") == 3, r.stdout
