"""The C drop-in: a benchmark's kernel_stencil calling gbs_run, with the
artifact's harness (-s/-t/-n/-c) and OpenMP branch unchanged. Generated from
the artifact's sources where they are present and compiled and linked
against libgbstencil.so (running it needs a GPU)."""
import importlib.util
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _artifact_dir() -> Path:
    """The artifact's sources: AN5D_ARTIFACT_DIR, else the directory the
    oracle's pin was last built from (oracle/_ref/artifact_dir)."""
    import os
    if os.environ.get("AN5D_ARTIFACT_DIR"):
        return Path(os.environ["AN5D_ARTIFACT_DIR"])
    rec = ROOT / "oracle" / "_ref" / "artifact_dir"
    return Path(rec.read_text().strip()) if rec.exists() else ROOT / "missing-artifact"


ARTIFACT = _artifact_dir()
LIB = ROOT / "an5d-artifact_gb300" / "gbstencil" / "_lib"


def _gen():
    spec = importlib.util.spec_from_file_location("make_shims", ROOT / "an5d-artifact_gb300" / "shim" / "make_shims.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_shim_rewrites_only_the_scop_branch():
    m = _gen()
    src = ('#define BENCH_DIM 2\n#include "common.h"\n\ndouble kernel_stencil(SB_TYPE *A1, int compsize, '
           'int timestep, bool scop)\n{\n  double start_time = sb_time(), end_time = 0.0;\n'
           '  if (scop) {\n#pragma scop\n    for (;;) x = 1;\n#pragma endscop\n  }\n  else {\n    cpu();\n  }\n'
           '  return 0;\n}\n')
    out = m.shim("star2d1r", src)
    assert '#include "gbstencil.h"' in out and "gbs_run(&gd, A1, &gbs_ms)" in out
    assert "#pragma scop" not in out and "cpu();" in out and 'gbs_stencil_id("star2d1r")' in out
    assert "GBS_FP_EXACT" in out
    assert "GBS_FP_FMA" in m.shim("3d125pt", src.replace("star2d1r", "3d125pt"))
    with pytest.raises(ValueError):
        m.shim("x", "int main(void) { return 0; }\n")


@pytest.mark.skipif(not (ARTIFACT / "common.h").exists() or not shutil.which("gcc"),
                    reason="needs the artifact's sources and gcc")
@pytest.mark.parametrize("name,prec", [("star2d1r", "float"), ("j3d27pt", "double"), ("gradient2d", "float"),
                                       ("3d125pt", "float")])
def test_shim_compiles_and_links(tmp_path, name, prec):
    m = _gen()
    m.main([str(ARTIFACT), str(tmp_path), name])
    if not (LIB / "libgbstencil.so").exists():
        pytest.skip("engine not built")
    exe = tmp_path / f"{name}_{prec}"
    r = subprocess.run(["gcc", "-O2", "-fopenmp", f"-DSB_TYPE={prec}", f"-I{ARTIFACT}", f"-I{ROOT / 'include'}",
                        str(tmp_path / f"{name}_gbs.c"), f"-L{LIB}", "-lgbstencil", f"-Wl,-rpath,{LIB}", "-lm",
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert exe.exists()
