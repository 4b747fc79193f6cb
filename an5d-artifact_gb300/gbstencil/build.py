"""Builds ``libgbstencil.so`` (the engine and its kernel family) for sm_103a.

The kernel family is instantiated per (stencil, element type, fp mode) in
separate translation units (``csrc/inst.cu`` compiled with different -D
values) so that nvcc runs them in parallel. Objects are cached under
``_build/`` keyed by a hash of the flags and every source they include, so a
rebuild only recompiles what changed. No cmake: plain nvcc.

    python -m gbstencil.build               # from an5d-artifact_gb300/
    python -m gbstencil.build --regcap=64   # register-capped variant
"""
from __future__ import annotations

import hashlib
import json
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent                      # an5d-artifact_gb300/
CSRC = ROOT / "csrc"
BUILD = ROOT / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libgbstencil.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Wno-deprecated-gpu-targets"] + ARCH


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def stencils():
    return json.loads((PKG / "stencils.json").read_text())["stencils"]


def units():
    """(object name, source, extra flags) for every translation unit."""
    out = []
    for sid, s in enumerate(stencils()):
        for t, T in (("f", "float"), ("d", "double")):
            for m, fma in (("e", 0), ("m", 1)):
                name = f"picks_{sid}_{t}_{m}"
                out.append((name, CSRC / "inst.cu",
                            [f"-DGBS_SID={sid}", f"-DGBS_T={T}", f"-DGBS_FMA={fma}",
                             f"-DGBS_PICK=picks_{sid}_{t}_{m}"]))
    for m in (0, 1):  # the batched kernel, exact and FMA mode
        out.append((f"batch_{m}", CSRC / "batch.cu", [f"-DGBS_FMA={m}"]))
    for src in sorted(CSRC.glob("*.cu")):
        if src.name not in ("inst.cu", "batch.cu"):
            out.append((src.stem, src, []))
    return out


def source_hash(src: Path, flags) -> str:
    h = hashlib.sha1()
    h.update(" ".join(NVCC_FLAGS + flags).encode())
    h.update(src.read_bytes())
    for hdr in sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) +
                      list((ROOT.parent / "include").glob("*.h"))):
        h.update(hdr.name.encode())
        h.update(hdr.read_bytes())
    return h.hexdigest()


def compile_unit(unit, verbose=False, build_dir=BUILD):
    name, src, flags = unit
    obj = build_dir / f"{name}.o"
    stamp = build_dir / f"{name}.hash"
    key = source_hash(src, flags)
    if obj.exists() and stamp.exists() and stamp.read_text() == key:
        return name, False, ""
    cmd = [nvcc()] + NVCC_FLAGS + flags + ["-I", str(CSRC), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    stamp.write_text(key)
    return name, True, r.stderr if verbose else ""


def lib_path(regcap: int = 0) -> Path:
    """The library of a build; regcap > 0: the register-capped variant."""
    return LIB if regcap <= 0 else LIBDIR / f"regcap{regcap}" / "libgbstencil.so"


def build(jobs: int | None = None, verbose: bool = False, regcap: int = 0) -> Path:
    """Compiles and links the engine. regcap > 0 builds a variant whose
    stencil kernels are limited to about that many registers per thread
    (through their launch bounds' minimum resident CTAs per SM), the
    counterpart of the artifact's REGNUM sweep (all.sh:14-19, nvcc
    --maxrregcount in make_sconf.sh)."""
    build_dir = BUILD if regcap <= 0 else BUILD.parent / f"_build_regcap{regcap}"
    lib = lib_path(regcap)
    build_dir.mkdir(exist_ok=True)
    lib.parent.mkdir(parents=True, exist_ok=True)
    jobs = jobs or max(1, os.cpu_count() or 1)
    us = units()
    if regcap > 0:
        us = [(n, s, f + [f"-DGBS_REGCAP={regcap}"]) for n, s, f in us]
    # the slowest units first: the batched kernels (every 2-D stencil in one
    # unit), then the big-radius 3-D boxes
    us.sort(key=lambda u: 0 if u[0].startswith("batch_") else (1 if "picks_1" in u[0] else 2))
    changed = False
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for name, did, log in ex.map(lambda u: compile_unit(u, verbose, build_dir), us):
            changed |= did
            if verbose and log:
                print(log)
    if changed or not lib.exists():
        objs = [str(build_dir / f"{u[0]}.o") for u in us]
        tmp = lib.with_suffix(".so.tmp")
        cmd = [nvcc(), "-shared"] + ARCH + ["-cudart", "shared", "-o", str(tmp)] + objs + [
            "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    import time
    t0 = time.time()
    cap = next((int(a.split("=")[1]) for a in sys.argv if a.startswith("--regcap=")), 0)
    print(build(verbose="-v" in sys.argv, regcap=cap), f"{time.time() - t0:.1f}s")
