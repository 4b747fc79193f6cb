"""The CPU oracle, pinned against the AN5D artifact's own CPU path.

* against the committed golden fixtures (made by tests/golden/make_golden.py
  from the artifact's own init_grid and kernel_stencil(scop=false)), bit for
  bit, on any machine;
* against the artifact's CPU path built here from its unmodified sources
  (oracle/_ref), bit for bit, on extra sizes, when those libraries exist.
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import pyoracle as po

GOLDEN = json.loads((Path(__file__).parent / "golden" / "reference_outputs.json").read_text())["cases"]
DT = {"float": np.float32, "double": np.float64}


def _digest(A, T):
    return hashlib.sha256(np.ascontiguousarray(A[T % 2]).tobytes()).hexdigest()


@pytest.fixture(scope="module", autouse=True)
def _oracle_built():
    po.lib()


@pytest.mark.parametrize("case", GOLDEN, ids=lambda c: f"{c['stencil']}-{c['dtype']}-{c['compsize']}-{c['timestep']}")
def test_oracle_matches_golden(case):
    dt = DT[case["dtype"]]
    A = po.init_grid(case["stencil"], case["compsize"], dt)
    po.run(case["stencil"], A, case["compsize"], case["timestep"])
    assert _digest(A, case["timestep"]) == case["sha256"]
    flat = A[case["timestep"] % 2].reshape(-1)
    for i, v in case["samples"]:
        assert flat[i] == dt(v)


needs_ref = pytest.mark.skipif(not po.ref_available(), reason="artifact sources not built here (oracle/_ref)")


@needs_ref
@pytest.mark.parametrize("name", [s["name"] for s in po.STENCILS])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_oracle_matches_reference_build(name, dt):
    dim = po.BY_NAME[name][1]["dim"]
    for n, T in ((31, 3), (8, 4)) if dim == 2 else ((9, 3), (6, 2)):
        A = po.ref_init_grid(name, n, dt)
        B = po.init_grid(name, n, dt)
        assert np.array_equal(A.view(np.uint8), B.view(np.uint8)), "init_grid differs"
        po.ref_run(name, A, n, T, scop=False)
        po.run(name, B, n, T)
        assert np.array_equal(A[T % 2].view(np.uint8), B[T % 2].view(np.uint8))
        # and the other plane too (u_{T-1} in the interior)
        assert np.array_equal(A.view(np.uint8), B.view(np.uint8))


@needs_ref
def test_reference_scop_and_openmp_branches_agree():
    """The artifact's two branches (scop loop and OpenMP loop) compute the
    same bits when built without contraction; the oracle restates both."""
    for name in ("star2d1r", "gradient2d", "box3d1r"):
        n = 17 if po.BY_NAME[name][1]["dim"] == 2 else 7
        A = po.ref_init_grid(name, n, np.float32)
        B = A.copy()
        po.ref_run(name, A, n, 3, scop=True)
        po.ref_run(name, B, n, 3, scop=False)
        assert np.array_equal(A.view(np.uint8), B.view(np.uint8))


def test_oracle_uneven_grid_is_axiswise():
    """The oracle's per-axis extents: a 2-D grid with n=(5, 9) equals the
    same computation done on the transposed problem when the stencil is
    symmetric under transposition of its taps (checked with box2d1r's
    structure via explicit numpy)."""
    name = "star2d1r"
    n = (5, 9)
    rng = np.random.default_rng(0)
    A = rng.random((2, n[0] + 2, n[1] + 2)).astype(np.float64)
    A[1] = A[0]
    B = A.copy()
    po.run(name, A, list(n), 2)
    c = po.reference_coefficients(name, np.float64)
    for t in range(2):
        s, d = B[t % 2], B[(t + 1) % 2]
        d[1:-1, 1:-1] = (c[0] * s[:-2, 1:-1] + c[1] * s[1:-1, :-2] + c[2] * s[1:-1, 1:-1]
                         + c[3] * s[1:-1, 2:] + c[4] * s[2:, 1:-1])
    assert np.array_equal(A[0], B[0])
