"""Writes the C drop-in for each benchmark of an AN5D artifact checkout.

    python make_shims.py <artifact dir> <out dir> [stencil ...]

For each <stencil>.c of the artifact it writes <out dir>/<stencil>_gbs.c:
the same file with the body of the scop branch of kernel_stencil
(`if (scop) { #pragma scop ... #pragma endscop }`, e.g. star2d1r.c:14-25)
replaced by one gbs_run call, and `#include "gbstencil.h"` after common.h.
The OpenMP branch (the -c comparison) and the harness (common.h: -s/-t/-n/-c,
init_grid, check_result) stay the artifact's own. kernel_stencil keeps its
contract (common.h:42): both planes of A1 advanced `timestep` steps, result
in plane timestep % 2, return value the device milliseconds of the loop
(end_time = start_time + ms, which the function's own return statement
turns into ms). The generated files are the user's (they contain the
artifact's code); none is part of this repository.

Build one (the artifact's common.h next to it):

    gcc -O3 -fopenmp -DSB_TYPE=float -I<artifact dir> -I<repo>/include star2d1r_gbs.c \\
        -L<lib dir> -lgbstencil -Wl,-rpath,<lib dir> -lm
"""
from __future__ import annotations

import re
import sys
from pathlib import Path

TABLE = Path(__file__).resolve().parent.parent / "gbstencil" / "stencils.json"

CALL = """  if (scop) {
    /* GB300 engine (libgbstencil): the same time loop, %(what)s */
    gbs_desc gd = {0};
    double gbs_ms = 0.0;
    gd.stencil = gbs_stencil_id("%(name)s");
    gd.dtype = sizeof(SB_TYPE) == sizeof(double) ? GBS_F64 : GBS_F32;
    for (int a = 0; a < BENCH_DIM; a++) gd.n[a] = compsize;
    gd.timestep = timestep;
    gd.fp_mode = %(mode)s;
    if (gbs_run(&gd, A1, &gbs_ms) != GBS_OK) {
      fprintf(stderr, "gbstencil: %%s\\n", gbs_last_error());
      exit(EXIT_FAILURE);
    }
    end_time = start_time + gbs_ms;
    (void)A;
  }
"""


def shim(name: str, src: str) -> str:
    """The drop-in version of one benchmark source."""
    m = re.search(r"^  if \(scop\) \{\n#pragma scop\n.*?^#pragma endscop\n  \}\n", src, re.S | re.M)
    if not m:
        raise ValueError(f"{name}: no scop branch of the expected shape")
    # stencils without an exact form in the engine (3d125pt) run in FMA mode,
    # which agrees with the CPU branch within the documented tolerance
    import json
    exact = True
    if TABLE.exists():
        recs = {r["name"]: r for r in json.loads(TABLE.read_text())["stencils"]}
        exact = recs.get(name, {}).get("exact", True)
    fill = {"name": name, "mode": "GBS_FP_EXACT" if exact else "GBS_FP_FMA",
            "what": "exact arithmetic" if exact else "FMA mode (no exact form)"}
    out = src[:m.start()] + CALL % fill + src[m.end():]
    inc = '#include "common.h"\n'
    if inc not in out:
        raise ValueError(f"{name}: no common.h include")
    return out.replace(inc, inc + '#include "gbstencil.h"\n', 1)


def main(argv):
    if len(argv) < 2:
        print(__doc__)
        return 2
    src_dir, out_dir = Path(argv[0]), Path(argv[1])
    out_dir.mkdir(parents=True, exist_ok=True)
    names = argv[2:] or sorted(p.stem for p in src_dir.glob("*.c"))
    for n in names:
        (out_dir / f"{n}_gbs.c").write_text(shim(n, (src_dir / f"{n}.c").read_text()))
        print(out_dir / f"{n}_gbs.c")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
