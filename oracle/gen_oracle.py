"""Generate ``oracle_stencils.c``, the CPU oracle, from the stencil tap table.

TEST INFRASTRUCTURE ONLY. The oracle is the reference the CUDA engine is tested against: only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use it. No product code path calls it.

For every stencil of the table and every element type (float ``f``, double
``d``, long double ``q``) it emits

    void oracle_<name>_<t>(T *A, const int *n, int timestep,
                           const T *coef, T divisor, T eps)

which restates the reference's OpenMP CPU branch (e.g. ``star2d1r.c:26-37``):
for every timestep a ``#pragma omp parallel for`` over the outermost interior
index, the update expression evaluated as one left-to-right sum of
``coef[t] * A[t%2][...]`` products in the order the source writes them, then
the divisor. ``n`` holds the interior extent per axis (the reference is cubic,
``n[0]==n[1]==n[2]==compsize``; the batched tests use uneven grids). The
gradient form restates ``gradient2d.c:17-21`` with the same C type
promotions (float squares summed in float, then the double ``sqrt`` and
division); the grouped form of ``3d125pt.c:18-48`` sums each group in T and
combines the groups with their double literals in double. Compile with ``-ffp-contract=off`` so that no product is fused
into an add: this makes the build's results independent of the host ISA
(gcc contracts to FMA by default on aarch64, not on x86-64 without -mfma).

Coefficients come in through ``coef`` so that the same code serves the
reference literals (converted to T exactly as C converts ``0.1873f``) and the
random coefficients of the synthetic workloads.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

TYPES = {"f": "float", "d": "double", "q": "long double"}


def ident(name):
    return name.replace("-", "_")


def emit_linear(rec, t, T):
    dim, r = rec["dim"], rec["rad"]
    name = ident(rec["name"])
    lines = []
    lines.append(f"void oracle_{name}_{t}({T} *A1, const int *n, int timestep,")
    lines.append(f"    const {T} *coef, {T} divisor, {T} eps)")
    lines.append("{")
    lines.append("  (void)eps; (void)divisor;")
    if dim == 2:
        lines.append(f"  const long d0 = n[0] + {2 * r}, d1 = n[1] + {2 * r};")
        lines.append(f"  {T} (*A)[d0][d1] = ({T} (*)[d0][d1])A1;")
    else:
        lines.append(f"  const long d0 = n[0] + {2 * r}, d1 = n[1] + {2 * r}, d2 = n[2] + {2 * r};")
        lines.append(f"  {T} (*A)[d0][d1][d2] = ({T} (*)[d0][d1][d2])A1;")
    idx = ["i", "j", "k"][:dim]
    terms = []
    for ti, term in enumerate(rec["terms"]):
        sub = "".join(f"[{v}{o:+d}]" if o else f"[{v}]" for v, o in zip(idx, term["off"]))
        terms.append(f"coef[{ti}] * A[t%2]{sub}")
    expr = "\n            + ".join(terms)
    if rec["divisor"]:
        expr = f"({expr}) / divisor"
    lhs = "A[(t+1)%2]" + "".join(f"[{v}]" for v in idx)
    lines.append("  for (int t = 0; t < timestep; t++) {")
    lines.append("#pragma omp parallel for schedule(static)")
    lines.append(f"    for (long i = {r}; i < d0 - {r}; i++)")
    lines.append(f"      for (long j = {r}; j < d1 - {r}; j++)")
    if dim == 3:
        lines.append(f"        for (long k = {r}; k < d2 - {r}; k++)")
    lines.append(f"          {lhs} =")
    lines.append(f"            {expr};")
    lines.append("  }")
    lines.append("}")
    return "\n".join(lines)


def emit_grouped(rec, t, T):
    """3d125pt.c:18-48: sum over groups of ``c * (A + A + ...)`` with double
    literals c: each group sum in T (left to right), the products and their
    sum in double (long double for the long double oracle), rounded once on
    store. coef == NULL: the source literals; else group g takes coef[first
    term of g] (callers pass group-constant coefficients)."""
    dim, r = rec["dim"], rec["rad"]
    name = ident(rec["name"])
    wide = "long double" if t == "q" else "double"
    idx = ["i", "j", "k"][:dim]
    lines = [f"void oracle_{name}_{t}({T} *A1, const int *n, int timestep,",
             f"    const {T} *coef, {T} divisor, {T} eps)",
             "{",
             "  (void)eps; (void)divisor;",
             f"  const long d0 = n[0] + {2 * r}, d1 = n[1] + {2 * r}, d2 = n[2] + {2 * r};",
             f"  {T} (*A)[d0][d1][d2] = ({T} (*)[d0][d1][d2])A1;"]
    first = 0
    for g, grp in enumerate(rec["groups"]):
        lines.append(f"  const {wide} c{g} = coef ? ({wide})coef[{first}] : ({wide}){grp['literal']};")
        first += len(grp["refs"])
    groups = []
    for g, grp in enumerate(rec["groups"]):
        refs = []
        for off in grp["refs"]:
            refs.append("A[t%2]" + "".join(f"[{v}{o:+d}]" if o else f"[{v}]" for v, o in zip(idx, off)))
        groups.append(f"c{g} * ({T})(" + " + ".join(refs) + ")")
    lhs = "A[(t+1)%2]" + "".join(f"[{v}]" for v in idx)
    lines += ["  for (int t = 0; t < timestep; t++) {",
              "#pragma omp parallel for schedule(static)",
              f"    for (long i = {r}; i < d0 - {r}; i++)",
              f"      for (long j = {r}; j < d1 - {r}; j++)",
              f"        for (long k = {r}; k < d2 - {r}; k++)",
              f"          {lhs} = ({T})(" + "\n            + ".join(groups).replace("\\n", "\n") + ");",
              "  }",
              "}"]
    return "\n".join(lines)


def emit_gradient(rec, t, T):
    r = rec["rad"]
    name = ident(rec["name"])
    diffs = []
    for (di, dj) in rec["neighbours"]:
        sub = f"[i{di:+d}]" if di else "[i]"
        sub += f"[j{dj:+d}]" if dj else "[j]"
        d = f"(A[t%2][i][j] - A[t%2]{sub})"
        diffs.append(f"{d} * {d}")
    s = " +\n                 ".join(diffs)
    # 1.0f / sqrt(x): the literal is converted to double, sqrt is the double
    # libm function, the sum A + q is evaluated in double and rounded on store.
    wide = "long double" if t == "q" else "double"
    sqrt_fn = "sqrtl" if t == "q" else "sqrt"
    return "\n".join([
        f"void oracle_{name}_{t}({T} *A1, const int *n, int timestep,",
        f"    const {T} *coef, {T} divisor, {T} eps)",
        "{",
        "  (void)divisor;",
        f"  const long d0 = n[0] + {2 * r}, d1 = n[1] + {2 * r};",
        f"  {T} (*A)[d0][d1] = ({T} (*)[d0][d1])A1;",
        f"  const {wide} numer = ({wide})coef[0];",
        "  for (int t = 0; t < timestep; t++) {",
        "#pragma omp parallel for schedule(static)",
        f"    for (long i = {r}; i < d0 - {r}; i++)",
        f"      for (long j = {r}; j < d1 - {r}; j++) {{",
        f"        const {T} s = eps + {s};",
        f"        A[(t+1)%2][i][j] = ({T})(({wide})A[t%2][i][j] + numer / {sqrt_fn}(({wide})s));",
        "      }",
        "  }",
        "}",
    ])


def main(argv):
    table = Path(argv[1])
    out = Path(argv[2])
    recs = json.loads(table.read_text())["stencils"]
    parts = [
        "/* Generated by oracle/gen_oracle.py from the stencil tap table.",
        " * TEST INFRASTRUCTURE ONLY: the CPU oracle for the CUDA engine's",
        " * parity tests and the timed CPU baseline. Do not edit by hand. */",
        "#include <math.h>",
        "",
    ]
    for rec in recs:
        for t, T in TYPES.items():
            if rec["kind"] == "linear" and rec.get("groups"):
                parts.append(emit_grouped(rec, t, T))
            elif rec["kind"] == "linear":
                parts.append(emit_linear(rec, t, T))
            else:
                parts.append(emit_gradient(rec, t, T))
            parts.append("")
    # dispatch table
    for t, T in TYPES.items():
        parts.append(f"typedef void (*oracle_fn_{t})({T} *, const int *, int, const {T} *, {T}, {T});")
        parts.append(f"const oracle_fn_{t} oracle_table_{t}[] = {{")
        for rec in recs:
            parts.append(f"  oracle_{ident(rec['name'])}_{t},")
        parts.append("};")
        parts.append("")
    out.write_text("\n".join(parts))


if __name__ == "__main__":
    main(sys.argv)
