"""Generate the stencil tap table from the AN5D artifact's benchmark sources.

Run once, in a checkout that has the artifact next to it:

    python gen_stencil_table.py <artifact-dir>

It reads the ``#pragma scop`` region of every in-scope ``<stencil>.c``
(e.g. ``star2d1r.c:14-24``), parses the update expression with a small
recursive-descent parser and writes two files that the engine and the oracle
build from:

* ``stencils.json`` (this directory): one record per stencil with its
  dimension, radius, ``BENCH_FPP``, the terms in source order (offset and the
  float literal as written), the divisor and the evaluation form;
* ``../csrc/stencil_table.cuh``: the same table as C++ types whose term lists
  are compile-time constants (``terms(f)`` calls ``f`` once per term with
  ``std::integral_constant`` offsets), used to instantiate the kernel family.

Nothing here is hand-entered: the coefficients, the term order (which fixes
the floating-point summation order) and the quirks (the doubled
``A[i-4][j]`` tap of ``star2d4r.c:19,24``, the ``/118`` and ``/159``
divisors, the nonlinear ``gradient2d.c:17-21``) all come from the source.
``3d125pt.c`` (not in the artifact's benchmark set) has a third form: a sum
of groups ``c * (A + A + ...)`` with double literals, whose float build
sums each group in float and combines the groups in double. Its record
lists the groups and its terms (one per occurrence, duplicates kept), and it
has no exact mode in the engine (``exact: false``): the kernel family
evaluates it in FMA mode only.
"""
from __future__ import annotations

import json
import re
import struct
import sys
from fractions import Fraction
from pathlib import Path

STENCILS = [
    "star2d1r", "star2d2r", "star2d3r", "star2d4r",
    "box2d1r", "box2d2r", "box2d3r", "box2d4r",
    "j2d5pt", "j2d9pt", "j2d9pt-gol", "gradient2d",
    "star3d1r", "star3d2r", "star3d3r", "star3d4r",
    "box3d1r", "box3d2r", "box3d3r", "box3d4r",
    "j3d27pt", "3d125pt",
]


# --------------------------------------------------------------------------
# Exact decimal -> binary32 rounding (round to nearest, ties to even), the
# rounding a C compiler applies to a literal like ``0.1873f``.
# --------------------------------------------------------------------------
def _f32_bits(x: float) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


def _f32_from_bits(b: int) -> float:
    return struct.unpack("<f", struct.pack("<I", b))[0]


def round_to_f32(text: str) -> float:
    """Correctly rounded binary32 value of a decimal literal (no suffix)."""
    q = Fraction(text)
    approx = struct.unpack("<f", struct.pack("<f", float(q)))[0]
    best = None
    b0 = _f32_bits(approx)
    cands = []
    for db in (-2, -1, 0, 1, 2):
        b = b0 + db
        if 0 <= b < 0x7F800000 or (0x80000000 <= b < 0xFF800000):
            cands.append(_f32_from_bits(b))
    for c in cands:
        d = abs(Fraction(c) - q)
        key = (d, _f32_bits(c) & 1)  # ties go to the even mantissa
        if best is None or key < best[0]:
            best = (key, c)
    return best[1]


# --------------------------------------------------------------------------
# Tokeniser / parser for the scop right-hand sides.
# --------------------------------------------------------------------------
TOKEN = re.compile(
    r"\s*(?:(?P<num>\d+\.\d*(?:[eE][-+]?\d+)?f?|\d*\.\d+(?:[eE][-+]?\d+)?f?|\d+f?)"
    r"|(?P<ref>A\[t%2\](?:\[[^\]]*\]){2,3})"
    r"|(?P<id>[A-Za-z_]\w*)"
    r"|(?P<op>[-+*/()]))"
)


def tokenize(s: str):
    pos, out = 0, []
    s = s.strip()
    while pos < len(s):
        m = TOKEN.match(s, pos)
        if not m or m.end() == pos:
            raise ValueError(f"cannot tokenise at: {s[pos:pos + 40]!r}")
        pos = m.end()
        for kind in ("num", "ref", "id", "op"):
            if m.group(kind) is not None:
                out.append((kind, m.group(kind)))
                break
    return out


def parse_index(expr: str, var: str) -> int:
    expr = expr.replace(" ", "")
    if expr == var:
        return 0
    m = re.fullmatch(re.escape(var) + r"([-+])(\d+)", expr)
    if not m:
        raise ValueError(f"unexpected index {expr!r} for {var}")
    v = int(m.group(2))
    return v if m.group(1) == "+" else -v


class Parser:
    """expr := term (('+'|'-') term)* ; term := unary (('*'|'/') unary)* ;
    unary := '-' unary | atom ; atom := num | ref | id '(' expr ')' | '(' expr ')'"""

    def __init__(self, toks, names):
        self.t, self.i, self.names = toks, 0, names

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.peek()
        if val is not None and tok[1] != val:
            raise ValueError(f"expected {val!r}, got {tok}")
        self.i += 1
        return tok

    def expr(self):
        node = self.term()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            node = ("add" if op == "+" else "sub", node, self.term())
        return node

    def term(self):
        node = self.unary()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            node = ("mul" if op == "*" else "div", node, self.unary())
        return node

    def unary(self):
        if self.peek()[1] == "-":
            self.take()
            return ("neg", self.unary())
        return self.atom()

    def atom(self):
        kind, val = self.take()
        if kind == "num":
            return ("num", val)
        if kind == "ref":
            idx = re.findall(r"\[([^\]]*)\]", val)[1:]
            return ("ref", tuple(parse_index(e, n) for e, n in zip(idx, self.names)))
        if kind == "id":
            self.take("(")
            arg = self.expr()
            self.take(")")
            return ("call", val, arg)
        if val == "(":
            node = self.expr()
            self.take(")")
            return node
        raise ValueError(f"unexpected token {val!r}")


def literal_value(text: str):
    """(is_float_literal, value). ``0.1873f`` -> binary32; ``118`` -> int."""
    if text.endswith("f"):
        return True, round_to_f32(text[:-1])
    if "." in text or "e" in text.lower():
        return False, float(text)
    return False, int(text)


def flatten_sum(node, sign=1):
    """Left-to-right list of (sign, subtree) for a chain of + / -."""
    if node[0] == "add":
        return flatten_sum(node[1], sign) + [(1 * sign, node[2])]
    if node[0] == "sub":
        return flatten_sum(node[1], sign) + [(-1 * sign, node[2])]
    return [(sign, node)]


def linear_terms(node):
    terms = []
    chain = flatten_sum(node)
    for pos, (sgn, t) in enumerate(chain):
        if t[0] != "mul":
            raise ValueError(f"not a product: {t}")
        c, r = t[1], t[2]
        neg = False
        if c[0] == "neg":
            neg, c = True, c[1]
        if c[0] != "num" or r[0] != "ref":
            raise ValueError(f"unexpected product {t}")
        if sgn < 0 and pos == 0:
            raise ValueError("leading subtraction")
        is_f, v = literal_value(c[1])
        if not is_f:
            raise ValueError(f"coefficient is not a float literal: {c[1]}")
        s = -1.0 if (neg != (sgn < 0)) else 1.0
        terms.append({"off": list(r[1]), "literal": ("-" if s < 0 else "") + c[1],
                      "value": s * v})
    return terms


def analyse(name: str, src: str):
    dim = int(re.search(r"#define BENCH_DIM (\d+)", src).group(1))
    fpp = int(re.search(r"#define BENCH_FPP (\d+)", src).group(1))
    rad = int(re.search(r"#define BENCH_RAD (\d+)", src).group(1))
    head = src.split("#pragma scop")[0]
    scop_start = head.count("\n") + 1
    scop = src.split("#pragma scop", 1)[1].split("#pragma endscop", 1)[0]
    scop_end = scop_start + scop.count("\n")
    # the loop variables in array order, as the assignment indexes A
    m = re.search(r"A\[\(t\+1\)%2\]((?:\[\w+\])+)\s*=", scop)
    names = re.findall(r"\[(\w+)\]", m.group(1))
    assert len(names) == dim, (name, names)
    rhs = scop[m.end():].rsplit(";", 1)[0]
    tree = Parser(tokenize(rhs), names).expr()

    rec = {"name": name, "dim": dim, "rad": rad, "fpp": fpp,
           "source": f"{name}.c:{scop_start}-{scop_end}"}
    divisor = None
    body = tree
    if tree[0] == "div" and tree[2][0] == "num":
        is_f, dv = literal_value(tree[2][1])
        if is_f:
            raise ValueError("float divisor not expected")
        divisor, body = dv, tree[1]
    rec["exact"] = True
    try:
        terms = linear_terms(body)
        rec.update(kind="linear", terms=terms, divisor=divisor)
    except ValueError:
        try:
            groups = group_terms(body)
            terms = [{"off": list(o), "literal": g["literal"], "value": g["value"], "group": gi}
                     for gi, g in enumerate(groups) for o in g["refs"]]
            rec.update(kind="linear", terms=terms, divisor=divisor, groups=groups, exact=False)
        except ValueError:
            rec.update(analyse_gradient(tree, dim))
    if rec["kind"] == "linear":
        rows = [t["off"][0] for t in rec["terms"]]
        rec["grouped"] = all(a <= b for a, b in zip(rows, rows[1:]))
        if not rec["exact"]:
            rec["form"] = "assoc"   # FMA mode only: any term order
        else:
            rec["form"] = "assoc" if (rec["grouped"] and is_box(rec)) else "direct"
        rec["ntaps"] = len({tuple(t["off"]) for t in rec["terms"]})
        rec["nterms"] = len(rec["terms"])
        rmax = max(max(abs(o) for o in t["off"]) for t in rec["terms"])
        assert rmax == rad, (name, rmax, rad)
    return rec


def group_terms(node):
    """``c1 * (A + A + ...) + c2 * (...) + ...`` with double literals c
    (3d125pt.c:18-48): [{literal, value, refs: [offset, ...]}] in source
    order."""
    groups = []
    for sgn, t in flatten_sum(node):
        if sgn < 0 or t[0] != "mul" or t[1][0] != "num":
            raise ValueError("not a grouped sum")
        is_f, v = literal_value(t[1][1])
        if is_f:
            raise ValueError("grouped sums take double literals")
        refs = []
        for s2, r in flatten_sum(t[2]):
            if s2 < 0 or r[0] != "ref":
                raise ValueError("group is not a sum of grid references")
            refs.append(list(r[1]))
        groups.append({"literal": t[1][1], "value": float(v), "refs": refs})
    return groups


def is_box(rec):
    """A stencil with off-centre taps in the outermost direction that also
    move in an inner direction (a 'box'); the others are stars."""
    return any(t["off"][0] != 0 and any(o != 0 for o in t["off"][1:])
               for t in rec["terms"])


def analyse_gradient(tree, dim):
    """``A[c] + 1.0f / sqrt(EPS + sum_n (A[c]-A[n])*(A[c]-A[n]))``
    (``gradient2d.c:17-21``)."""
    if tree[0] != "add" or tree[1] != ("ref", (0,) * dim):
        raise ValueError("unsupported expression")
    q = tree[2]
    if q[0] != "div" or q[1][0] != "num" or q[2][0] != "call" or q[2][1] != "sqrt":
        raise ValueError("unsupported expression")
    num_is_f, num = literal_value(q[1][1])
    chain = flatten_sum(q[2][2])
    (s0, eps_node), rest = chain[0], chain[1:]
    eps_is_f, eps = literal_value(eps_node[1])
    nbrs = []
    for sgn, t in rest:
        assert sgn > 0 and t[0] == "mul" and t[1] == t[2] and t[1][0] == "sub"
        a, b = t[1][1], t[1][2]
        assert a == ("ref", (0,) * dim) and b[0] == "ref"
        nbrs.append(list(b[1]))
    assert num_is_f and eps_is_f
    return {"kind": "gradient", "numerator": num, "numerator_literal": q[1][1],
            "eps": eps, "eps_literal": eps_node[1], "neighbours": nbrs,
            "divisor": None, "grouped": False, "form": "direct",
            "ntaps": 1 + len(nbrs), "nterms": len(nbrs)}


# --------------------------------------------------------------------------
# Emitters
# --------------------------------------------------------------------------
def c_ident(name):
    return name.replace("-", "_")


def hexf(v: float) -> str:
    return float(v).hex()


def emit_header(recs) -> str:
    out = [
        "// Generated by gbstencil/gen_stencil_table.py from the artifact's",
        "// <stencil>.c scop regions. Do not edit by hand.",
        "#pragma once",
        "#include <type_traits>",
        "",
        "namespace gbs {",
        "template <int N> using C = std::integral_constant<int, N>;",
        "enum { KIND_LINEAR = 0, KIND_GRADIENT = 1 };",
        "",
    ]
    for sid, r in enumerate(recs):
        n = c_ident(r["name"])
        out.append(f"// {r['name']}: {r['source']}")
        out.append(f"struct st_{n} {{")
        out.append(f"  static constexpr int kId = {sid}, kDim = {r['dim']}, kRad = {r['rad']}, kFpp = {r['fpp']};")
        kind = "KIND_LINEAR" if r["kind"] == "linear" else "KIND_GRADIENT"
        out.append(f"  static constexpr int kKind = {kind};")
        out.append(f"  static constexpr int kTerms = {r['nterms']};")
        out.append(f"  static constexpr bool kHasDiv = {'true' if r['divisor'] else 'false'};")
        out.append(f"  static constexpr bool kGrouped = {'true' if r['grouped'] else 'false'};")
        out.append(f"  static constexpr bool kAssoc = {'true' if r['form'] == 'assoc' else 'false'};")
        out.append(f"  static constexpr bool kExact = {'true' if r.get('exact', True) else 'false'};")
        offs_all = [t["off"] for t in r["terms"]] if r["kind"] == "linear" else r["neighbours"]
        rows = ", ".join("{" + ", ".join(str(v) for v in (list(o) + [0] * (3 - len(o)))) + "}" for o in offs_all)
        out.append(f"  static constexpr int kOff[kTerms][3] = {{{rows}}};")
        out.append("  // f(term index, di, dj, dk) once per term, in source order")
        out.append("  template <class F> __host__ __device__ __forceinline__ static void terms(F &&f) {")
        if r["kind"] == "linear":
            offs = [t["off"] for t in r["terms"]]
        else:
            offs = r["neighbours"]
        for ti, o in enumerate(offs):
            o3 = list(o) + [0] * (3 - len(o))
            out.append(f"    f(C<{ti}>(), C<{o3[0]}>(), C<{o3[1]}>(), C<{o3[2]}>());")
        out.append("  }")
        out.append("};")
        out.append("")
    out.append("// X(id, struct) for every stencil, in table order")
    out.append("#define GBS_FOR_EACH_STENCIL(X) \\")
    lines = [f"  X({sid}, st_{c_ident(r['name'])})" for sid, r in enumerate(recs)]
    out.append(" \\\n".join(lines))
    out.append("")
    out.append(f"constexpr int kNumStencils = {len(recs)};")
    out.append("template <int ID> struct StencilById;")
    for sid, r in enumerate(recs):
        out.append(f"template <> struct StencilById<{sid}> {{ using type = st_{c_ident(r['name'])}; }};")
    out.append("}  // namespace gbs")
    out.append("")
    return "\n".join(out)


def emit_host_table(recs) -> str:
    """Plain C table for host code: names, shapes, reference coefficients."""
    out = [
        "// Generated by gbstencil/gen_stencil_table.py. Do not edit by hand.",
        "#pragma once",
        "typedef struct { int di, dj, dk; double coef; } gbs_tap_t;",
        "typedef struct {",
        "  const char *name; int dim, rad, fpp, kind, nterms, grouped, assoc;",
        "  int divisor;            /* 0 = none */",
        "  float numerator, eps;   /* gradient form only */",
        "  const gbs_tap_t *terms; /* linear: coefficient per term; gradient: neighbours */",
        "} gbs_stencil_def_t;",
        "",
    ]
    for r in recs:
        n = c_ident(r["name"])
        out.append(f"static const gbs_tap_t gbs_terms_{n}[] = {{")
        if r["kind"] == "linear":
            for t in r["terms"]:
                o = list(t["off"]) + [0] * (3 - r["dim"])
                out.append(f"  {{{o[0]}, {o[1]}, {o[2]}, {hexf(t['value'])}}},  /* {t['literal']} */")
        else:
            for o in r["neighbours"]:
                o = list(o) + [0] * (3 - r["dim"])
                out.append(f"  {{{o[0]}, {o[1]}, {o[2]}, 0.0}},")
        out.append("};")
    out.append("")
    out.append("static const gbs_stencil_def_t gbs_stencil_defs[] = {")
    for r in recs:
        n = c_ident(r["name"])
        kind = 0 if r["kind"] == "linear" else 1
        num = hexf(r.get("numerator", 0.0)) + "f"
        eps = hexf(r.get("eps", 0.0)) + "f"
        out.append(f"  {{\"{r['name']}\", {r['dim']}, {r['rad']}, {r['fpp']}, {kind}, {r['nterms']}, "
                   f"{int(r['grouped'])}, {int(r['form'] == 'assoc')}, {r['divisor'] or 0}, {num}, {eps}, gbs_terms_{n}}},")
    out.append("};")
    out.append(f"#define GBS_NUM_STENCILS {len(recs)}")
    out.append("")
    return "\n".join(out)


def main(argv):
    src_dir = Path(argv[1] if len(argv) > 1 else ".")
    here = Path(__file__).resolve().parent
    recs = [analyse(n, (src_dir / f"{n}.c").read_text()) for n in STENCILS]
    for r in recs:
        if r["kind"] == "linear":
            for t in r["terms"]:
                t["value_hex"] = hexf(t["value"])
    (here / "stencils.json").write_text(json.dumps({"stencils": recs}, indent=1) + "\n")
    csrc = here.parent / "csrc"
    (csrc / "stencil_table.cuh").write_text(emit_header(recs))
    (csrc / "stencil_defs.h").write_text(emit_host_table(recs))
    for r in recs:
        print(f"{r['name']:11s} D={r['dim']} r={r['rad']} fpp={r['fpp']:4d} kind={r['kind']:8s} "
              f"terms={r['nterms']:4d} taps={r['ntaps']:4d} div={r['divisor']} grouped={r['grouped']} form={r['form']}")


if __name__ == "__main__":
    main(sys.argv)
