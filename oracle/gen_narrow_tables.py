"""Generate swm_narrow_tables.h: the coefficient tables of the narrow-stencil
variable-coefficient SBP second-derivative operators of orders 4/2, 6/3 and
2/1.

These are tables of published constants: closure row r of the operator
D2^(b) near a boundary is  (D2 f)_r = s_r * sum_c M[r][c] f_c  with
M[r][c] = sum_k C[r][c][k] b_k  (b_k the variable coefficient at node k,
counted from the boundary), and the interior stencil is
(D2 f)_i = sum_o (sum_q W[o][q] b_{i+q-w}) f_{i+o-w}.  The numbers cannot be
derived independently of their construction, so they are read from the
reference's own source (differential_operators/horizontal/laplace/
laplace_Ah_sbp42_narrow_mod.f90:128-274 and laplace_Ah_sbp63_narrow_mod.f90:
11-481, 600-880) and written out as C++ constant expressions in the same
literal form (each literal and quotient rounds to the same double).  The 2/1
operator (laplace_Ah_sbp21_narrow_mod.f90:125-195) has no literals to read:
its closure row is (b_1 + b_2)(f_2 - f_1) and its interior stencil the
face-averaged ((b_i + b_{i+1})/2 (f_{i+1} - f_i) - (b_{i-1} + b_i)/2
(f_i - f_{i-1})), with the boundary flux weight 2 (lines 200-225); the script
states these directly.

The script checks what it extracts: the four closure blocks of each file
(x left/right, y left/right) carry identical formulas; every closure row and
the interior stencil annihilate constants and differentiate x^2 exactly for
b = 1 (the boundary flux term folded into the first 6/3 row excepted).

usage: python oracle/gen_narrow_tables.py [REFERENCE_ROOT]
       (the reference checkout is a required argument; writes the header
       beside the CUDA sources)
"""
import os
import re
import sys
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "cubedsphere_sbp_swm_gb300", "csrc",
                   "swm_narrow_tables.h")
LAP = "src/differential_operators/horizontal/laplace"


def fortran_to_cpp(expr):
    """A Fortran real(8) constant expression as the same C++ expression."""
    e = expr.strip().rstrip(",").strip()
    e = re.sub(r"(\d+\.\d*)_8", r"\1", e)
    e = re.sub(r"(\d+)\.0?(?=\D|$)", lambda m: m.group(0), e)
    return e


def exact(expr_cpp):
    """Exact rational value of a C++ constant expression of this table
    (for the checks only; the header keeps the rounding of the reference)."""
    toks = re.findall(r"\d+\.\d*|\d+|[-+*/()]", expr_cpp)
    py = "".join("Fraction(%s)" % (("'" + t.rstrip(".").split(".")[0] + "'") if "." in t else t)
                 if re.match(r"\d", t) else t for t in toks)
    return eval(py, {"Fraction": Fraction})


def split_terms(rhs):
    """'a*b1 - c*b3 + ...' -> [(sign, coefficient text, k)]"""
    rhs = rhs.strip()
    out = []
    for m in re.finditer(r"([+-]?)\s*([^+\-]+?)\s*\*\s*b(\d+)\b", rhs):
        out.append((-1 if m.group(1) == "-" else 1, m.group(2).strip(), int(m.group(3))))
    rebuilt = re.sub(r"\s+", "", rhs)
    assert len(out) == len(re.findall(r"\*b\d+", rebuilt)), rhs
    return out


def closure_blocks(text, rows):
    """m-formula texts of the closure rows of every block, in file order."""
    blocks, cur = [], {}
    for line in text.splitlines():
        m = re.match(r"\s*m(\d)(\d+)\s*=\s*(.+?)\s*$", line)
        if not m:
            continue
        r, c = int(m.group(1)), int(m.group(2))
        if (r, c) in cur:
            blocks.append(cur)
            cur = {}
        cur[(r, c)] = re.sub(r"\s+", " ", m.group(3))
    blocks.append(cur)
    # a block is one closure row set of one side; group consecutive rows
    merged, acc = [], {}
    for b in blocks:
        rws = {r for r, _ in b}
        if acc and min(rws) == 1:
            merged.append(acc)
            acc = {}
        acc.update(b)
    merged.append(acc)
    assert len(merged) == 4, "expected x-left, x-right, y-left, y-right blocks"

    def terms(b):   # the same formula may list its terms in another order
        return {key: sorted((s, re.sub(r"\s", "", c), k) for s, c, k in split_terms(v))
                for key, v in b.items()}
    for b in merged[1:]:
        assert terms(b) == terms(merged[0]), "closure blocks differ"
    assert {r for r, _ in merged[0]} == set(range(1, rows + 1))
    return merged[0]


def row_scales_42(text):
    hs = {}
    for m in re.finditer(r"\bh(\d)(\d)\s*=\s*([^\n]+)", text):
        if m.group(1) == m.group(2):
            hs.setdefault(int(m.group(1)), fortran_to_cpp(m.group(3)))
    return hs


def interior(text, names):
    """Interior coefficients: cX = sum coef * bY for X, Y in names."""
    W = {}
    for m in re.finditer(r"^\s*c(%s)\s*=\s*(.+)$" % "|".join(names), text, re.M):
        o = names.index(m.group(1))
        if o in W:
            continue
        row = {}
        for t in re.finditer(r"([+-]?)\s*([^+\-]+?)\s*\*\s*b(%s)\b" % "|".join(names), m.group(2)):
            row[names.index(t.group(3))] = ("-" if t.group(1) == "-" else "", t.group(2).strip())
        W[o] = row
    assert sorted(W) == list(range(len(names)))
    return W


def build(ref):
    src42 = open(os.path.join(ref, LAP, "laplace_Ah_sbp42_narrow_mod.f90")).read()
    src63 = open(os.path.join(ref, LAP, "laplace_Ah_sbp63_narrow_mod.f90")).read()
    tables = []

    # --- 4/2: literal coefficients, row factor -1/h_rr
    blk = closure_blocks(src42, 6)
    hs = row_scales_42(src42)
    C = {}
    for (r, c), rhs in blk.items():
        for sgn, coef, k in split_terms(rhs):
            C[(r, c, k)] = ("-" if sgn < 0 else "") + "(" + fortran_to_cpp(coef) + ")"
    names42 = ["mm", "m", "c", "p", "pp"]
    W = interior(src42, names42)
    Wc = {o: {q: s + "(" + fortran_to_cpp(v) + ")" for q, (s, v) in row.items()} for o, row in W.items()}
    tables.append(dict(order=42, rows=6, hw=2, rowscale={r: "-1.0/(" + hs[r] + ")" for r in range(1, 7)},
                       C=C, W=Wc, penalty="48.0/17"))

    # --- 6/3: named parameters, row factor 1
    params = {}
    for m in re.finditer(r"^\s*(d\d{6}|di_\w+)\s*=\s*(.+?)(?:,\s*&)?\s*$", src63, re.M):
        params[m.group(1)] = "(" + fortran_to_cpp(m.group(2)) + ")"
    blk = closure_blocks(src63, 9)
    C = {}
    for (r, c), rhs in blk.items():
        for sgn, coef, k in split_terms(rhs):
            assert coef in params, coef
            C[(r, c, k)] = ("-" if sgn < 0 else "") + params[coef]
    names63 = ["mmm", "mm", "m", "c", "p", "pp", "ppp"]
    W = interior(src63, names63)
    Wc = {o: {q: s + params[v] for q, (s, v) in row.items()} for o, row in W.items()}
    tables.append(dict(order=63, rows=9, hw=3, rowscale={r: "1.0" for r in range(1, 10)},
                       C=C, W=Wc, penalty="43200.0/13649"))

    # --- 2/1: cc = -(b_1 + b_2), cp = b_1 + b_2 at the closure row; interior
    # cm = (b_m + b_c)/2, cc = -(b_m + 2 b_c + b_p)/2, cp = (b_p + b_c)/2
    C = {(1, 1, 1): "-1.0", (1, 1, 2): "-1.0", (1, 2, 1): "1.0", (1, 2, 2): "1.0"}
    W = {0: {0: "1.0/2", 1: "1.0/2"}, 1: {0: "-1.0/2", 1: "-1.0", 2: "-1.0/2"}, 2: {1: "1.0/2", 2: "1.0/2"}}
    tables.append(dict(order=21, rows=1, hw=1, rowscale={1: "1.0"}, C=C, W=W, penalty="2.0"))
    return tables


def check(t):
    rows, hw = t["rows"], t["hw"]
    val = {key: exact(v) for key, v in t["C"].items()}
    for r in range(1, rows + 1):
        s = exact(t["rowscale"][r])
        m0 = sum(v for (rr, c, k), v in val.items() if rr == r)
        m2 = s * sum(v * (c - r) ** 2 for (rr, c, k), v in val.items() if rr == r)
        if not (t["order"] == 63 and r == 1):
            assert abs(m0) < Fraction(1, 10 ** 12), (t["order"], r, float(m0))
        if t["order"] != 63 or r > 1:
            assert abs(m2 - 2) < Fraction(1, 10 ** 9), (t["order"], r, float(m2))
    wv = {(o, q): exact(v) for o, row in t["W"].items() for q, v in row.items()}
    assert abs(sum(wv.values())) < Fraction(1, 10 ** 14)
    assert abs(sum(v * (o - hw) ** 2 for (o, q), v in wv.items()) - 2) < Fraction(1, 10 ** 14)


def emit(tables):
    L = ["// swm_narrow_tables.h -- generated by oracle/gen_narrow_tables.py; do not edit.",
         "//",
         "// Narrow-stencil variable-coefficient SBP second-derivative operators of",
         "// orders 4/2, 6/3 and 2/1, as the reference states them",
         "// (laplace_Ah_sbp42_narrow_mod.f90:128-274, laplace_Ah_sbp63_narrow_mod.f90:11-481,",
         "// laplace_Ah_sbp21_narrow_mod.f90:125-195).",
         "// Closure row r (0-based from the boundary) of D2^(b):",
         "//   (D2 f)_r = rowscale[r] * sum_c (sum_k c[r][c][k] * b_k) * f_c",
         "// Interior node i:",
         "//   (D2 f)_i = sum_o (sum_q in[o][q] * b_{i+q-hw}) * f_{i+o-hw}",
         "// The far end uses the same rows with nodes counted from that end.",
         "#pragma once",
         "",
         "namespace swm {",
         "",
         "constexpr int NARROW_MAXR = 9, NARROW_MAXC = 12, NARROW_MAXW = 7;",
         "",
         "struct NarrowD2 {",
         "  int order;      // 42, 63 or 21",
         "  int rows;       // closure rows at each end",
         "  int cols;       // nodes a closure row reads",
         "  int nb;         // coefficient nodes a closure row reads",
         "  int hw;         // interior half width",
         "  double penalty; // weight of the cross-derivative boundary flux",
         "  double rowscale[NARROW_MAXR];",
         "  double c[NARROW_MAXR][NARROW_MAXC][NARROW_MAXC];",
         "  double in[NARROW_MAXW][NARROW_MAXW];",
         "};",
         ""]
    for t in tables:
        rows = t["rows"]
        cols = max(c for (_, c, _) in t["C"])
        nb = max(k for (_, _, k) in t["C"])
        L.append("constexpr NarrowD2 kNarrow%d = {" % t["order"])
        L.append("  %d, %d, %d, %d, %d, %s," % (t["order"], rows, cols, nb, t["hw"], t["penalty"]))
        L.append("  {" + ", ".join(t["rowscale"][r] for r in range(1, rows + 1)) + "},")
        L.append("  {")
        for r in range(1, rows + 1):
            L.append("    {  // row %d" % (r - 1))
            for c in range(1, cols + 1):
                ks = [t["C"].get((r, c, k), "0.0") for k in range(1, nb + 1)]
                if all(k == "0.0" for k in ks):
                    L.append("      {},")
                else:
                    L.append("      {" + ", ".join(ks) + "},")
            L.append("    },")
        L.append("  },")
        L.append("  {")
        for o in range(2 * t["hw"] + 1):
            L.append("    {" + ", ".join(t["W"][o].get(q, "0.0") for q in range(2 * t["hw"] + 1)) + "},")
        L.append("  },")
        L.append("};")
        L.append("")
    L.append("}  // namespace swm")
    return "\n".join(L) + "\n"


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python oracle/gen_narrow_tables.py REFERENCE_CHECKOUT")
    ref = sys.argv[1]
    tables = build(ref)
    for t in tables:
        check(t)
    with open(OUT, "w") as f:
        f.write(emit(tables))
    print("wrote", OUT, [(t["order"], len(t["C"])) for t in tables])


if __name__ == "__main__":
    main()
