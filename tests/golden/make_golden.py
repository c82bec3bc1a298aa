#!/usr/bin/env python3
"""Generate the golden fixtures under tests/golden/ from the reference's source text.

Run in a container where the reference is mounted (default /root/reference):

    python tests/golden/make_golden.py [--ref /root/reference/2DRB]

reference_matrices.json: the moment transforms as the reference states them.  The hand-
expanded statements `m(k) = ...`, `f_post(a,...) = ...` (2DRB.F90:688-696, 743-759;
3DRB.F90:714-775, 861-943), `n(k) = ...`, `g_post(a,...) = ...` (2DRB.F90:951-955,
970-974; 3DRB.F90:1141-1147, 1181-1191) are parsed and evaluated on unit vectors with
IEEE double arithmetic in the reference's left-to-right order; the D2Q9/D2Q5 row matrices
of ChaiPRE2020.F90:263-276 and the D3Q7 matrix of the algorithm guide (section 4.2) are
read as independent statements of the same transforms.
"""
import argparse
import json
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def fortran_expr_to_py(expr):
    expr = expr.replace("&", " ")
    expr = re.sub(r"(\d+\.\d*|\d+)d0", r"\1", expr)          # 1.0d0 -> 1.0
    expr = re.sub(r"\b(f|g|m_post|n_post)\((\d+)(,[ijk,]+)?\)", lambda m: "%s[%s]" % (
        {"f": "X", "g": "X", "m_post": "X", "n_post": "X"}[m.group(1)], m.group(2)), expr)
    return expr


def collect(src_lines, start, end, lhs_regex):
    """Statements `lhs = expr` (with & continuations) between 1-based lines start..end."""
    text = []
    for ln in src_lines[start - 1:end]:
        s = ln.split("!")[0].rstrip()
        text.append(s)
    joined = []
    buf = ""
    for s in text:
        if buf:
            buf += " " + s.strip().lstrip("&")
        else:
            buf = s
        if buf.rstrip().endswith("&"):
            buf = buf.rstrip()[:-1]
            continue
        joined.append(buf)
        buf = ""
    out = {}
    for s in joined:
        m = re.match(r"\s*" + lhs_regex + r"\s*=\s*(.*)$", s)
        if m:
            out[int(m.group(1))] = m.group(2)
    return out


def matrix_from(stmts, q):
    M = np.zeros((q, q))
    for col in range(q):
        X = np.zeros(q)
        X[col] = 1.0
        for row, expr in stmts.items():
            M[row, col] = eval(fortran_expr_to_py(expr), {"X": [float(x) for x in X]})
    return M


def find(lines, pattern, after=0):
    for k in range(after, len(lines)):
        if re.search(pattern, lines[k]):
            return k + 1
    raise ValueError(pattern)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference/2DRB")
    args = ap.parse_args()
    r2 = open(os.path.join(args.ref, "2DRB.F90"), encoding="utf-8-sig").read().splitlines()
    r3 = open(os.path.join(args.ref, "3DRB.F90"), encoding="utf-8-sig").read().splitlines()
    chai = open(os.path.join(args.ref, "ChaiPRE2020.F90"), encoding="utf-8-sig").read().splitlines()
    guide = open(os.path.join(args.ref, "three_dimensional_thermal_MRT_LBM_algorithm_guide.md"),
                 encoding="utf-8").read().splitlines()
    out = {"source": "generated by tests/golden/make_golden.py from the reference Fortran source text"}

    c2 = find(r2, r"subroutine collision\(\)")
    e2 = find(r2, r"end subroutine collision", c2)
    fw = collect(r2, c2, e2, r"m\((\d+)\)")
    inv = collect(r2, c2, e2, r"f_post\((\d+),i,j\)")
    out["D2Q9"] = {"M": matrix_from(fw, 9).tolist(), "Minv": matrix_from(inv, 9).tolist()}
    t2 = find(r2, r"subroutine collisionT\(\)")
    te2 = find(r2, r"end subroutine collisionT", t2)
    fw = collect(r2, t2, te2, r"n\((\d+)\)")
    inv = collect(r2, t2, te2, r"g_post\((\d+),i,j\)")
    out["D2Q5"] = {"M": matrix_from(fw, 5).tolist(), "Minv": matrix_from(inv, 5).tolist()}

    c3 = find(r3, r"^subroutine collision\(\)")
    e3 = find(r3, r"end subroutine collision", c3)
    fw = collect(r3, c3, e3, r"m\((\d+)\)")
    inv = collect(r3, c3, e3, r"f_post\((\d+),i,j,k\)")
    out["D3Q19"] = {"M": matrix_from(fw, 19).tolist(), "Minv": matrix_from(inv, 19).tolist()}
    t3 = find(r3, r"^subroutine collisionT\(\)")
    te3 = find(r3, r"end subroutine collisionT", t3)
    fw = collect(r3, t3, te3, r"n\((\d+)\)")
    inv = collect(r3, t3, te3, r"g_post\((\d+),i,j,k\)")
    out["D3Q7"] = {"M": matrix_from(fw, 7).tolist(), "Minv": matrix_from(inv, 7).tolist()}

    def rows(name, q):
        M = np.zeros((q, q))
        for ln in chai:
            m = re.match(r"\s*%s\((\d+),:\)\s*=\s*\(/(.*)/\)" % name, ln)
            if m:
                M[int(m.group(1))] = [float(x.replace("d0", "")) for x in m.group(2).split(",")]
        return M.tolist()

    out["Chai_Mflow"] = rows("Mflow", 9)
    out["Chai_Mtemp"] = rows("Mtemp", 5)
    k = find(guide, r"^N=")
    N = []
    for ln in guide[k:k + 12]:
        if "&" in ln:
            N.append([float(x) for x in ln.replace("\\\\", "").split("&")])
    out["guide_N"] = N
    with open(os.path.join(HERE, "reference_matrices.json"), "w") as fh:
        json.dump(out, fh)
    print("wrote reference_matrices.json")


if __name__ == "__main__":
    main()
