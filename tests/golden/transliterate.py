"""Mechanical Fortran -> Python transliteration of the reference's step subroutines.

Used only by tests/golden/make_golden.py, in a container where the reference source is
mounted, to execute the reference's own statements (collision, streaming, bounceback,
macro, collisionT, streamingT, bouncebackT, macroT of 2DRB.F90 / 3DRB.F90) on small
inputs and store the results as fixtures.  The translation is syntactic:

* the C preprocessor switches are resolved for a chosen set of #defines;
* `do v = a, b` / `enddo`, `if (...) then` / `elseif` / `else` / `endif` and one-line
  `if (...) stmt` become Python blocks; declarations, OpenMP directives, I/O and comments
  are dropped; `real(kind=8), parameter :: X = expr` inside a body becomes `X = expr`;
* `1.0d0` literals become Python floats, `dble`/`dsqrt`/`dabs` map to float/math.sqrt/abs,
  relational and logical operators map to Python's, array references `a(i,j)` become
  `a[i,j]` on numpy arrays allocated with room for the Fortran index ranges.

Python evaluates + - * / left to right with one IEEE double rounding per operation and no
fused multiply-add, which is how gfortran evaluates these expressions without -ffast-math,
so the fixtures are the reference's arithmetic.
"""
import math
import re

import numpy as np

ARRAYS = {"f", "f_post", "g", "g_post", "rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev", "Fx", "Fy",
          "ex", "ey", "ez", "opp", "exT", "eyT", "ezT", "oppT", "omega", "omegaT", "m", "meq", "m_post", "s",
          "fSource", "n", "neq", "q", "n_post", "up", "vp", "wp", "Tp", "un"}
LOCAL_ARRAYS = ["m", "meq", "m_post", "s", "fSource", "n", "neq", "q", "n_post", "un"]


def preprocess(lines, defines):
    out, stack = [], []
    for ln in lines:
        t = ln.strip()
        if t.startswith("#ifdef") or t.startswith("#ifndef"):
            name = t.split()[1]
            cond = (name in defines) if t.startswith("#ifdef") else (name not in defines)
            stack.append([cond, cond])
            continue
        if t.startswith("#else"):
            stack[-1][0] = not stack[-1][1]
            continue
        if t.startswith("#endif"):
            stack.pop()
            continue
        if all(c for c, _ in stack):
            out.append(ln)
    return out


def extract(lines, name):
    start = None
    for k, ln in enumerate(lines):
        if re.match(r"\s*subroutine\s+%s\s*\(\s*\)" % re.escape(name), ln, re.I):
            start = k + 1
            break
    if start is None:
        raise ValueError("subroutine %s not found" % name)
    for k in range(start, len(lines)):
        if re.match(r"\s*end\s+subroutine\s+%s\b" % re.escape(name), lines[k], re.I):
            return lines[start:k]
    raise ValueError("end of %s not found" % name)


def strip_comment(ln):
    if ln.lstrip().startswith("!$"):
        return ""
    return ln.split("!")[0]


def join_continuations(lines):
    out, buf = [], ""
    for ln in lines:
        s = strip_comment(ln).rstrip()
        if not s.strip():
            if buf:
                continue
            continue
        if buf:
            s = buf + " " + s.strip().lstrip("&")
        if s.rstrip().endswith("&"):
            buf = s.rstrip()[:-1]
            continue
        buf = ""
        out.append(s)
    return out


def convert_expr(e):
    e = re.sub(r"(\d+\.\d*|\d+)[dD]([+-]?\d+)", lambda m: "%se%s" % (m.group(1), m.group(2)), e)
    for a, b in ((".EQ.", "=="), (".NE.", "!="), (".GT.", ">"), (".LT.", "<"), (".GE.", ">="), (".LE.", "<="),
                 (".AND.", " and "), (".OR.", " or "), (".NOT.", " not "), (".TRUE.", "True"), (".FALSE.", "False")):
        e = re.sub(re.escape(a), b, e, flags=re.I)
    e = re.sub(r"\bdble\s*\(", "float(", e)
    e = re.sub(r"\bdsqrt\s*\(", "math.sqrt(", e)
    e = re.sub(r"\bdabs\s*\(", "abs(", e)
    # array references -> subscripts
    out, stack, k = [], [], 0
    while k < len(e):
        m = re.match(r"[A-Za-z_][A-Za-z0-9_]*", e[k:])
        if m:
            name = m.group(0)
            k2 = k + len(name)
            j = k2
            while j < len(e) and e[j] == " ":
                j += 1
            if j < len(e) and e[j] == "(" and name in ARRAYS:
                out.append(name + "[")
                stack.append("]")
                k = j + 1
                continue
            out.append(name)
            k = k2
            continue
        ch = e[k]
        if ch == "(":
            stack.append(")")
            out.append("(")
        elif ch == ")":
            out.append(stack.pop())
        else:
            out.append(ch)
        k += 1
    return "".join(out)


def to_python(body_lines, defines):
    lines = join_continuations(preprocess(body_lines, defines))
    py, ind = [], 1
    pad = lambda: "    " * ind
    for s in lines:
        t = s.strip()
        low = t.lower()
        if low.startswith(("use ", "implicit ", "return", "write", "open", "close", "call ", "stop")):
            continue
        mpar = re.match(r"real\s*\(\s*kind\s*=\s*8\s*\)\s*,\s*parameter\s*::\s*(\w+)\s*=\s*(.+)$", t, re.I)
        if mpar:
            py.append(pad() + "%s = %s" % (mpar.group(1), convert_expr(mpar.group(2))))
            continue
        if "::" in t:
            continue  # declaration
        mdo = re.match(r"do\s+(\w+)\s*=\s*(.+?)\s*,\s*(.+)$", t, re.I)
        if mdo:
            py.append(pad() + "for %s in range(%s, (%s) + 1):" % (mdo.group(1), convert_expr(mdo.group(2)),
                                                                convert_expr(mdo.group(3))))
            ind += 1
            py.append(pad() + "pass")
            continue
        if re.match(r"end\s*do$", t, re.I):
            ind -= 1
            continue
        mif = re.match(r"if\s*\((.*)\)\s*then$", t, re.I)
        if mif:
            py.append(pad() + "if %s:" % convert_expr(mif.group(1)))
            ind += 1
            py.append(pad() + "pass")  # blocks whose only statements (I/O, stop) were dropped
            continue
        melif = re.match(r"else\s*if\s*\((.*)\)\s*then$", t, re.I)
        if melif:
            ind -= 1
            py.append(pad() + "elif %s:" % convert_expr(melif.group(1)))
            ind += 1
            py.append(pad() + "pass")
            continue
        if re.match(r"else$", t, re.I):
            ind -= 1
            py.append(pad() + "else:")
            ind += 1
            py.append(pad() + "pass")
            continue
        if re.match(r"end\s*if$", t, re.I):
            ind -= 1
            continue
        m1 = re.match(r"if\s*\((.*?)\)\s+(\w.*)$", t, re.I)
        if m1 and "=" in m1.group(2):
            # one-line if: find the condition's closing parenthesis
            depth, cut = 0, None
            for k, ch in enumerate(t):
                if ch == "(":
                    depth += 1
                elif ch == ")":
                    depth -= 1
                    if depth == 0:
                        cut = k
                        break
            cond, stmt = t[t.index("(") + 1:cut], t[cut + 1:].strip()
            py.append(pad() + "if %s: %s" % (convert_expr(cond), convert_expr(stmt)))
            continue
        py.append(pad() + convert_expr(t))
    return py


def compile_subroutine(src_lines, name, defines):
    body = extract(src_lines, name)
    code = ["def %s(ns):" % name, "    globals().update(ns)"]
    code += ["    %s = ns.get('%s')" % (a, a) for a in sorted(ARRAYS)]
    code += to_python(body, defines)
    code += ["    ns.update({k: v for k, v in locals().items() if k != 'ns'})"]
    return "\n".join(code)


class ReferenceSubroutines:
    """The step subroutines of one reference file, executable on a namespace of module
    variables (scalars and numpy arrays indexed with the Fortran bounds)."""

    NAMES = ("collision", "streaming", "bounceback", "macro", "collisionT", "streamingT", "bouncebackT", "macroT")

    def __init__(self, path, defines, extra=()):
        src = open(path, encoding="utf-8-sig").read().splitlines()
        self.source = {}
        self.fn = {}
        for name in self.NAMES + tuple(extra):
            code = compile_subroutine(src, name, defines)
            self.source[name] = code
            glb = {"math": math, "np": np}
            exec(code, glb)
            self.fn[name] = glb[name]

    def run(self, name, ns):
        for a in LOCAL_ARRAYS:
            ns.setdefault(a, np.zeros(32))
        self.fn[name](ns)

    def step(self, ns):
        for name in self.NAMES:
            self.run(name, ns)
