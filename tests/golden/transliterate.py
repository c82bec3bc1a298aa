"""Mechanical Fortran -> Python transliteration of the reference's subroutines.

Used only by tests/golden/make_golden.py, in a container where the reference source is
mounted, to execute the reference's own statements (the time-step subroutines, the
restart reconstruction and the post-processing diagnostics of 2DRB.F90 / 3DRB.F90) on
small inputs and store the results as fixtures.  The translation is syntactic:

* the C preprocessor switches are resolved for a chosen set of #defines;
* `do v = a, b` / `do while (c)` / `enddo`, `if (...) then` / `elseif` / `else` /
  `endif` and one-line `if (...) stmt` become Python blocks; OpenMP directives, I/O and
  comments are dropped; `real(kind=8), parameter :: X = expr` inside a body becomes
  `X = expr`;
* declarations of local arrays allocate zero arrays large enough for their Fortran index
  ranges (indices are used as written); dummy arguments are bound to the actual arguments
  of each call, and after a call the actual arguments that are variables receive the
  dummies' final values (Fortran passes by reference);
* `1.0d0` literals become Python floats, `dble`/`dsqrt`/`dabs` map to float/math.sqrt/abs,
  `min`/`max`/`mod`/`huge` to their Python equivalents, relational and logical operators
  map to Python's, array references `a(i,j)` become `a[i,j]`, a section `a(l:h)` becomes
  `a[l:h+1]`, and an array constructor `a = (/ ... /)` fills `a` from its lower bound.

Python evaluates + - * / left to right with one IEEE double rounding per operation and no
fused multiply-add, which is how gfortran evaluates these expressions without -ffast-math,
so the fixtures are the reference's arithmetic.
"""
import math
import re

import numpy as np

# module arrays of commondata / commondata3d that the subroutines index
ARRAYS = {"f", "f_post", "g", "g_post", "rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev", "Fx", "Fy",
          "ex", "ey", "ez", "opp", "exT", "eyT", "ezT", "oppT", "omega", "omegaT", "m", "meq", "m_post", "s",
          "fSource", "n", "neq", "q", "n_post", "up", "vp", "wp", "Tp", "un", "xp", "yp", "zp", "NuVolAvg",
          "ReVolAvg"}
LOCAL_ARRAYS = ["m", "meq", "m_post", "s", "fSource", "n", "neq", "q", "n_post", "un"]
INTRINSIC_SKIP = ("use ", "implicit ", "write", "open", "close", "stop", "print", "flush")
# `return` hands the subroutine's variables back to the caller's namespace first
RETURN = "ns.update({k: v for k, v in locals().items() if k != 'ns'}); return"


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
    """(dummy argument names, body lines) of subroutine `name`."""
    start, args = None, []
    for k, ln in enumerate(lines):
        if re.match(r"\s*subroutine\s+%s\s*\(" % re.escape(name), ln, re.I):
            head, j = ln.split("!")[0], k
            while ")" not in head:  # an argument list continued with '&'
                j += 1
                head = head.rstrip().rstrip("&") + " " + lines[j].split("!")[0].strip().lstrip("&")
            m = re.match(r"\s*subroutine\s+%s\s*\(([^)]*)\)" % re.escape(name), head, re.I)
            start = j + 1
            args = [a.strip() for a in m.group(1).split(",") if a.strip()]
            break
    if start is None:
        raise ValueError("subroutine %s not found" % name)
    for k in range(start, len(lines)):
        if re.match(r"\s*end\s+subroutine\s+%s\b" % re.escape(name), lines[k], re.I):
            body = lines[start:k]
            for c, ln in enumerate(body):  # internal procedures are compiled on their own
                if re.match(r"\s*contains\s*$", ln, re.I):
                    body = body[:c]
                    break
            return args, body
    raise ValueError("end of %s not found" % name)


def strip_comment(ln):
    if ln.lstrip().startswith("!$"):
        return ""
    # a '!' inside a string literal is not a comment
    out, quote = [], None
    for ch in ln:
        if quote:
            out.append(ch)
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        elif ch == "!":
            break
        out.append(ch)
    return "".join(out)


def join_continuations(lines):
    out, buf = [], ""
    for ln in lines:
        s = strip_comment(ln).rstrip()
        if not s.strip():
            continue
        if buf:
            s = buf + " " + s.strip().lstrip("&")
        if s.rstrip().endswith("&"):
            buf = s.rstrip()[:-1]
            continue
        buf = ""
        out.extend(split_statements(s))
    return out


def split_statements(s):
    """Statements separated by ';' outside string literals."""
    parts, cur, quote = [], "", None
    for ch in s:
        if quote:
            cur += ch
            if ch == quote:
                quote = None
            continue
        if ch in "'\"":
            quote = ch
        if ch == ";":
            parts.append(cur)
            cur = ""
            continue
        cur += ch
    parts.append(cur)
    return [p for p in parts if p.strip()]


def split_top(text, sep=","):
    parts, depth, cur = [], 0, ""
    for ch in text:
        if ch in "([":
            depth += 1
        elif ch in ")]":
            depth -= 1
        if ch == sep and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    parts.append(cur)
    return [p.strip() for p in parts]


def convert_expr(e, arrays=ARRAYS):
    e = re.sub(r"(\d+\.\d*|\d+)[dD]([+-]?\d+)", lambda m: "%se%s" % (m.group(1), m.group(2)), e)
    for a, b in ((".EQ.", "=="), (".NE.", "!="), (".GT.", ">"), (".LT.", "<"), (".GE.", ">="), (".LE.", "<="),
                 (".AND.", " and "), (".OR.", " or "), (".NOT.", " not "), (".TRUE.", "True"), (".FALSE.", "False")):
        e = re.sub(re.escape(a), b, e, flags=re.I)
    e = re.sub(r"/=", "!=", e)
    e = re.sub(r"\bdble\s*\(", "float(", e)
    e = re.sub(r"\bdsqrt\s*\(", "math.sqrt(", e)
    e = re.sub(r"\bdabs\s*\(", "abs(", e)
    e = re.sub(r"\bichar\s*\(\s*(\w+)\s*\(\s*(\w+)\s*:\s*\w+\s*\)\s*\)", r"ord(\1[(\2)-1])", e, flags=re.I)
    e = re.sub(r"\blen_trim\s*\(\s*(\w+)\s*\)", r"len(\1.rstrip())", e, flags=re.I)
    e = re.sub(r"\breal\s*\(", "_real(", e)
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
            if j < len(e) and e[j] == "(" and name in arrays:
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
    s = "".join(out)
    # Fortran sections l:h are inclusive
    return re.sub(r"\[([^\[\]:]*):([^\[\]:,]*)\]", lambda m: "[%s:(%s)+1]" % (m.group(1), m.group(2)), s)


def parse_declaration(t):
    """(dummy?, integer?, [(name, dims or None)]) of a declaration line `spec :: list`."""
    spec, rest = t.split("::", 1)
    mdim = re.search(r"dimension\s*\((.*)\)", spec, re.I)
    common = split_top(mdim.group(1)) if mdim else None
    items = []
    for part in split_top(rest):
        if not part or "=" in part:
            continue
        m = re.match(r"(\w+)\s*(\((.*)\))?$", part)
        if m:
            items.append((m.group(1), split_top(m.group(3)) if m.group(3) else common))
    return "intent" in spec.lower(), "integer" in spec.lower(), items


def is_single(t):
    spec = t.split("::", 1)[0].lower().replace(" ", "")
    return spec.startswith("real(kind=4)")


def to_python(body_lines, defines, dummies=(), overrides=None):
    overrides = overrides or {}
    lines = join_continuations(preprocess(body_lines, defines))
    # pass 1: array names (module, local, dummy)
    arrays = set(ARRAYS)
    local_alloc, local_scalars, ints, bounds, singles, local_strings = [], [], set(), {}, set(), []
    spelled = {d.lower(): d for d in dummies}  # Fortran names are case-insensitive
    for s in lines:
        t = s.strip()
        if "::" in t:
            for name, _ in parse_declaration(t)[2]:
                spelled.setdefault(name.lower(), name)
        if "::" in t and t.lower().startswith("character") and "intent" not in t.lower().split("::")[0]:
            for name, _ in parse_declaration(t)[2]:
                if name not in dummies:
                    local_strings.append(name)
            continue
        if "::" in t and "parameter" not in t.lower().split("::")[0] and not t.lower().startswith("character"):
            is_dummy, is_int, items = parse_declaration(t)
            if is_single(t):
                singles.update(n for n, _ in items)
            for name, dims in items:
                if dims is None:
                    if is_int:
                        ints.add(name)
                    if not is_dummy and name not in dummies:
                        local_scalars.append((name, is_int))
                    continue
                arrays.add(name)
                if all(d.strip() == ":" for d in dims):
                    continue  # allocatable: the allocate statement creates it
                if len(dims) == 1:
                    lo, hi = dims[0].split(":", 1) if ":" in dims[0] else ("1", dims[0])
                    bounds[name] = (lo.strip(), hi.strip())
                if not is_dummy and name not in dummies:
                    local_alloc.append((name, dims, is_int))
    py, ind = [], 1
    pad = lambda: "    " * ind
    cx = lambda e: convert_expr(e, arrays)
    lower = {}
    for name, dims, is_int in local_alloc:
        if name in LOCAL_ARRAYS:
            continue  # step work arrays come from the namespace
        shape = []
        for d in dims:
            lo, hi = d.split(":", 1) if ":" in d else ("1", d)
            shape.append("int(%s) + 1" % cx(hi))
            lower.setdefault(name, cx(lo))
        py.append(pad() + "%s = np.zeros((%s,)%s)" % (name, ", ".join(shape), ", dtype=np.int64" if is_int else ""))
    # Fortran locals start undefined; outputs of calls must exist before the call
    for name, is_int in local_scalars:
        py.append(pad() + "%s = %s" % (name, "0" if is_int else "0.0"))
    for name in local_strings:
        py.append(pad() + "%s = ''" % name)
    # module scalars the body assigns are locals of the Python function: start them from the
    # module's values (a statement like `x = x + 1` reads them first)
    declared = {n for n, _ in local_scalars} | set(dummies) | arrays
    assigned = []
    for s in lines:
        m = re.match(r"^\s*(?:if\s*\(.*\)\s*)?(\w+)\s*=(?!=)", s.strip(), re.I)
        if m and m.group(1) not in declared and m.group(1) not in assigned and m.group(1).lower() not in ("do", "if"):
            assigned.append(m.group(1))
    for name in assigned:
        py.append(pad() + "if %r in ns: %s = ns[%r]" % (name, name, name))
    local_names = ({n for n, _ in local_scalars} | set(dummies) | set(assigned)) - arrays

    def assignment(stmt):
        """`name = expr` with an integer target truncates like Fortran's integer assignment."""
        m = re.match(r"^(\w+)\s*=(?!=)\s*(.+)$", stmt)
        if m and m.group(1) in ints:
            return "%s = int(%s)" % (m.group(1), cx(m.group(2)))
        return cx(stmt)

    def respell(t):
        out, quote, k = [], None, 0
        while k < len(t):
            ch = t[k]
            if quote:
                out.append(ch)
                quote = None if ch == quote else quote
                k += 1
                continue
            if ch in "'\"":
                quote = ch
                out.append(ch)
                k += 1
                continue
            m = re.match(r"[A-Za-z_]\w*", t[k:])
            if m and (k == 0 or not (t[k - 1].isalnum() or t[k - 1] == "_")):
                w = m.group(0)
                out.append(spelled.get(w.lower(), w) if w.lower() not in ("if", "do", "then") else w)
                k += len(w)
                continue
            out.append(ch)
            k += 1
        return "".join(out)

    def emit(expr):
        """`write(unit) expr` of an unformatted stream: the value's bytes."""
        e = expr.strip()
        if re.match(r"^(['\"]).*\1$", e):
            return "_emit(%s, 'str')" % e
        kind = "f4" if e in singles else ("i4" if re.match(r"^-?\d+$", e) or e in ints else "auto")
        return "_emit(%s, %r)" % (cx(e), kind)

    def whole_array_reductions(t):
        # minval(a) / maxval(a) over the declared index range of a 1-D array
        return re.sub(r"\b(minval|maxval)\s*\(\s*(\w+)\s*\)",
                      lambda m: "_%s(%s, %s, %s)" % (m.group(1).lower(), m.group(2), *bounds[m.group(2)]), t)

    for s in lines:
        t = whole_array_reductions(respell(s.strip()))
        low = t.lower()
        mw = re.match(r"write\s*\(\s*(\w+)\s*\)\s*(.+)$", t, re.I)
        if mw and not mw.group(2).lstrip().startswith("("):
            py.append(pad() + emit(mw.group(2)))  # unformatted stream write
            continue
        if low.startswith(INTRINSIC_SKIP) or low.startswith("character") or "ctime(" in low:
            continue  # I/O, declarations of strings, wall-clock time stamps
        mpar = re.match(r"(real|integer)\s*\(\s*kind\s*=\s*\d\s*\)\s*,\s*parameter\s*::\s*(.+)$", t, re.I)
        if mpar:
            for item in split_top(mpar.group(2)):
                name, expr = item.split("=", 1)
                name = name.strip()
                value = repr(overrides[name]) if name in overrides else cx(expr.strip())
                py.append(pad() + "%s = %s" % (name, value))
            continue
        if "::" in t:
            continue  # declaration
        if re.match(r"return$", t, re.I):
            py.append(pad() + RETURN)
            continue
        malloc = re.match(r"allocate\s*\((.*)\)\s*$", t, re.I)
        if malloc:  # allocate(a(n1), b(n2,n3)): zero arrays indexed from 1
            for item in split_top(malloc.group(1)):
                m = re.match(r"(\w+)\s*\((.*)\)$", item)
                dims = ", ".join("int(%s) + 1" % cx(d) for d in split_top(m.group(2)))
                py.append(pad() + "%s = np.zeros((%s,))" % (m.group(1), dims))
            continue
        if re.match(r"deallocate\s*\(", t, re.I):
            continue
        mcall = re.match(r"call\s+(\w+)\s*\((.*)\)\s*$", t, re.I)
        if mcall:
            actual = split_top(mcall.group(2))

            def arg(a):
                msec = re.match(r"^(\w+)\s*\(\s*([^:,()]+)\s*:\s*([^:,()]+)\s*\)$", a)
                if msec and msec.group(1) in arrays:  # a section becomes a dummy indexed from 1
                    return "_section(%s, %s, %s)" % (msec.group(1), cx(msec.group(2)), cx(msec.group(3)))
                return cx(a)

            py.append(pad() + "_r = _call(%r, [%s])" % (mcall.group(1), ", ".join(arg(a) for a in actual)))
            for pos, a in enumerate(actual):
                # write back into this subroutine's own scalars and array elements
                melem = re.match(r"^(\w+)\s*\(([^:]*)\)$", a)
                if a in local_names:
                    py.append(pad() + "%s = _r[%d]" % (a, pos))
                elif melem and melem.group(1) in arrays:
                    py.append(pad() + "%s = _r[%d]" % (cx(a), pos))
            continue
        if re.match(r"call\s+\w+\s*$", t, re.I) or re.match(r"call\s+\w+\s*\(\s*\)\s*$", t, re.I):
            continue  # argument-less calls (macroT, ...) are run by the caller
        mwhile = re.match(r"do\s+while\s*\((.*)\)$", t, re.I)
        if mwhile:
            py.append(pad() + "while %s:" % cx(mwhile.group(1)))
            ind += 1
            py.append(pad() + "pass")
            continue
        mdo = re.match(r"do\s+(\w+)\s*=\s*(.+)$", t, re.I)
        if mdo and not re.match(r"do\s+while\b", t, re.I):
            bounds3 = split_top(mdo.group(2))
            start, stop = cx(bounds3[0]), cx(bounds3[1])
            if len(bounds3) == 3:  # do v = a, b, step
                step = cx(bounds3[2])
                py.append(pad() + "for %s in range(%s, (%s) + (1 if (%s) > 0 else -1), %s):" % (
                    mdo.group(1), start, stop, step, step))
            else:
                py.append(pad() + "for %s in range(%s, (%s) + 1):" % (mdo.group(1), start, stop))
            ind += 1
            py.append(pad() + "pass")
            continue
        if re.match(r"end\s*do$", t, re.I):
            ind -= 1
            continue
        mif = re.match(r"if\s*\((.*)\)\s*then$", t, re.I)
        if mif:
            py.append(pad() + "if %s:" % cx(mif.group(1)))
            ind += 1
            py.append(pad() + "pass")  # blocks whose only statements (I/O, stop) were dropped
            continue
        melif = re.match(r"else\s*if\s*\((.*)\)\s*then$", t, re.I)
        if melif:
            ind -= 1
            py.append(pad() + "elif %s:" % cx(melif.group(1)))
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
        mctor = re.match(r"(\w+)\s*=\s*\(/(.*)/\)$", t)
        if mctor:
            items = split_top(mctor.group(2))
            lo = lower.get(mctor.group(1), "1")
            py.append(pad() + "%s[%s:%s + %d] = [%s]" % (mctor.group(1), lo, lo, len(items),
                                                       ", ".join(cx(i) for i in items)))
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
            if stmt.lower().startswith(INTRINSIC_SKIP):
                continue
            if re.match(r"return$", stmt, re.I):
                py.append(pad() + "if %s: %s" % (cx(cond), RETURN))
                continue
            py.append(pad() + "if %s: %s" % (cx(cond), assignment(stmt)))
            continue
        py.append(pad() + assignment(t))
    return py


def compile_subroutine(src_lines, name, defines, overrides=None):
    args, body = extract(src_lines, name)
    code = ["def %s(ns):" % name, "    globals().update(ns)"]
    code += ["    %s = ns.get('%s')" % (a, a) for a in sorted(ARRAYS)]
    code += ["    %s = ns['%s']" % (a, a) for a in args]
    code += to_python(body, defines, dummies=args, overrides=overrides)
    code += ["    ns.update({k: v for k, v in locals().items() if k != 'ns'})"]
    return args, "\n".join(code)


def _huge(x):
    return 1.7976931348623157e308


class ReferenceSubroutines:
    """Subroutines of one reference file, executable on a namespace of module variables
    (scalars and numpy arrays indexed with the Fortran bounds)."""

    NAMES = ("collision", "streaming", "bounceback", "macro", "collisionT", "streamingT", "bouncebackT", "macroT")

    def __init__(self, path, defines, extra=(), overrides=None):
        self.src = open(path, encoding="utf-8-sig").read().splitlines()
        self.defines = defines
        self.overrides = overrides or {}
        self.source = {}
        self.fn = {}
        self.args = {}
        self.module = None
        self.stream = []  # bytes written by `write(unit) value` statements
        for name in self.NAMES + tuple(extra):
            self.add(name)

    def _emit(self, value, kind):
        import struct
        if kind == "str":
            self.stream.append(value.encode("ascii"))
        elif kind == "f4":
            self.stream.append(struct.pack("<f", value))
        elif kind == "i4" or (kind == "auto" and isinstance(value, (int, np.integer))):
            self.stream.append(struct.pack("<i", int(value)))
        else:
            self.stream.append(struct.pack("<d", float(value)))

    def take_stream(self):
        out, self.stream = b"".join(self.stream), []
        return out

    def add(self, name):
        args, code = compile_subroutine(self.src, name, self.defines, self.overrides)
        self.source[name] = code
        self.args[name] = args
        glb = {"math": math, "np": np, "min": min, "max": max, "mod": lambda a, b: int(math.fmod(a, b)),
               "sin": math.sin, "cos": math.cos,
               "_minval": lambda a, lo, hi: min(a[lo:hi + 1]), "_maxval": lambda a, lo, hi: max(a[lo:hi + 1]),
               "huge": _huge, "ctime": lambda *a: "", "time": lambda *a: 0, "_call": self._call,
               "_emit": self._emit, "adjustl": lambda x: x, "trim": lambda x: x,
               "nint": lambda x: int(math.copysign(math.floor(abs(x) + 0.5), x)), "_real": lambda x, kind=4: np.float32(x) if kind == 4 else float(x),
               "_section": lambda a, lo, hi: np.concatenate(([0.0], a[lo:hi + 1]))}
        exec(code, glb)
        self.fn[name] = glb[name]

    def _call(self, name, actual):
        if name not in self.fn:
            self.add(name)
        ns = dict(self.module)
        ns.update(zip(self.args[name], actual))
        self.fn[name](ns)
        self.last_ns = ns
        return [ns[a] for a in self.args[name]]

    def run(self, name, ns):
        for a in LOCAL_ARRAYS:
            ns.setdefault(a, np.zeros(32))
        if name not in self.fn:
            self.add(name)
        self.module = ns
        self.fn[name](ns)

    def step(self, ns):
        for name in self.NAMES:
            self.run(name, ns)
