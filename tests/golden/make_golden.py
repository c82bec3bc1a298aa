#!/usr/bin/env python3
"""Generate the golden fixtures under tests/golden/ from the reference's source text.

Run where the reference's sources are readable, naming their 2DRB directory:

    python tests/golden/make_golden.py --ref <reference checkout>/2DRB

(or set LBM_REFERENCE_2DRB to that directory).

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
import math
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
    ap.add_argument("--ref", default=os.environ.get("LBM_REFERENCE_2DRB"),
                    help="the reference's 2DRB directory (default: $LBM_REFERENCE_2DRB)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("name the reference's 2DRB directory with --ref or LBM_REFERENCE_2DRB")
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
    make_step_fixtures(args.ref)




# ---------------------------------------------------------------------------------------
# step fixtures: the reference's own subroutines executed on small perturbed states
# ---------------------------------------------------------------------------------------
def module_constants(src_lines, module_name, defines, overrides):
    """Evaluate the `parameter` declarations of the reference's commondata module in order,
    with the lattice size and physics numbers overridden."""
    from transliterate import convert_expr, join_continuations, preprocess
    start = next(k for k, ln in enumerate(src_lines) if re.match(r"\s*module\s+%s\b" % module_name, ln, re.I))
    end = next(k for k in range(start, len(src_lines)) if re.match(r"\s*end\s+module", src_lines[k], re.I))
    lines = join_continuations(preprocess(src_lines[start + 1:end], defines))
    ns = {"math": math}
    for s in lines:
        m = re.match(r".*parameter\s*::\s*(.+)$", s, re.I)
        if not m:
            continue
        rhs, depth, cur, parts = m.group(1), 0, "", []
        for ch in rhs:
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            if ch == "," and depth == 0:
                parts.append(cur)
                cur = ""
            else:
                cur += ch
        parts.append(cur)
        for part in parts:
            name, expr = part.split("=", 1)
            name = name.strip()
            if name in overrides:
                ns[name] = overrides[name]
                continue
            expr = convert_expr(expr).replace("acos(", "math.acos(")
            ns[name] = eval(expr, ns)
    return ns


def lattice_tables(src_text, dim):
    def vec(name):
        if dim == 3:
            m = re.search(r"^\s*%s\s*=\s*\(/(.*?)/\)" % name, src_text, re.M)
        else:
            m = re.search(r"data\s+%s\s*/(.*?)/" % name, src_text)
        return np.array([int(x) for x in m.group(1).split(",")])
    if dim == 3:
        return {k: vec(k) for k in ("ex", "ey", "ez", "opp", "exT", "eyT", "ezT", "oppT")}
    return {"ex": vec("ex"), "ey": vec("ey")}


def make_state(dim, nx, ny, nz, consts, tables, rng):
    """A perturbed module state: near-equilibrium populations with random deviations, random
    T, consistent rho/u, random B_prev.  Arrays carry the Fortran index ranges."""
    q, qt = (19, 7) if dim == 3 else (9, 5)
    shp = (nx + 2, ny + 2, nz + 2) if dim == 3 else (nx + 2, ny + 2)
    ns = dict(consts)
    ns.update(tables)
    ns["f"] = np.zeros((q,) + shp)
    ns["f_post"] = np.zeros((q,) + shp)
    ns["g"] = np.zeros((qt,) + shp)
    ns["g_post"] = np.zeros((qt,) + shp)
    for a in ("rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev", "Fx", "Fy", "up", "vp", "wp", "Tp"):
        ns[a] = np.zeros(shp)
    if dim == 3:
        w = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
        wT = np.array([consts["omegaT0"]] + [consts["omegaT1"]] * 6)
        exs = (tables["ex"], tables["ey"], tables["ez"])
        exT = (tables["exT"], tables["eyT"], tables["ezT"])
    else:
        w = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
        wT = np.array([consts["omegaT0"]] + [consts["omegaT1"]] * 4)
        exs = (tables["ex"], tables["ey"])
        exT = (tables["ex"][:5], tables["ey"][:5])
    inner = tuple(slice(1, n + 1) for n in ((nx, ny, nz) if dim == 3 else (nx, ny)))
    ishape = tuple(s.stop - 1 for s in inner)
    rho = 1.0 + 1e-3 * rng.standard_normal(ishape)
    vel = [0.03 * rng.standard_normal(ishape) for _ in range(dim)]
    T = 0.5 * rng.uniform(-1, 1, ishape)
    for a in range(q):
        eu = sum(exs[d][a] * vel[d] for d in range(dim))
        u2 = sum(vv * vv for vv in vel)
        ns["f"][(a,) + inner] = w[a] * rho * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * u2) + 1e-4 * rng.standard_normal(ishape)
    for a in range(qt):
        eu = sum(exT[d][a] * vel[d] for d in range(dim))
        ns["g"][(a,) + inner] = wT[a] * T * (1 + 3 * eu) + 1e-4 * rng.standard_normal(ishape)
    ns["rho"][inner] = rho
    ns["u"][inner] = vel[0]
    ns["v"][inner] = vel[1]
    if dim == 3:
        ns["w"][inner] = vel[2]
    ns["T"][inner] = T
    ns["Bx_prev"][inner] = vel[0] * T + 1e-4 * rng.standard_normal(ishape)
    ns["By_prev"][inner] = vel[1] * T + 1e-4 * rng.standard_normal(ishape)
    if dim == 3:
        ns["Bz_prev"][inner] = vel[2] * T + 1e-4 * rng.standard_normal(ishape)
    return ns, inner


FIELDS_OUT = {2: ["f", "g", "rho", "u", "v", "T", "Bx_prev", "By_prev", "Fx", "Fy", "f_post", "g_post"],
              3: ["f", "g", "rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev", "f_post", "g_post"]}


RESTART_OUT = {2: ["rho", "u", "v", "T", "Bx_prev", "By_prev", "Fx", "Fy"],
               3: ["rho", "u", "v", "w", "T", "Bx_prev", "By_prev", "Bz_prev"]}


def to_fortran_layout(arr, inner, pop):
    """numpy array with Fortran index ranges -> the (nz,)ny,nx(,q) C-order layout of
    lbm_get_state (direction fastest, x next)."""
    if pop:
        sub = arr[(slice(None),) + inner]
        return np.ascontiguousarray(np.transpose(sub, tuple(range(sub.ndim - 1, 0, -1)) + (0,)))
    sub = arr[inner]
    return np.ascontiguousarray(np.transpose(sub))


def step_fixture(ref_dir, case):
    from transliterate import ReferenceSubroutines
    dim = case["dim"]
    path = os.path.join(ref_dir, "2DRB.F90" if dim == 2 else "3DRB.F90")
    src_lines = open(path, encoding="utf-8-sig").read().splitlines()
    src_text = "\n".join(src_lines)
    defines = set(case["defines"])
    over = {"nx": case["nx"], "ny": case["ny"], "Rayleigh": case["Ra"], "Prandtl": case["Pr"], "Mach": case["Mach"]}
    if "SideHeatedHa" in case["defines"]:
        # Ha and the field angle (2DRB.F90:89-90); phi = deg*(pi/180) in the reference's order
        over["Ha"] = case["Ha"]
        over["phi"] = case["phi_deg"] * (math.acos(-1.0) / 180.0)
    if dim == 3:
        over["nz"] = case["nz"]
    consts = module_constants(src_lines, "commondata3d" if dim == 3 else "commondata", defines, over)
    legacy = "EnableLegacyThermalScheme" in defines
    if dim == 3:
        consts["omegaT0"] = (1.0 - consts["paraA"]) / 7.0 if legacy else 1.0 / 4.0
        consts["omegaT1"] = (6.0 + consts["paraA"]) / 42.0 if legacy else 1.0 / 8.0
    else:
        consts["omegaT0"] = (1.0 - consts["paraA"]) / 5.0 if legacy else 1.0 / 3.0
        consts["omegaT1"] = (consts["paraA"] + 4.0) / 20.0 if legacy else 1.0 / 6.0
    tables = lattice_tables(src_text, dim)
    rng = np.random.default_rng(case["seed"])
    ns, inner = make_state(dim, case["nx"], case["ny"], case.get("nz", 1), consts, tables, rng)
    q, qt = (19, 7) if dim == 3 else (9, 5)
    ns["omega"] = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12) if dim == 3 else \
        np.array([4.0 / 9.0] + [1.0 / 9.0] * 4 + [1.0 / 36.0] * 4)
    ns["omegaT"] = np.array([consts["omegaT0"]] + [consts["omegaT1"]] * (qt - 1))
    ns["qf"], ns["qt"] = q, qt
    out = {}
    for name in FIELDS_OUT[dim]:
        out["in_" + name] = to_fortran_layout(ns[name], inner, name in ("f", "g", "f_post", "g_post"))
    subs = ReferenceSubroutines(path, defines, extra=("reconstruct_macro_from_fg",))
    for _ in range(case["steps"]):
        subs.step(ns)
    for name in FIELDS_OUT[dim]:
        out["out_" + name] = to_fortran_layout(ns[name], inner, name in ("f", "g", "f_post", "g_post"))
    diag = diagnostics(subs, ns, dim, case)
    writer_bytes, writer_meta = writers(path, defines, ns, dim, case)
    out.update(writer_bytes)
    diag["writers"] = writer_meta
    # restart from the stepped f and g: initial with loadInitField = 1 reads them and calls
    # reconstruct_macro_from_fg, whose first statement (call macroT) the translation drops
    subs.run("macroT", ns)
    subs.run("reconstruct_macro_from_fg", ns)
    for name in RESTART_OUT[dim]:
        out["rst_" + name] = to_fortran_layout(ns[name], inner, False)
    meta = {k: v for k, v in case.items() if k != "defines"}
    meta["defines"] = sorted(defines)
    meta["constants"] = {k: consts[k] for k in ("tauf", "viscosity", "diffusivity", "gBeta", "Qk", "paraA")}
    if "SideHeatedHa" in defines:
        meta["constants"]["B2sigemarho"] = consts["B2sigemarho"]
    meta["diagnostics"] = diag
    return out, meta


FINE_PER_UNIT = 20  # calc_psi_absmax_fine_spline's nFinePerUnit for the fixtures (10000 in the reference)


def writers(path, defines, ns0, dim, case):
    """The reference's Tecplot writers and stream-function post-processing on the stepped
    state: the bytes each writes (`plt_*` arrays) and the numbers it computes."""
    import copy
    from transliterate import ReferenceSubroutines
    subs = ReferenceSubroutines(path, defines, overrides={"nFinePerUnit": FINE_PER_UNIT})
    L = ns0["lengthUnit"]
    base = dict(ns0)
    base["xp"] = coords(case["nx"], L)
    base["yp"] = coords(case["ny"], L)
    if dim == 3:
        base["zp"] = coords(case["nz"], L)
    base["itc"] = 0

    def fresh():
        return {k: (copy.deepcopy(v) if isinstance(v, np.ndarray) else v) for k, v in base.items()}

    files, meta = {}, {}
    if dim == 2:
        subs.take_stream()
        subs.run("output_Tecplot", fresh())
        files["plt_fields"] = subs.take_stream()
        ns = fresh()
        subs.run("calc_psi_vort_and_output", ns)
        files["plt_psiVort"] = subs.take_stream()
        subs.module = ns
        subs._call("output_psi_center_abs", [ns["psi"]])
        meta["psi"] = {"psi_center": float(subs.last_ns["psi_center"]), "psi_abs_max": float(ns["psi_abs_max"]),
                       "x_at_max": float(ns["x_at_max"]), "y_at_max": float(ns["y_at_max"]),
                       "psi_center_abs_fine": float(ns["psi_center_abs_fine"]), "nFinePerUnit": FINE_PER_UNIT}
        inner = (slice(1, case["nx"] + 1), slice(1, case["ny"] + 1))
        arrays = {"psi_psi": to_fortran_layout(ns["psi"], inner, False),
                  "psi_vort": to_fortran_layout(ns["vort"], inner, False)}
    else:
        arrays = {}
        for name in ("write_full_fields_plt", "write_midplane_x", "write_midplane_y", "write_midplane_z",
                     "write_midplane_stream_x", "write_midplane_stream_y", "write_midplane_stream_z"):
            subs.module = fresh()
            subs.take_stream()
            subs._call(name, ["file.plt"])
            files["plt_" + name] = subs.take_stream()
    out = {k: np.frombuffer(v, dtype=np.uint8) for k, v in files.items()}
    out.update(arrays)
    return out, meta


def coords(n, L):
    """xp(0:n+1) as the reference sets it (3DRB.F90:444-465, 2DRB.F90:463-476)."""
    c = np.zeros(n + 2)
    c[n + 1] = float(n)
    for i in range(1, n + 1):
        c[i] = float(i) - 0.5
    return c / L


def diagnostics(subs, ns0, dim, case):
    """The reference's post-processing subroutines on the stepped state, each on a fresh
    copy of the module namespace; returns their results by name."""
    import copy
    L = ns0["lengthUnit"]
    base = dict(ns0)
    base["xp"] = coords(case["nx"], L)
    base["yp"] = coords(case["ny"], L)
    if dim == 3:
        base["zp"] = coords(case["nz"], L)
    base["dimensionlessTime"] = 0
    base["NuVolAvg"] = np.zeros(16)
    base["ReVolAvg"] = np.zeros(16)
    wall_keys = ("Nu_hot", "Nu_cold", "Nu_middle", "Nu_hot_max", "Nu_hot_max_position", "Nu_hot_min",
                 "Nu_hot_min_position")
    res = {}

    def run(name, *args):
        ns = {k: (copy.deepcopy(v) if isinstance(v, np.ndarray) else v) for k, v in base.items()}
        if args:
            subs.module = ns
            subs._call(name, list(args))
            return subs.last_ns
        subs.run(name, ns)
        return ns

    ns = run("calNuRe")
    res["calNuRe"] = {"Nu": float(ns["NuVolAvg"][1]), "Re": float(ns["ReVolAvg"][1])}
    for name in ("RBcalc_Nu_global", "SideHeatedcalc_Nu_global"):
        res[name] = {"Nu_global": float(run(name)["Nu_global"])}
    for name in ("RBcalc_Nu_wall_avg", "SideHeatedcalc_Nu_wall_avg"):
        ns = run(name)
        res[name] = {k: float(ns[k]) for k in wall_keys}
    vsc = base["velocityScaleCompare"]
    if dim == 2:
        for name, keys in (("SideHeatedcalc_umid_max", ("umax_fit", "y_fit", "xmid")),
                           ("RBcalc_umid_max", ("umax_fit", "y_fit", "xmid")),
                           ("SideHeatedcalc_vmid_max", ("vmax_fit", "x_fit", "ymid")),
                           ("RBcalc_vmid_max", ("vmax_fit", "x_fit", "ymid"))):
            ns = run(name)
            res[name] = {"value": float(ns[keys[0]] * ns["coef"]), "pos1": float(ns[keys[1]]), "pos2": 0.0,
                         "mid": float(ns[keys[2]])}
    else:
        for name, keys in (("calc_umid_max_common", ("umax", "yAtU", "zAtU", "targetX")),
                           ("calc_vmid_max_common", ("vmax", "xAtV", "zAtV", "targetY")),
                           ("calc_wmid_max_common", ("wmax", "xAtW", "yAtW", "targetZ"))):
            ns = run(name, "tag")
            res[name] = {"value": float(ns[keys[0]] * vsc), "pos1": float(ns[keys[1]]), "pos2": float(ns[keys[2]]),
                         "mid": float(ns[keys[3]])}
    return res


STEP_CASES = [
    dict(name="rb2d_periodic", dim=2, nx=10, ny=6, Ra=1e5, Pr=0.71, Mach=0.1 * math.sqrt(3.0), steps=4, seed=7,
         defines=["steadyFlow", "HorizontalWallsNoslip", "VerticalWallsPeriodicalU", "RayleighBenardCell",
                  "HorizontalWallsConstT", "VerticalWallsPeriodicalT", "EnableUseG"]),
    dict(name="rb2d_noslip_nog", dim=2, nx=8, ny=7, Ra=2e4, Pr=7.0, Mach=0.1, steps=2, seed=11,
         defines=["steadyFlow", "HorizontalWallsNoslip", "VerticalWallsNoslip", "RayleighBenardCell",
                  "HorizontalWallsConstT", "VerticalWallsAdiabatic"]),
    dict(name="side2d_ha", dim=2, nx=8, ny=9, Ra=1e5, Pr=0.71, Mach=0.1, steps=3, seed=12, Ha=15.0, phi_deg=30.0,
         defines=["steadyFlow", "HorizontalWallsNoslip", "VerticalWallsNoslip", "SideHeatedCell",
                  "HorizontalWallsAdiabatic", "VerticalWallsConstT", "SideHeatedHa", "EnableUseG"]),
    dict(name="rb3d_noslip", dim=3, nx=6, ny=5, nz=4, Ra=1e6, Pr=0.71, Mach=0.1 * math.sqrt(3.0), steps=3, seed=8,
         defines=["steadyFlow", "HorizontalWallsNoslip", "VerticalWallsNoslip", "SpanwiseWallsNoslip",
                  "RayleighBenardCell", "HorizontalWallsConstT", "VerticalWallsAdiabatic", "SpanwiseWallsAdiabatic",
                  "EnableUseG"]),
    dict(name="side3d_default", dim=3, nx=5, ny=6, nz=4, Ra=1e5, Pr=0.71, Mach=0.1, steps=3, seed=9,
         defines=["steadyFlow", "HorizontalWallsNoslip", "VerticalWallsNoslip", "SpanwiseWallsNoslip",
                  "SideHeatedCell", "VerticalWallsConstT", "HorizontalWallsAdiabatic", "SpanwiseWallsAdiabatic",
                  "EnableUseG"]),
    dict(name="rb3d_periodic_legacy", dim=3, nx=6, ny=5, nz=4, Ra=1e5, Pr=0.71, Mach=0.02, steps=3, seed=10,
         defines=["steadyFlow", "HorizontalWallsNoslip", "VerticalWallsPeriodicalU", "SpanwiseWallsPeriodicalU",
                  "RayleighBenardCell", "HorizontalWallsConstT", "VerticalWallsPeriodicalT",
                  "SpanwiseWallsPeriodicalT", "EnableUseG", "EnableLegacyThermalScheme"]),
]


def make_step_fixtures(ref_dir):
    import sys
    sys.path.insert(0, HERE)
    index = {}
    for case in STEP_CASES:
        out, meta = step_fixture(ref_dir, case)
        np.savez_compressed(os.path.join(HERE, "step_%s.npz" % case["name"]), **out)
        index[case["name"]] = meta
        print("wrote step_%s.npz" % case["name"])
    with open(os.path.join(HERE, "step_cases.json"), "w") as fh:
        json.dump(index, fh, indent=1)


if __name__ == "__main__":
    main()
