"""The Fortran ISO_C_BINDING module (shipped as source; no Fortran compiler in the build
image) against the C header: every bound name is a declared C function, the derived types
list the C structs' fields in order with matching kinds, and the integer constants equal
the header's #defines."""
import os
import re

from test_cpu_abi import ROOT, declared_functions

MOD = os.path.join(ROOT, "-2d-3d-_gb300", "fortran", "lbm_gpu_mod.F90")
HDR = os.path.join(ROOT, "include", "lbm_gpu.h")


def fortran_text():
    text = open(MOD).read()
    text = re.sub(r"!.*", "", text)            # comments
    return re.sub(r"&\s*\n\s*", " ", text)      # continuation lines


def test_bound_names_are_declared():
    names = set(re.findall(r'bind\(C,\s*name="(lbm_[A-Za-z0-9_]+)"\)', fortran_text()))
    assert len(names) >= 35
    missing = names - declared_functions()
    assert not missing, missing


def test_reference_surface_is_bound():
    names = set(re.findall(r'bind\(C,\s*name="(lbm_[A-Za-z0-9_]+)"\)', fortran_text()))
    for sub in ("initial", "collision", "streaming", "bounceback", "macro", "collisionT", "streamingT",
                "bouncebackT", "macroT", "check", "calNuRe", "RBcalc_Nu_global", "RBcalc_Nu_wall_avg",
                "SideHeatedcalc_Nu_global", "SideHeatedcalc_Nu_wall_avg", "SideHeatedcalc_umid_max",
                "RBcalc_umid_max", "backupData", "reload", "output_binary", "output_Tecplot",
                "calc_psi_vort_and_output"):
        assert "lbm_" + sub in names, sub


def c_struct_fields(name):
    text = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(\w+)\s+(.*)", decl)
        ctype, names = m.group(1), m.group(2)
        for nm in names.split(","):
            nm = nm.strip()
            arr = re.match(r"(\w+)\[(\d+)\]", nm)
            fields.append((arr.group(1) if arr else nm, ctype, int(arr.group(2)) if arr else 1))
    return fields


def fortran_type_fields(name):
    body = re.search(r"type, bind\(C\) :: %s\n(.*?)end type %s" % (name, name), fortran_text(), re.S).group(1)
    fields = []
    for line in body.strip().splitlines():
        kind, names = line.split("::")
        for nm in names.split(","):
            nm = nm.strip()
            arr = re.match(r"(\w+)\((\d+)\)", nm)
            fields.append((arr.group(1) if arr else nm, kind.strip(), int(arr.group(2)) if arr else 1))
    return fields


KINDS = {"int32_t": "integer(c_int32_t)", "uint64_t": "integer(c_int64_t)", "double": "real(c_double)"}


def test_derived_types_match_structs():
    for name in ("lbm_params", "lbm_nu_wall", "lbm_mid_max", "lbm_psi_summary"):
        c = c_struct_fields(name)
        f = fortran_type_fields(name)
        assert [x[0].lower() for x in c] == [x[0].lower() for x in f], name
        for (cn, ct, cc), (fn, fk, fc) in zip(c, f):
            assert KINDS[ct] == fk and cc == fc, (name, cn, ct, fk)


def test_constants_match_header():
    defines = dict(re.findall(r"#define (LBM_[A-Z0-9_]+)\s+(-?\d+)", open(HDR).read()))
    consts = re.findall(r"(LBM_[A-Z0-9_]+)\s*=\s*(-?\d+)", fortran_text())
    assert len(consts) >= 40
    for name, value in consts:
        assert name in defines and defines[name] == value, (name, value, defines.get(name))
