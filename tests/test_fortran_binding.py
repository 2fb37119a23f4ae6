"""The Fortran binding (include/wpf_gb300.f90) against the C headers and the
ctypes mirror: every C entry point has a bind(C) interface of the same name
whose arguments agree in number, passing (by value / by reference) and kind;
every C struct has a bind(C) type with the same fields in the same order and
kinds, hence the same offsets as the ctypes structures the tests use; every
status / flag constant has the same value.  Compiled with gfortran where one
exists (the reference driver is Fortran; its call sites are
wPFAW3D.f90:2249-2280)."""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
F90 = os.path.join(INC, "wpf_gb300.f90")
HEADERS = [os.path.join(INC, "wpf.h"), os.path.join(INC, "wpf_net.h")]

# C scalar type -> the iso_c_binding kind that has its size
C_KIND = {"double": "c_double", "float": "c_float", "int": "c_int", "int32_t": "c_int32_t",
          "uint32_t": "c_int32_t", "int64_t": "c_int64_t", "uint64_t": "c_int64_t"}
SIZE = {"c_double": 8, "c_float": 4, "c_int": 4, "c_int32_t": 4, "c_int64_t": 8}
OPAQUE = {"wpf_handle", "wpf_net", "void", "char", "uint16_t"}


def _c_source():
    text = "".join(open(h).read() for h in HEADERS)
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def c_functions():
    out = {}
    for m in re.finditer(r"\b(int|const char\s*\*)\s*(wpf_\w+)\s*\(([^)]*)\)\s*;", _c_source()):
        args = []
        for a in m.group(3).split(","):
            a = a.replace("const", " ").strip()
            if not a:
                continue
            depth = a.count("*")
            base = a.replace("*", " ").split()[0]
            args.append((base, depth))
        out[m.group(2)] = (m.group(1).replace(" ", ""), args)
    return out


def c_structs():
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", _c_source(), flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            base, names = decl.split(None, 1)
            fields += [(n.strip(), C_KIND[base]) for n in names.split(",")]
        out[m.group(1)] = fields
    return out


def c_defines():
    return {m.group(1): int(m.group(2))
            for m in re.finditer(r"#define\s+(WPF_\w+)\s+(-?\d+)\b", _c_source())}


def _f90():
    lines, buf = [], ""
    for raw in open(F90):
        line = raw.split("!")[0].rstrip()
        if line.endswith("&"):
            buf += line[:-1] + " "
            continue
        lines.append(re.sub(r"\s+", " ", buf + line.strip()).strip())
        buf = ""
    return [ln for ln in lines if ln]


def _decl(line):
    """'real(c_double), intent(in), optional :: a(*), b' -> (kind, attrs, [(name, array)])"""
    lhs, rhs = line.split("::")
    parts = [p.strip() for p in re.split(r",(?![^(]*\))", lhs)]
    m = re.match(r"(integer|real|type)\((\w+)\)", parts[0])
    kind = m.group(2)
    names = [(n.strip().split("(")[0], "(" in n) for n in re.split(r",(?![^(]*\))", rhs)]
    return kind, set(parts[1:]), names


def f_types():
    out, cur = {}, None
    for ln in _f90():
        m = re.match(r"type, bind\(C\) :: (\w+)", ln)
        if m:
            cur = m.group(1)
            out[cur] = []
        elif ln.startswith("end type"):
            cur = None
        elif cur and "::" in ln:
            kind, _, names = _decl(ln)
            out[cur] += [(n, kind) for n, _ in names]
    return out


def f_functions():
    out, cur = {}, None
    for ln in _f90():
        m = re.match(r"(integer\(c_int\)|type\(c_ptr\)) function (\w+)\(([^)]*)\) bind\(C, name=\"(\w+)\"\)",
                     ln)
        if m:
            cur = {"ret": m.group(1), "args": [a.strip() for a in m.group(3).split(",") if a.strip()],
                   "cname": m.group(4), "decl": {}}
            out[m.group(2)] = cur
        elif ln.startswith("end function"):
            cur = None
        elif cur and "::" in ln and not ln.startswith("import"):
            kind, attrs, names = _decl(ln)
            for n, arr in names:
                cur["decl"][n] = (kind, "value" in attrs, arr, "optional" in attrs)
    return out


def f_parameters():
    return {m.group(1): int(m.group(2))
            for m in (re.match(r"integer\(\w+\), parameter :: (WPF_\w+) = (-?\d+)$", ln) for ln in _f90())
            if m}


def test_every_entry_point_is_bound():
    cf, ff = c_functions(), f_functions()
    assert len(cf) >= 45
    assert set(cf) == set(ff), (set(cf) ^ set(ff))
    for name, (ret, cargs) in cf.items():
        f = ff[name]
        assert f["cname"] == name
        assert (ret == "int") == (f["ret"] == "integer(c_int)"), name
        assert len(f["args"]) == len(cargs), name
        for an, (base, depth) in zip(f["args"], cargs):
            kind, value, arr, optional = f["decl"][an]
            where = f"{name}({an})"
            if depth == 0:                      # scalar by value
                assert value and kind == C_KIND[base], where
            elif kind == "c_ptr" and value:     # any single pointer, passed as an address
                assert depth == 1, where
            elif kind == "c_ptr":               # a pointer the callee writes (T**)
                assert depth == 2 and not value, where
            else:                               # by reference: scalar, array or struct
                assert depth == 1 and not value and base not in OPAQUE, where
                assert kind == (base if base.startswith("wpf_") else C_KIND[base]), where
            if optional:                        # an absent optional array passes NULL
                assert arr and not value, where


def test_every_struct_matches_c_and_ctypes():
    from mizuho_edit_gb300 import capi
    cs, fs = c_structs(), f_types()
    assert set(cs) == set(fs) == {"wpf_params", "wpf_well", "wpf_solver_opts", "wpf_step_stats",
                                  "wpf_diag"}
    mirror = {"wpf_params": capi.Params, "wpf_well": capi.Well, "wpf_solver_opts": capi.SolverOpts,
              "wpf_step_stats": capi.StepStats, "wpf_diag": capi.Diag}
    ctype_kind = {C.c_double: "c_double", C.c_int32: "c_int32_t", C.c_int64: "c_int64_t"}
    for name, fields in cs.items():
        assert fields == fs[name], name
        # offsets by the C layout rules (natural alignment) equal the ctypes offsets
        st = mirror[name]
        off = 0
        for (fname, kind), (pname, ptype) in zip(fields, st._fields_):
            size = SIZE[kind]
            off = (off + size - 1) // size * size
            assert pname.rstrip("_") == fname, (name, fname, pname)
            assert ctype_kind[ptype] == kind, (name, fname)
            assert getattr(st, pname).offset == off, (name, fname)
            off += size
        assert C.sizeof(st) == (off + 7) // 8 * 8, name


def test_constants_match():
    cd, fp = c_defines(), f_parameters()
    for k, v in cd.items():
        assert fp.get(k) == v, k
    assert set(fp) == set(cd)


def test_binding_compiles(tmp_path):
    fc = shutil.which("gfortran") or shutil.which("flang") or shutil.which("flang-new")
    if not fc:
        pytest.skip("no Fortran compiler on this machine")
    r = subprocess.run([fc, "-std=f2018", "-c", F90, "-o", str(tmp_path / "wpf_gb300.o"),
                        "-J", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
