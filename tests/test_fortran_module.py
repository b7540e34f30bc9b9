"""include/tara.f90 (the ISO_C_BINDING module for Fortran hosts) against
include/tara.h and the built library.

Neither machine has a Fortran compiler, so the module is checked by reading:
every C function of the header other than the gfortran-mangled drop-ins has
exactly one bind(C) interface of that name; the library exports it; the result
and every dummy argument have a type and passing mode that match the C
parameter (value vs reference, handle vs array, struct by reference); and the
bind(C) derived types list the C structs' members in order with matching kinds.
Where gfortran exists, the module is also compiled and linked."""
from __future__ import annotations

import re
import shutil
import subprocess

import pytest

from conftest import ROOT

HEADER = ROOT / "include" / "tara.h"
MODULE = ROOT / "include" / "tara.f90"


# ------------------------------------------------------------------ C side
def _c_text() -> str:
    t = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    t = "\n".join(l for l in t.splitlines() if not l.lstrip().startswith("#"))
    return t.replace('extern "C" {', "").replace("}", "}\n")


def c_structs() -> dict[str, list[tuple[str, str]]]:
    out = {}
    for body, name in re.findall(r"typedef\s+struct\s+\w+\s*\{(.*?)\}\s*(\w+)\s*;", _c_text(), flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.match(r"(unsigned\s+\w+|long\s+long|\w+)\s+(.*)", decl)
            for n in m.group(2).split(","):
                fields.append((m.group(1), n.strip()))
        out[name] = fields
    return out


def c_opaque() -> set[str]:
    return set(re.findall(r"typedef\s+struct\s+(\w+)\s+\1\s*;", _c_text()))


def _c_type(decl: str, with_name: bool = True):
    """(base type, pointer depth) of a parameter or return declaration."""
    d = re.sub(r"\bconst\b", " ", decl)
    depth = d.count("*")
    words = d.replace("*", " ").split()
    if with_name:
        words = words[:-1]
    return " ".join(words), depth


def c_functions() -> dict[str, tuple[tuple[str, int], list[tuple[str, int]]]]:
    t = re.sub(r"typedef\s+struct\s+\w+\s*\{.*?\}\s*\w+\s*;", "", _c_text(), flags=re.S)
    t = re.sub(r"typedef\s+struct\s+\w+\s+\w+\s*;", "", t)
    out = {}
    for stmt in t.split(";"):
        m = re.match(r"\s*([\w\s\*]+?)\s*\b(\w+)\s*\(([^()]*)\)\s*$", stmt, flags=re.S)
        if not m:
            continue
        ret = _c_type(m.group(1), with_name=False)
        params = [] if m.group(3).strip() in ("", "void") else [_c_type(p) for p in m.group(3).split(",")]
        out[m.group(2)] = (ret, params)
    return out


# ------------------------------------------------------------------ Fortran side
def _f_text() -> str:
    t = re.sub(r"!.*", "", MODULE.read_text())
    return re.sub(r"&\s*\n\s*", " ", t)


def _decls(body: str) -> dict[str, tuple[str, set[str], bool]]:
    out = {}
    for line in body.splitlines():
        if "::" not in line:
            continue
        lhs, rhs = line.split("::", 1)
        parts = [p.strip().lower() for p in re.split(r",(?![^()]*\))", lhs)]
        spec, attrs = parts[0].replace(" ", ""), set(p.replace(" ", "") for p in parts[1:])
        for n in re.split(r",(?![^()]*\))", rhs):
            n = n.strip()
            if n:
                out[n.split("(")[0].strip().lower()] = (spec, attrs, "(" in n)
    return out


def f_interfaces() -> dict[str, tuple[str, list[str], dict]]:
    """bind name -> (result spec or 'subroutine', dummy names, declarations)."""
    t = _f_text()
    head = t.split("\ncontains", 1)[0]
    out = {}
    pat = re.compile(r"^\s*(?:(\S+)\s+function|(subroutine))\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)"
                     r"(.*?)^\s*end\s+(?:function|subroutine)", re.M | re.S)
    for m in pat.finditer(head):
        res = m.group(1).replace(" ", "").lower() if m.group(1) else "subroutine"
        dummies = [d.strip().lower() for d in m.group(4).split(",") if d.strip()]
        assert m.group(5) not in out, f"two interfaces bind {m.group(5)}"
        out[m.group(5)] = (res, dummies, _decls(m.group(6)))
    return out


def f_types() -> dict[str, list[tuple[str, str]]]:
    out = {}
    for name, body in re.findall(r"type,\s*bind\(C\)\s*::\s*(\w+)(.*?)end\s+type", _f_text(), flags=re.S | re.I):
        fields = []
        for line in body.splitlines():
            if "::" in line:
                spec, names = line.split("::")
                fields += [(spec.strip().replace(" ", "").lower(), n.strip().lower()) for n in names.split(",")]
        out[name.lower()] = fields
    return out


# ------------------------------------------------------------------ matching rules
SCALAR = {"int": "integer(c_int)", "double": "real(c_double)", "uint64_t": "integer(c_int64_t)",
          "float": "real(c_float)", "size_t": "integer(c_size_t)", "long long": "integer(c_long_long)"}
BYREF = {"double": {"real(c_double)", "complex(c_double_complex)"}, "int": {"integer(c_int)"},
         "float": {"real(c_float)"}, "long long": {"integer(c_long_long)"}, "uint64_t": {"integer(c_int64_t)"},
         "char": {"character(kind=c_char)"}}
STRUCTS = c_structs()
OPAQUE = c_opaque()


def dummy_matches(c: tuple[str, int], spec: str, attrs: set[str]) -> bool:
    base, depth = c
    value = "value" in attrs
    if "optional" in attrs and value:
        return False
    if depth == 0:
        return value and SCALAR.get(base) == spec
    if depth == 2:
        return not value and spec == "type(c_ptr)" and ("intent(out)" in attrs or "intent(inout)" in attrs)
    if value:  # a pointer by value: handles, device arrays, streams, NULL-able host arrays
        return spec == "type(c_ptr)" and (base in OPAQUE or base in ("void", "double", "float", "int"))
    if base in STRUCTS:
        return spec == f"type({base})"
    return spec in BYREF.get(base, set())


def result_matches(c: tuple[str, int], res: str) -> bool:
    base, depth = c
    if depth == 0:
        return res == "subroutine" if base == "void" else res == SCALAR.get(base)
    return res == "type(c_ptr)"


# ------------------------------------------------------------------ tests
def test_every_c_function_has_one_interface():
    funcs, ifs = c_functions(), f_interfaces()
    want = {n for n in funcs if not n.endswith("_")}
    assert "tara2d_create" in want and "tara_version" in want and len(want) > 100
    assert sorted(want - set(ifs)) == [], "C functions without a Fortran interface"
    assert sorted(set(ifs) - want) == [], "Fortran interfaces without a C function"


def test_bound_names_are_exported():
    import tara_gb300 as tg

    L = tg.lib()
    assert [n for n in f_interfaces() if not hasattr(L, n)] == []


def test_results_and_arguments_match():
    funcs, ifs = c_functions(), f_interfaces()
    bad = []
    for name, (res, dummies, decls) in ifs.items():
        cret, cparams = funcs[name]
        if not result_matches(cret, res):
            bad.append(f"{name}: result {res} for C {cret}")
        if len(dummies) != len(cparams):
            bad.append(f"{name}: {len(dummies)} dummies for {len(cparams)} C parameters")
            continue
        for d, cp in zip(dummies, cparams):
            if d not in decls:
                bad.append(f"{name}: dummy {d} undeclared")
                continue
            spec, attrs, _ = decls[d]
            if not dummy_matches(cp, spec, attrs):
                bad.append(f"{name}: dummy {d} ({spec}, {sorted(attrs)}) for C {cp}")
    assert bad == []


def test_derived_types_follow_the_c_structs():
    ft = f_types()
    assert set(ft) == set(STRUCTS), (set(ft) ^ set(STRUCTS))
    for name, cfields in STRUCTS.items():
        f = ft[name]
        assert [n for _, n in f] == [n.lower() for _, n in cfields], name
        assert [s for s, _ in f] == [SCALAR[t] for t, _ in cfields], name


def test_rules_reject_mismatches():
    """The matcher is not vacuous: wrong kinds and passing modes fail."""
    assert dummy_matches(("int", 0), "integer(c_int)", {"value"})
    assert not dummy_matches(("int", 0), "integer(c_int)", set())
    assert not dummy_matches(("double", 0), "integer(c_int)", {"value"})
    assert not dummy_matches(("tara2d", 2), "type(c_ptr)", {"value"})
    assert not dummy_matches(("double", 1), "real(c_float)", {"intent(in)"})
    assert not dummy_matches(("tara2d_config", 1), "type(tara3d_config)", {"intent(in)"})
    assert not dummy_matches(("double", 1), "real(c_double)", {"value", "optional"})
    assert not result_matches(("int", 0), "subroutine")


@pytest.mark.skipif(shutil.which("gfortran") is None, reason="no Fortran compiler on this machine")
def test_module_compiles_and_links(tmp_path):
    prog = tmp_path / "use_tara.f90"
    prog.write_text("program use_tara\n  use tara_gb300\n  implicit none\n"
                    "  print '(a)', tara_string(tara_version())\nend program use_tara\n")
    lib = ROOT / "tara_gb300"
    subprocess.run(["gfortran", "-std=f2018", "-Wall", "-J", str(tmp_path), str(MODULE), str(prog),
                    "-L", str(lib), "-ltara", f"-Wl,-rpath,{lib}", "-o", str(tmp_path / "use_tara")],
                   check=True, cwd=str(tmp_path))
    r = subprocess.run([str(tmp_path / "use_tara")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "sm_103a" in r.stdout
