"""The C ABI from C: include/tara.h compiles as strict C11 and as C++17, a C
program links libtara.so, and a caller shaped like gfortran's implicit-interface
calls (tests/abi/fortran_caller.c: no header, all arguments by reference,
complex(8) as double _Complex) reaches the drop-ins, whose argument checks
refuse bad shapes without a GPU and leave every array untouched."""
from __future__ import annotations

import shutil
import subprocess

import pytest

from conftest import ROOT

INC = ROOT / "include"
LIBDIR = ROOT / "tara_gb300"
ABI = ROOT / "tests" / "abi"

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc is not installed")

STRICT = ["-Wall", "-Wextra", "-pedantic", "-Werror"]


def test_header_compiles_as_c11_and_cxx17(tmp_path):
    src = tmp_path / "only_header.c"
    src.write_text('#include "tara.h"\nint main(void) { return TARA_OK; }\n')
    subprocess.run(["gcc", "-std=c11", *STRICT, "-I", str(INC), "-c", str(src), "-o", str(tmp_path / "a.o")],
                   check=True)
    if shutil.which("g++"):
        cxx = tmp_path / "only_header.cpp"
        cxx.write_text('#include "tara.h"\nint main() { return tara_last_error() == TARA_OK ? 0 : 1; }\n')
        subprocess.run(["g++", "-std=c++17", *STRICT, "-I", str(INC), "-c", str(cxx), "-o", str(tmp_path / "b.o")],
                       check=True)


def test_c_and_fortran_style_callers(tmp_path):
    exe = tmp_path / "abi_check"
    subprocess.run(["gcc", "-std=c11", *STRICT, "-I", str(INC), str(ABI / "header_user.c"),
                    str(ABI / "fortran_caller.c"), "-L", str(LIBDIR), "-ltara",
                    f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
