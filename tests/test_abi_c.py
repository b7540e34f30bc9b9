"""The C ABI from C: include/tara.h compiles as strict C11 and as C++17, a C
program links libtara.so, and a caller shaped like gfortran's implicit-interface
calls (tests/abi/fortran_caller.c: no header, all arguments by reference,
complex(8) as double _Complex) reaches the drop-ins, whose argument checks
refuse bad shapes without a GPU and leave every array untouched.  On a GPU, a
compiled C program runs the reference's driver loop through the drop-ins
(tests/abi/reference_loop.c) and matches the FFTW-backed golden vectors."""
from __future__ import annotations

import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, rel_l2

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


def _build_loop(tmp_path):
    exe = tmp_path / "reference_loop"
    subprocess.run(["gcc", "-std=c11", *STRICT, str(ABI / "reference_loop.c"), "-L", str(LIBDIR),
                    "-ltara", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)], check=True)
    return exe


def test_reference_loop_program_builds(tmp_path):
    assert _build_loop(tmp_path).exists()


def _run_loop(tmp_path, exe, mode, w, steps, nu, dt):
    ny, nh = w.shape
    src, dst = tmp_path / f"{mode}_in.bin", tmp_path / f"{mode}_out.bin"
    np.ascontiguousarray(w, np.complex128).tofile(src)
    r = subprocess.run([str(exe), mode, str(2 * (nh - 1)), str(ny), str(steps), repr(nu), repr(dt),
                        str(src), str(dst)], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    return np.fromfile(dst, np.complex128).reshape(ny, nh)


@pytest.mark.gpu
def test_reference_loop_from_c_matches_golden(tmp_path, golden):
    """2000 steps of derive2csh_ + ab2csh_ + the host rotation of
    src/main2csh.f95:114-126 from a compiled C caller (config 1: 64^2, nu = 0.01,
    dt = 1e-4, the double-shear-layer initial state) within 1e-10 of the FFTW
    oracle, and one rk42css_ call within 1e-12."""
    exe = _build_loop(tmp_path)
    w = _run_loop(tmp_path, exe, "ab2", golden["ic_spec"], 2000, 0.01, 1e-4)
    assert rel_l2(w, golden["ab2_plain_2000"]) < 1e-10
    w = _run_loop(tmp_path, exe, "rk4", golden["ic_spec"], 1, 0.01, 1e-4)
    assert rel_l2(w, golden["rk42css_1"]) < 1e-12
