"""CPU tests of the input.ini layer: the reference parser's semantics
(lib/iniparser/cfgio_mod.f90), Fortran list-directed reads
(lib/iniparser/string_conv_mod.f90:95-99) and list-directed output records."""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

import tara_gb300 as tg
from tara_gb300.build_ext import REFERENCE


def read_d(s: str):
    v = ctypes.c_double()
    rc = tg.lib().tara_fortran_read_double(s.encode(), ctypes.byref(v))
    return rc, v.value


def read_i(s: str):
    v = ctypes.c_longlong()
    rc = tg.lib().tara_fortran_read_int(s.encode(), ctypes.byref(v))
    return rc, v.value


@pytest.mark.parametrize("text,value", [
    ("0.010d0", 0.01), ("2.0d0", 2.0), ("2.0D0", 2.0), ("0.00010d0", 1e-4), ("1e-4", 1e-4),
    ("25.0d0", 25.0), ("  7 ", 7.0), (".5", 0.5), ("5.", 5.0), ("-1.5q0", -1.5),
    ("1.0+05", 1.0e5), ("1.0-2", 1.0e-2), ("2*3.5", 3.5), ("1.0d0 # comment", 1.0),
    ("4.0,5.0", 4.0),
    # a slash ends list-directed input: the reference's "d = 3.0d0/128.0d0" reads 3.0
    ("3.0d0/128.0d0", 3.0),
])
def test_fortran_read_double(text, value):
    rc, v = read_d(text)
    assert rc == tg.TARA_OK
    assert v == value


@pytest.mark.parametrize("text", ["abc", "", "   ", ",1.0", "/", "1.0x", "1.0d", "--1"])
def test_fortran_read_double_rejects(text):
    rc, _ = read_d(text)
    assert rc == tg.TARA_ERR_INI


def test_fortran_read_double_special():
    assert math.isinf(read_d("Infinity")[1]) and math.isnan(read_d("NaN")[1])


@pytest.mark.parametrize("text,value", [("64", 64), (" 64 ! c", 64), ("+3", 3), ("-12,", -12),
                                        ("2*8", 8)])
def test_fortran_read_int(text, value):
    assert read_i(text) == (tg.TARA_OK, value)


@pytest.mark.parametrize("text", ["6.4e1", "64.0", "x", "", "12y"])
def test_fortran_read_int_rejects(text):
    assert read_i(text)[0] == tg.TARA_ERR_INI


INI = """# test input (the reference's keys)
[dimension]
dim = 2
; semicolon comment
[grid]
Nx = 64
Ny = ${Nx}
Nz = ${grid:Nx}
[length]
Lx = 2.0d0
Lx = 9.0d0
[initialProfile]
d = 3.0d0/128.0d0
[problem]
hydrotype = "screen"
[dimension]
extra = 5
[DEFAULTS]
nu = 0.010d0
"""


@pytest.fixture
def ini_path(tmp_path):
    p = tmp_path / "in.ini"
    p.write_text(INI)
    return p


def ini_get(path, sec, key):
    buf = ctypes.create_string_buffer(512)
    rc = tg.lib().tara_ini_get(str(path).encode(), sec.encode(), key.encode(), buf, 512)
    return rc, buf.value.decode()


def test_ini_sections_keys_and_interpolation(ini_path):
    assert ini_get(ini_path, "dimension", "dim") == (tg.TARA_OK, "2")
    assert ini_get(ini_path, "grid", "Ny") == (tg.TARA_OK, "64")      # ${key}
    assert ini_get(ini_path, "grid", "Nz") == (tg.TARA_OK, "64")      # ${sec:key}
    assert ini_get(ini_path, "length", "Lx") == (tg.TARA_OK, "2.0d0")  # first match wins
    assert ini_get(ini_path, "problem", "hydrotype") == (tg.TARA_OK, "screen")  # unquoted
    assert ini_get(ini_path, "dimension", "extra") == (tg.TARA_OK, "5")  # reopened section
    # DEFAULTS fallback for a missing key and for a missing section
    assert ini_get(ini_path, "resistivity", "nu") == (tg.TARA_OK, "0.010d0")
    assert ini_get(ini_path, "grid", "nu") == (tg.TARA_OK, "0.010d0")
    rc, _ = ini_get(ini_path, "grid", "missing")
    assert rc == tg.TARA_ERR_INI
    assert "Cannot find the key" in tg.last_error()[1]


def test_ini_bad_section_title(tmp_path):
    p = tmp_path / "bad.ini"
    p.write_text("[grid\nNx = 4\n")
    assert ini_get(p, "grid", "Nx")[0] == tg.TARA_ERR_INI


def record(*v):
    arr = (ctypes.c_double * len(v))(*v)
    buf = ctypes.create_string_buffer(4096)
    assert tg.lib().tara_fortran_list_record(arr, len(v), buf, 4096) == tg.TARA_OK
    return buf.value.decode()


def test_list_directed_output_style():
    assert record(1.0) == "   1.0000000000000000     "
    assert record(12.5) == "   12.500000000000000     "
    assert record(0.1) == "  0.10000000000000001     "
    assert record(1e-4) == "   1.0000000000000000E-004"
    assert record(0.0) == "   0.0000000000000000     "
    assert record(-2.5) == "  -2.5000000000000000     "
    assert record(1e20) == "   1.0000000000000000E+020"
    two = record(1.0, 2.0)
    assert two.split() == ["1.0000000000000000", "2.0000000000000000"]
    # a negative value with a 20-character F field stays separated from an E field
    assert record(0.098, -0.10000341643993921).split() == ["9.8000000000000004E-002",
                                                            "-0.10000341643993921"]


def test_run_ini_dispatch_without_gpu(tmp_path, capfd):
    L = tg.lib()
    p = tmp_path / "a.ini"
    base = ("[dimension]\ndim = {dim}\n[architecture]\narch = cpu\n[parallel]\nmode = {mode}\n"
            "[type]\ndomain = hydro\n[problem]\nhydrotype = bare\n")
    p.write_text(base.format(dim=1, mode="serial"))
    assert L.tara_run_ini(str(p).encode(), str(tmp_path / "o").encode(), 0) == tg.TARA_ERR_ARGS
    p.write_text(base.format(dim=2, mode="mpi"))
    capfd.readouterr()
    assert L.tara_run_ini(str(p).encode(), str(tmp_path / "o").encode(), 0) == tg.TARA_OK
    # src/main.f95's message, written and flushed before the call returns
    assert capfd.readouterr().out == " Under preparation. Please wait!\n"
    p.write_text("[dimension]\ndim = 2\n")  # arch missing
    assert L.tara_run_ini(str(p).encode(), str(tmp_path / "o").encode(), 0) == tg.TARA_ERR_INI
    p.write_text(base.format(dim=2, mode="serial").replace("[grid]", ""))  # no grid keys
    rc = L.tara_run_ini(str(p).encode(), str(tmp_path / "o").encode(), 0)
    assert rc == tg.TARA_ERR_INI and "Np" in tg.last_error()[1] + "particle"


def test_list_directed_output_round_trips():
    """17 significant digits: every finite REAL(8) written reads back exactly,
    through Python's float() and through the library's own Fortran reader."""
    rng = np.random.default_rng(7)
    vals = np.concatenate([rng.standard_normal(300) * 10.0 ** rng.integers(-300, 300, 300),
                           [5e-324, 2.2250738585072014e-308, 1.7976931348623157e308, -0.0, 1.0 / 3.0,
                            0.1, 123456789.125, 1e-5, 9.999999999999999e-2, 0.09999999999999999]])
    for v in vals:
        text = record(float(v)).strip()
        assert float(text.replace("E", "e")) == v, (v, text)
        out = ctypes.c_double()
        assert tg.lib().tara_fortran_read_double(text.encode(), ctypes.byref(out)) == tg.TARA_OK
        assert out.value == v, (v, text, out.value)


# the reference checkout named by TARA_REFERENCE, where one is given
REFERENCE_INI = (REFERENCE / "input.ini") if REFERENCE is not None else None


@pytest.mark.skipif(REFERENCE_INI is None or not REFERENCE_INI.exists(),
                    reason="no reference tree named by TARA_REFERENCE on this machine")
def test_reference_input_ini():
    """The reference's shipped input.ini, read where the reference tree exists:
    every key its programs read, through the same parser and list-directed reads
    (src/main.f95:26-30, src/main2css.f95:29-76).  d = 3.0d0/128.0d0 reads as
    3.0: the list-directed read stops at the slash."""
    def val(sec, key):
        rc, text = ini_get(REFERENCE_INI, sec, key)
        assert rc == tg.TARA_OK, (sec, key, tg.last_error())
        return text

    def dbl(sec, key):
        out = ctypes.c_double()
        assert tg.lib().tara_fortran_read_double(val(sec, key).encode(), ctypes.byref(out)) == tg.TARA_OK
        return out.value

    def num(sec, key):
        out = ctypes.c_longlong()
        assert tg.lib().tara_fortran_read_int(val(sec, key).encode(), ctypes.byref(out)) == tg.TARA_OK
        return out.value

    assert (num("dimension", "dim"), val("architecture", "arch"), val("parallel", "mode")) == (2, "cpu", "serial")
    assert (val("type", "domain"), val("problem", "hydrotype")) == ("hydro", "screen")
    assert (num("grid", "Nx"), num("grid", "Ny"), num("grid", "Nz"), num("particle", "Np")) == (64, 64, 64, 10)
    assert (dbl("length", "Lx"), dbl("length", "Ly"), dbl("length", "Lz")) == (2.0, 2.0, 2.0)
    assert (dbl("resistivity", "nu"), dbl("resistivity", "eta")) == (0.01, 0.0)
    assert (dbl("time", "time_min"), dbl("time", "time_max"), dbl("time", "dt")) == (0.0, 2.0, 1e-4)
    assert (dbl("initialProfile", "W0"), dbl("initialProfile", "m0"), dbl("initialProfile", "d")) == (25.0, 2.0, 3.0)
    assert dbl("initialB", "B0") == 0.0


def _g25_17(x: float) -> str:
    """gfortran's list-directed REAL(8) item built from printf conversions:
    F20.(16 - e) + 5 blanks for e in [-1, 16], else 1P E25.17 with a three-digit
    exponent; e from %.16E.  Fortran's F editing always writes the decimal
    point, also with no fraction digits (e = 16), where %.0f leaves it out."""
    if x != x or x in (float("inf"), float("-inf")):
        return " " + ("NaN" if x != x else ("Infinity" if x > 0 else "-Infinity")).rjust(25)
    e10 = 0 if x == 0.0 else int(("%.16E" % x).split("E")[1])
    if x == 0.0 or -1 <= e10 < 17:
        dec = 16 if x == 0.0 else 16 - e10
        return " " + ("%.*f" % (dec, x) + ("." if dec == 0 else "")).rjust(20) + "     "
    m, ex = ("%.16E" % x).split("E")
    ex = int(ex)
    return " " + ("%sE%s%03d" % (m, "-" if ex < 0 else "+", abs(ex))).rjust(25)


def test_list_directed_items_match_the_printf_rules():
    """The library formats each item from one correctly rounded conversion;
    over random values of every magnitude and the carry and limit cases it
    gives the same characters as the printf-based rules (17 integer digits keep
    their decimal point, as F editing writes it)."""
    assert record(1.6450126423277086e16) == "   16450126423277086.     "
    rng = np.random.default_rng(11)
    vals = list(rng.standard_normal(20000) * 10.0 ** rng.integers(-320, 308, 20000))
    vals += list(rng.standard_normal(20000) * 10.0 ** rng.integers(-3, 18, 20000))
    edge = [0.0, -0.0, 0.1, -0.1, 0.09999999999999999, 0.099999999999999999, 1.0, 9.999999999999999,
            99999999999999990.0, 1e16, 9.999999999999998e16, 1e17, -1e17, 5e-324, -5e-324,
            2.2250738585072014e-308, 1.7976931348623157e308, -1.7976931348623157e308, 0.5, 123456.78901234567,
            float("nan"), float("inf"), float("-inf")]
    for k in range(-20, 20):
        for m in (1.0, 9.999999999999999, 9.9999999999999996, 9.99999999999999999):
            edge += [m * 10.0 ** k, -m * 10.0 ** k]
    vals += edge
    for chunk in range(0, len(vals), 150):  # 150 items fit record()'s 4096-byte buffer
        part = vals[chunk:chunk + 150]
        assert record(*part) == "".join(_g25_17(float(v)) for v in part)


def test_grid_records_file_matches_the_records(tmp_path):
    """tara_write_grid_records: x outer, y inner, fields at j * nx + i, each line
    one record (checked whole on a small grid; on a grid of several 64 MB
    blocks, by its size and a sample of records at their fixed offsets)."""
    rng = np.random.default_rng(3)
    for nx, ny, nf, full in ((7, 5, 3, True), (1024, 512, 4, False)):
        xs, ys = rng.standard_normal(nx), rng.standard_normal(ny) * 1e-3
        fields = rng.standard_normal((nf, ny, nx)) * 10.0 ** rng.integers(-5, 20, (nf, ny, nx))
        path = tmp_path / f"g{nx}.dat"
        dp = ctypes.POINTER(ctypes.c_double)
        assert tg.lib().tara_write_grid_records(str(path).encode(), nx, ny, xs.ctypes.data_as(dp),
                                                ys.ctypes.data_as(dp), fields.ctypes.data_as(dp), nf) == tg.TARA_OK
        data = path.read_bytes()
        rec = 26 * (2 + nf) + 1
        assert len(data) == nx * ny * rec
        pts = [(i, j) for i in range(nx) for j in range(ny)] if full else \
            [(int(i), int(j)) for i, j in zip(rng.integers(0, nx, 300), rng.integers(0, ny, 300))] + [(0, 0), (nx - 1, ny - 1)]
        for i, j in pts:
            n = i * ny + j
            line = data[n * rec:(n + 1) * rec].decode()
            assert line == record(xs[i], ys[j], *fields[:, j, i]) + "\n"
    assert tg.lib().tara_write_grid_records(str(tmp_path / "no" / "dir.dat").encode(), 2, 2,
                                            xs.ctypes.data_as(dp), ys.ctypes.data_as(dp), None, 0) == tg.TARA_ERR_ARGS


def test_write_grid_records_python_wrapper(tmp_path):
    rng = np.random.default_rng(5)
    xs, ys = np.arange(4) * 0.5, np.arange(3) * 0.25
    f = rng.standard_normal((2, 3, 4))
    tg.write_grid_records(tmp_path / "s.dat", xs, ys, f)
    lines = (tmp_path / "s.dat").read_text().splitlines()
    assert len(lines) == 12
    assert lines[1] + "\n" == record(xs[0], ys[1], f[0, 1, 0], f[1, 1, 0]) + "\n"
    vals = np.array([[float(v) for v in ln.split()] for ln in lines])
    assert np.array_equal(vals[:, 2].reshape(4, 3), f[0].T)
    with pytest.raises(ValueError):
        tg.write_grid_records(tmp_path / "t.dat", xs, ys, f[:, :, :3])


def test_list_record_refuses_a_short_buffer():
    v = (ctypes.c_double * 3)(1.0, 2.0, 3.0)
    buf = ctypes.create_string_buffer(3 * 26)  # one byte short of the NUL
    assert tg.lib().tara_fortran_list_record(v, 3, buf, 3 * 26) == tg.TARA_ERR_ARGS
    assert buf.value == b"" and "needs 79 bytes" in tg.last_error()[1]
    buf = ctypes.create_string_buffer(3 * 26 + 1)
    assert tg.lib().tara_fortran_list_record(v, 3, buf, 3 * 26 + 1) == tg.TARA_OK
    assert len(buf.value) == 78
