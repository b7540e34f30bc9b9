"""CPU tests of libtara's C ABI: the library loads, exports every function that
include/tara.h declares, and rejects bad arguments before touching a GPU."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

import tara_gb300 as tg

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = []
    for hdr in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", hdr.read_text(), flags=re.S)
        names += re.findall(r"\b([a-z_][a-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(n for n in names if n not in {"sizeof"}))


def test_every_declared_symbol_is_exported():
    L = tg.lib()
    names = declared_functions()
    assert "derive2csh_" in names and "tara2d_step" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_fortran_symbols_use_gfortran_mangling():
    L = tg.lib()
    for n in ("derive2csh_", "ab2csh_", "derive2css_", "ab2css_", "rk42css_"):
        assert hasattr(L, n)


def test_version():
    assert b"sm_103a" in tg.lib().tara_version()


def _cfg(nx, ny):
    c = tg.Config2D()
    tg.lib().tara2d_default_config(ctypes.byref(c), nx, ny)
    return c


@pytest.mark.parametrize("nx,ny", [(88, 64), (64, 7), (3840, 64), (8192, 64), (0, 0), (64, 3), (4096 + 2048, 64)])
def test_create_rejects_bad_sizes(nx, ny):
    h = ctypes.c_void_p()
    rc = tg.lib().tara2d_create(ctypes.byref(_cfg(nx, ny)), ctypes.byref(h))
    assert rc == tg.TARA_ERR_ARGS
    assert not h.value
    assert tg.last_error()[0] == tg.TARA_ERR_ARGS


def test_create_rejects_bad_kinds():
    for field, val in (("rhs", 7), ("scheme", 5), ("precision", 9), ("lx", -1.0)):
        c = _cfg(64, 64)
        setattr(c, field, val)
        h = ctypes.c_void_p()
        assert tg.lib().tara2d_create(ctypes.byref(c), ctypes.byref(h)) == tg.TARA_ERR_ARGS


def test_dropin_bad_dims_records_error():
    w = np.zeros((64, 10), np.complex128)  # Nh inconsistent with Nx = 64
    L = tg.lib()
    ints = [ctypes.byref(ctypes.c_int(v)) for v in (64, 64, 10)]
    dbl = [ctypes.byref(ctypes.c_double(v)) for v in (0.01, 0.0)]
    p = w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    L.derive2csh_(*ints, *dbl, p, p, p, p)
    assert tg.last_error()[0] == tg.TARA_ERR_ARGS


def test_python_wrapper_raises_on_bad_args():
    with pytest.raises(tg.TaraError) as e:
        tg.fft2d_r2c(np.zeros((22, 22)))  # a factor 11: neither path takes it
    assert e.value.code == tg.TARA_ERR_ARGS


def test_finalize_without_contexts_is_ok():
    """With no drop-in context alive (nothing ran on a GPU) finalize frees
    nothing and reports success, any number of times."""
    tg.finalize()
    tg.finalize()
    assert tg.last_error()[0] == tg.TARA_OK


def test_no_silent_fallback_without_gpu():
    """With no usable GPU a valid request fails loudly (CUDA error), never
    computes on the CPU."""
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(tg.TaraError) as e:
        tg.Solver2D(64)
    assert e.value.code in (tg.TARA_ERR_CUDA, tg.TARA_ERR_NOMEM)


@pytest.mark.parametrize("cls,args", [("Solver2D", (64,)), ("Solver3D", (16,)), ("Coh2D", (64,)), ("Com2D", (64,))])
def test_failed_create_keeps_its_error_message(cls, args):
    """A create that fails after recording an error frees its half-built handle
    through the public destroy (which records success); the error code and
    message it recorded are what the caller reads back."""
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(tg.TaraError) as e:
        getattr(tg, cls)(*args)
    code, msg = tg.last_error()
    assert code == e.value.code and code in (tg.TARA_ERR_CUDA, tg.TARA_ERR_NOMEM) and msg


@pytest.mark.parametrize("name,nf", [("derive2coh_", 3), ("derive2com_", 6)])
def test_compressible_dropins_validate_before_the_gpu(name, nf):
    """Shape errors of the compressible drop-ins are recorded before any device
    call (Nh inconsistent with Nx, and a size outside the transforms' range)."""
    import numpy as np

    L = tg.lib()
    w = np.zeros((64, 10), np.complex128)
    fn = getattr(L, name)
    nout = 2 * nf if name == "derive2com_" else 6
    for nx, ny, nh in ((64, 64, 10), (88, 88, 45)):  # (88 = 8 * 11: no mixed-radix plan)
        args = [ctypes.byref(ctypes.c_int(v)) for v in (nx, ny, nh)]
        args += [ctypes.byref(ctypes.c_double(v)) for v in (3.14159265358979, 0.0)]
        args += [w.ctypes.data] * (nf + nout)
        fn(*args)
        assert tg.last_error()[0] == tg.TARA_ERR_ARGS


def test_compressible_common_views_share_the_block():
    """The three Fortran layouts of /comm/ read the same storage."""
    c = tg.coh_common()
    old = c.Lx
    c.Lx = 1.25
    assert tg.com_common().Lx == 1.25
    assert ctypes.addressof(tg.coh_common()) == ctypes.addressof(tg.com_common()) == ctypes.addressof(tg.mhd_common())
    c.Lx = old


@pytest.mark.parametrize("cls,shape,nf", [("Coh2D", (32, 17), 3), ("Com2D", (32, 17), 6),
                                          ("Solver3D", (16, 16, 9), 8)])
def test_handles_reject_states_of_another_shape(cls, shape, nf):
    """A state whose grid is not the handle's is refused before the library
    reads it (the C side copies exactly the handle's number of values)."""
    h = getattr(tg, cls).__new__(getattr(tg, cls))  # no device handle: validation only
    h._h, h.shape = None, shape
    bad = np.zeros((nf,) + tuple(s * 2 for s in shape[:-1]) + (shape[-1],), np.complex128)
    with pytest.raises(ValueError):
        h.set_state(bad)
    with pytest.raises(ValueError):
        h.set_state(np.zeros((nf,) + shape, np.complex128), hist=bad)
    with pytest.raises(ValueError):
        h.set_state(np.zeros((nf + 1,) + shape, np.complex128))
    if cls == "Solver3D":
        with pytest.raises(ValueError):
            h.set_state_real(np.zeros((8, 16, 16, 32)))  # nx = 16 for nh = 9


def test_features_need_one_scale_per_channel():
    h = tg.Solver2D.__new__(tg.Solver2D)  # no device handle: validation only
    h._h = None
    with pytest.raises(ValueError):
        h.features(0, 3, 0, scales=[1.0, 2.0])


@pytest.mark.parametrize("grid,dim,program,bad", [
    ("Nx = 88\nNy = 64\nNz = 64", 2, "tara2dHydSer", "Nx = 88"),
    ("Nx = 64\nNy = 8192\nNz = 64", 2, "tara2dHydSer", "Ny = 8192"),
    ("Nx = 64\nNy = 64\nNz = 384", 3, "tara3dMHDOMP", "Nz = 384"),
    ("Nx = 1024\nNy = 64\nNz = 64", 3, "tara3dMHDOMP", "Nx = 1024"),
])
def test_driver_refuses_unsupported_grids(tmp_path, grid, dim, program, bad):
    """The reference's input.ini may name any Nx, Ny, Nz (src/main2csh.f95:35-38);
    the `tara` driver refuses sizes its kernels do not take before touching a
    GPU, and says which sizes it takes."""
    import tara_gb300 as tg

    ini = (f"[dimension]\ndim = {dim}\n[architecture]\narch = cpu\n[parallel]\n"
           f"mode = {'serial' if dim == 2 else 'openmp'}\n[type]\ndomain = {'hydro' if dim == 2 else 'mhd'}\n"
           f"[problem]\nhydrotype = bare\n[particle]\nNp = 0\n[grid]\n{grid}\n"
           "[length]\nLx = 2.0d0\nLy = 2.0d0\nLz = 2.0d0\n[resistivity]\nnu = 0.01d0\neta = 0.0d0\n"
           "[time]\ntime_min = 0.0d0\ntime_max = 1.0d0\ndt = 0.001d0\n"
           "[initialProfile]\nW0 = 25.0d0\nm0 = 2.0d0\nd = 0.0234375d0\n")
    (tmp_path / "input.ini").write_text(ini)
    rc = tg.lib().tara_run_ini(str(tmp_path / "input.ini").encode(), str(tmp_path / "out").encode(), 1)
    code, msg = tg.last_error()
    assert rc == tg.TARA_ERR_ARGS and code == tg.TARA_ERR_ARGS
    assert program in msg and bad in msg and "powers of two" in msg
    if dim == 2:
        assert "factors are 2, 3, 5 and 7" in msg


@pytest.mark.parametrize("grid,domain,parallel", [
    ("Nx = 96\nNy = 112", "hydro", "serial"),     # factors 3 and 7
    ("Nx = 3600\nNy = 64", "hydro", "serial"),    # the longest mixed-radix length
    ("Nx = 120\nNy = 98", "hydro", "openmp"),     # compressible hydro (tara2dHydOMP)
    ("Nx = 80\nNy = 48", "mhd", "openmp"),        # compressible MHD (tara2dMHDOMP)
])
def test_driver_passes_mixed_radix_grids_to_the_solver(tmp_path, grid, domain, parallel):
    """Even lengths up to 3600 whose only prime factors are 2, 3, 5, 7 pass the
    driver's grid check for every 2D program: what follows is the solver (on a
    machine without a GPU, a device error, whose message survives the driver
    freeing its handles), never an argument error."""
    ini = (f"[dimension]\ndim = 2\n[architecture]\narch = cpu\n[parallel]\nmode = {parallel}\n[type]\n"
           f"domain = {domain}\n[problem]\nhydrotype = bare\n[particle]\nNp = 0\n[grid]\n{grid}\nNz = 64\n"
           "[length]\nLx = 2.0d0\nLy = 2.0d0\nLz = 2.0d0\n[resistivity]\nnu = 0.01d0\neta = 0.0d0\n"
           "[time]\ntime_min = 0.0d0\ntime_max = 0.0001d0\ndt = 0.0001d0\n"
           "[initialProfile]\nW0 = 25.0d0\nm0 = 2.0d0\nd = 0.0234375d0\n")
    (tmp_path / "input.ini").write_text(ini)
    tg.lib().tara_clear_error()
    rc = tg.lib().tara_run_ini(str(tmp_path / "input.ini").encode(), str(tmp_path / "out").encode(), 1)
    code, msg = tg.last_error()
    assert rc != tg.TARA_ERR_ARGS and code != tg.TARA_ERR_ARGS, msg
    assert "not supported" not in msg
    if rc != tg.TARA_OK:
        assert code == rc and msg


@pytest.mark.parametrize("prec", [tg.PREC_FP32, tg.PREC_DF64])
def test_mixed_radix_sizes_need_fp64(prec):
    """A 96 x 96 grid (factor 3) takes the mixed-radix path, which is FP64 only:
    the other precisions are refused before any device call."""
    c = _cfg(96, 96)
    c.precision = prec
    h = ctypes.c_void_p()
    assert tg.lib().tara2d_create(ctypes.byref(c), ctypes.byref(h)) == tg.TARA_ERR_ARGS
    code, msg = tg.last_error()
    assert code == tg.TARA_ERR_ARGS and "FP64" in msg


def test_mixed_radix_dropin_shape_checks():
    """The drop-ins take 96 (2^5 3) and 98 (2 7^2) but still refuse 88 (a factor 11) and odd lengths,
    recording the error before touching the arrays."""
    L = tg.lib()
    for nx, ny in ((88, 96), (96, 99)):
        nh = nx // 2 + 1
        w = np.zeros((ny, nh), np.complex128)
        ints = [ctypes.byref(ctypes.c_int(v)) for v in (nx, ny, nh)]
        dbl = [ctypes.byref(ctypes.c_double(v)) for v in (0.01, 0.0)]
        p = w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        tg.lib().tara_clear_error()
        L.derive2csh_(*ints, *dbl, p, p, p, p)
        assert tg.last_error()[0] == tg.TARA_ERR_ARGS
        assert not w.any()
