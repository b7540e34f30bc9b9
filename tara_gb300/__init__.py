"""tara_gb300: GB300-native pseudo-spectral RHS and time steppers of TARA.

This module is a thin ctypes binding of ``libtara.so`` (the C ABI in
``include/tara.h``).  All compute runs in the library's CUDA kernels; there is
no Python or CPU fallback: importing the module without the built library, or
calling it without a GPU, raises.
"""
from __future__ import annotations

import ctypes
import math
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libtara.so"

TARA_OK = 0
TARA_ERR_ARGS = 1
TARA_ERR_CUDA = 2
TARA_ERR_NONFINITE = 3
TARA_ERR_NOMEM = 4
TARA_ERR_TIMEOUT = 5
TARA_ERR_INI = 6

RHS_PLAIN, RHS_SCREEN = 0, 1
ENS_GRAPH, ENS_PERSISTENT4, ENS_PERSISTENT8 = 0, 1, 2
SCHEME_AB2, SCHEME_RK4 = 0, 1
PREC_FP64, PREC_FP32, PREC_DF64 = 0, 1, 2

PI_R4 = float(np.float32(3.1428))  # real(8), parameter :: pi = 3.1428 (default-real literal)


class TaraError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"tara error {code}: {msg}")
        self.code = code


class Config2D(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("rhs", ctypes.c_int),
        ("scheme", ctypes.c_int), ("precision", ctypes.c_int),
        ("nu", ctypes.c_double), ("dt", ctypes.c_double), ("alpha", ctypes.c_double),
        ("lam", ctypes.c_double), ("lx", ctypes.c_double), ("ly", ctypes.c_double),
        ("kpi", ctypes.c_double), ("batch", ctypes.c_int),
    ]


class Config3D(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("defined", ctypes.c_int),
        ("kpi", ctypes.c_double), ("lx", ctypes.c_double), ("ly", ctypes.c_double),
        ("lz", ctypes.c_double), ("mu", ctypes.c_double), ("eta", ctypes.c_double),
        ("cs", ctypes.c_double), ("nu_u", ctypes.c_double), ("eta_b", ctypes.c_double),
        ("dt", ctypes.c_double),
    ]


class CohConfig(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int)] + [
        (n, ctypes.c_double) for n in ("kpi", "lx", "ly", "mux", "muy", "cs", "dt")]


class ComConfig(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("defined", ctypes.c_int)] + [
        (n, ctypes.c_double) for n in ("kpi", "lx", "ly", "mu", "eta", "cs", "kf", "a", "dt")]


class ComCommon(ctypes.Structure):
    """The 2D compressible MHD code's view of /comm/ (src/derive2com.f95:43)."""
    _fields_ = [(n, ctypes.c_double) for n in ("Lx", "Ly", "spheat", "mu", "ms", "CS", "mu_0", "eta",
                                                 "dt", "kf", "A")]


class CohCommon(ctypes.Structure):
    """The 2D compressible code's view of /comm/ (src/derive2coh.f95:30)."""
    _fields_ = [(n, ctypes.c_double) for n in ("Lx", "Ly", "mux", "muy", "ms", "CS", "dt")]


class MhdCommon(ctypes.Structure):
    """The reference's common block /comm/ (src/derive3com.f95:62) as libtara sees it."""
    _fields_ = [("iret", ctypes.c_int32), ("thread_num", ctypes.c_int32)] + [
        (n, ctypes.c_double) for n in ("time_max", "Lx", "Ly", "Lz", "dx", "dy", "dz", "spheat",
                                       "mu", "ms", "CS", "mu_0", "eta", "dt", "kf")]


class FnoConfig(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("h", "w", "ci", "c", "co", "mx", "my", "layers", "p",
                                            "max_batch", "mode")] + [("seed", ctypes.c_uint64)]


FNO_BF16, FNO_FP32, FNO_BF16_TMEM = 0, 1, 2

_lib = None


def lib() -> ctypes.CDLL:
    """Load libtara.so (built in-tree by ``__graft_entry__.build()``)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("TARA_LIB", LIB_PATH))
        if not path.exists():
            raise ImportError(f"{path} is missing: build it with __graft_entry__.build()")
        L = ctypes.CDLL(str(path))
        _declare(L)
        _lib = L
    return _lib


def _declare(L: ctypes.CDLL) -> None:
    ip, dp, vp = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
    c_int, c_double = ctypes.c_int, ctypes.c_double
    L.tara_last_error.restype = c_int
    L.tara_last_error_message.restype = ctypes.c_char_p
    L.tara_version.restype = ctypes.c_char_p
    for name in ("derive2csh_",):
        getattr(L, name).argtypes = [ip, ip, ip, dp, dp, dp, dp, dp, dp]
    L.ab2csh_.argtypes = [ip, ip, ip, dp, dp, dp, dp, dp, dp, dp]
    L.derive2css_.argtypes = [ip, ip, ip, dp, dp, dp, dp, dp, dp, dp]
    L.ab2css_.argtypes = [ip, ip, ip, dp, dp, dp, dp, dp, dp, dp, dp]
    L.rk42css_.argtypes = [ip, ip, ip, dp, dp, dp, dp, dp, dp, dp, dp]
    for name in ("derive2csh_", "ab2csh_", "derive2css_", "ab2css_", "rk42css_"):
        getattr(L, name).restype = None
    L.tara_set_css_params.argtypes = [c_double, c_double, c_double]
    L.tara_set_css_params.restype = None
    L.tara_finalize.argtypes = []
    L.tara_finalize.restype = c_int
    cfgp = ctypes.POINTER(Config2D)
    L.tara2d_default_config.argtypes = [cfgp, c_int, c_int]
    L.tara2d_default_config.restype = None
    L.tara2d_create.argtypes = [cfgp, ctypes.POINTER(vp)]
    L.tara2d_destroy.argtypes = [vp]
    L.tara2d_set_state.argtypes = [vp, dp, dp]
    L.tara2d_get_state.argtypes = [vp, dp, dp]
    L.tara2d_set_state_device.argtypes = [vp, vp, vp]
    L.tara2d_get_state_device.argtypes = [vp, vp]
    L.tara2d_step.argtypes = [vp, c_int]
    L.tara2d_step_timed.argtypes = [vp, c_int, dp, ip, dp]
    L.tara2d_rhs.argtypes = [vp, dp]
    L.tara2d_diag.argtypes = [vp, dp, dp]
    L.tara2d_synchronize.argtypes = [vp]
    L.tara2d_stream.argtypes = [vp]
    L.tara2d_stream.restype = vp
    L.tara2d_launches_per_step.argtypes = [vp]
    L.tara2d_init_random.argtypes = [vp, c_double, c_double, ctypes.c_uint64]
    L.tara_derive2csh_noalloc.argtypes = [c_int, c_int, c_double, vp, vp, vp]
    c3p = ctypes.POINTER(Config3D)
    L.tara3d_default_config.argtypes = [c3p, c_int, c_int, c_int]
    L.tara3d_default_config.restype = None
    L.tara3d_create.argtypes = [c3p, ctypes.POINTER(vp)]
    L.tara3d_destroy.argtypes = [vp]
    L.tara3d_set_state.argtypes = [vp, vp, vp]
    L.tara3d_get_state.argtypes = [vp, vp, vp]
    L.tara3d_set_state_real.argtypes = [vp, vp]
    L.tara3d_init_orszag_tang.argtypes = [vp, ctypes.c_double, c_int, ctypes.c_uint64]
    L.tara3d_step.argtypes = [vp, c_int]
    L.tara3d_rhs.argtypes = [vp, vp]
    L.tara3d_synchronize.argtypes = [vp]
    L.derive3com_.argtypes = [ip] * 4 + [dp] * 2 + [vp] * 24
    L.derive3com_.restype = None
    L.ab3com_.argtypes = [ip] * 4 + [dp] * 2 + [vp] * 32
    L.ab3com_.restype = None
    L.tara_fortran_read_double.argtypes = [ctypes.c_char_p, dp]
    L.tara_fortran_read_int.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong)]
    L.tara_ini_get.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, c_int]
    L.tara_fortran_list_record.argtypes = [dp, c_int, ctypes.c_char_p, c_int]
    L.tara_run_ini.argtypes = [ctypes.c_char_p, ctypes.c_char_p, c_int]
    L.tara3d_diag.argtypes = [vp, dp]
    L.tara3d_stream.argtypes = [vp]
    L.tara3d_stream.restype = vp
    L.tara_measure_dfma_rate.argtypes = [c_int, dp]
    L.tara_twiddle_table.argtypes = [c_int, c_int, dp, c_int, ctypes.POINTER(c_int)]
    L.tara_write_grid_records.argtypes = [ctypes.c_char_p, c_int, c_int, dp, dp, dp, c_int]
    L.tara_coh2d_default_config.argtypes = [vp, c_int, c_int]
    L.tara_coh2d_default_config.restype = None
    L.tara_coh2d_create.argtypes = [vp, vp]
    L.tara_coh2d_destroy.argtypes = [vp]
    L.tara_coh2d_set_state.argtypes = [vp, vp, vp]
    L.tara_coh2d_get_state.argtypes = [vp, vp, vp]
    L.tara_coh2d_rhs.argtypes = [vp, vp]
    L.tara_coh2d_step.argtypes = [vp, c_int]
    L.tara_coh2d_synchronize.argtypes = [vp]
    L.tara_coh2d_launches_per_step.argtypes = [vp]
    L.tara_coh2d_stream.argtypes = [vp]
    L.tara_coh2d_stream.restype = vp
    L.tara_coh2d_init_vortices.argtypes = [vp, c_double, c_double]
    L.tara_com2d_default_config.argtypes = [vp, c_int, c_int]
    L.tara_com2d_default_config.restype = None
    L.tara_com2d_create.argtypes = [vp, vp]
    L.tara_com2d_destroy.argtypes = [vp]
    L.tara_com2d_set_state.argtypes = [vp, vp, vp]
    L.tara_com2d_get_state.argtypes = [vp, vp, vp]
    L.tara_com2d_rhs.argtypes = [vp, vp]
    L.tara_com2d_step.argtypes = [vp, c_int]
    L.tara_com2d_synchronize.argtypes = [vp]
    L.tara_com2d_launches_per_step.argtypes = [vp]
    L.tara_com2d_stream.argtypes = [vp]
    L.tara_com2d_stream.restype = vp
    L.tara_com2d_init_reference.argtypes = [vp, c_double, c_double, c_double]
    L.derive2com_.argtypes = [ip, ip, ip, dp, dp] + [vp] * 18
    L.derive2com_.restype = None
    L.ab2com_.argtypes = [ip, ip, ip, dp, dp] + [vp] * 24
    L.ab2com_.restype = None
    L.derive2coh_.argtypes = [ip, ip, ip, dp, dp] + [vp] * 9
    L.derive2coh_.restype = None
    L.ab2coh_.argtypes = [ip, ip, ip, dp, dp] + [vp] * 12
    L.ab2coh_.restype = None
    L.tara2d_set_state_run.argtypes = [vp, c_int, dp, dp]
    L.tara2d_get_state_run.argtypes = [vp, c_int, dp, dp]
    L.tara2d_diag_run.argtypes = [vp, c_int, dp, dp]
    L.tara2d_init_random_run.argtypes = [vp, c_int, c_double, c_double, ctypes.c_uint64]
    L.tara_ens_create.argtypes = [c_int, vp, c_int, c_int, c_double, c_double, c_double,
                                  ctypes.POINTER(vp)]
    L.tara_ens_destroy.argtypes = [vp]
    L.tara_ens_autotune.argtypes = [vp, c_int]
    L.tara_ens_set_form.argtypes = [vp, c_int]
    L.tara_ens_form.argtypes = [vp, ip, dp]
    L.tara_ens_step.argtypes = [vp, c_int]
    L.tara_ens_synchronize.argtypes = [vp]
    L.tara_ens_stream.argtypes = [vp]
    L.tara_ens_stream.restype = vp
    L.tara_ens_get_state.argtypes = [vp, c_int, dp]
    L.tara_ens_set_state.argtypes = [vp, c_int, dp]
    L.tara_ens_diag.argtypes = [vp, c_int, dp, dp]
    L.tara_ens_groups.argtypes = [vp]
    L.tara_ens_group_info.argtypes = [vp, c_int, ip, ip, ip, dp]
    L.tara_ens_launches_per_step.argtypes = [vp]
    L.tara2d_diag_reference.argtypes = [vp, vp, dp, dp]
    L.tara2d_real_fields.argtypes = [vp, vp, dp, dp, dp, dp]
    L.tara_fft2d_r2c.argtypes = [c_int, c_int, c_int, dp, dp]
    L.tara_fft2d_c2r.argtypes = [c_int, c_int, c_int, dp, dp]
    fcp = ctypes.POINTER(FnoConfig)
    L.tara_fno_default_config.argtypes = [fcp]
    L.tara_fno_default_config.restype = None
    L.tara_fno_create.argtypes = [fcp, ctypes.POINTER(vp)]
    L.tara_fno_destroy.argtypes = [vp]
    L.tara_fno_num_params.argtypes = [vp]
    L.tara_fno_num_params.restype = ctypes.c_size_t
    fp = ctypes.POINTER(ctypes.c_float)
    L.tara_fno_get_params.argtypes = [vp, fp]
    L.tara_fno_set_params.argtypes = [vp, fp]
    L.tara_fno_get_grads.argtypes = [vp, fp]
    L.tara_fno_set_mode.argtypes = [vp, c_int]
    L.tara_fno_set_fused.argtypes = [vp, c_int]
    L.tara_fno_forward.argtypes = [vp, vp, vp, c_int]
    L.tara_fno_train_step.argtypes = [vp, vp, vp, vp, c_int, c_int, ctypes.c_float, dp]
    L.tara_fno_adam_steps.argtypes = [vp]
    L.tara_fno_adam_steps.restype = ctypes.c_longlong
    L.tara_fno_stream.argtypes = [vp]
    L.tara_fno_stream.restype = vp
    L.tara2d_filter.argtypes = [vp, c_int, c_int, vp, vp, vp]
    L.tara_particles_create.argtypes = [vp, c_double, c_double, c_double, c_int, dp, dp, ctypes.POINTER(vp)]
    L.tara_particles_destroy.argtypes = [vp]
    L.tara_particles_advance.argtypes = [vp, c_double]
    L.tara_particles_get.argtypes = [vp, dp, dp]
    L.tara_park_miller_rand.argtypes = [ctypes.POINTER(ctypes.c_uint64)]
    L.tara_park_miller_rand.restype = ctypes.c_float
    L.tara2d_autotune.argtypes = [vp, c_int, ip, dp]
    L.tara2d_set_variants.argtypes = [vp, ip]
    L.tara2d_set_state_real_device.argtypes = [vp, c_int, vp]
    L.tara2d_spectrum.argtypes = [vp, c_int, c_int, dp]
    L.tara_closure_create.argtypes = [vp, vp, dp, c_double, ctypes.POINTER(vp)]
    L.tara2d_features.argtypes = [vp, c_int, c_int, dp, vp]
    L.tara_closure_augment.argtypes = [vp, vp, c_int, c_int, c_int, vp, vp]
    L.tara_closure_destroy.argtypes = [vp]
    L.tara_closure_step.argtypes = [vp, c_int]


def _check(rc: int) -> None:
    if rc != TARA_OK:
        raise TaraError(rc, lib().tara_last_error_message().decode())


def last_error() -> tuple[int, str]:
    L = lib()
    return L.tara_last_error(), L.tara_last_error_message().decode()


def _dp(a: np.ndarray):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _as_spectrum(a: np.ndarray, nh: int, ny: int) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if a.shape != (ny, nh):
        raise ValueError(f"expected a ({ny}, {nh}) half spectrum, got {a.shape}")
    return a


# ---------------------------------------------------------------------------
# Fortran drop-ins, called exactly as the reference's callers call them
# ---------------------------------------------------------------------------
def _ints(*v):
    return [ctypes.byref(ctypes.c_int(int(x))) for x in v]


def _dbls(*v):
    return [ctypes.byref(ctypes.c_double(float(x))) for x in v]


def derive2csh(omegak: np.ndarray, nu: float, time: float = 0.0) -> np.ndarray:
    """subroutine derive2csh (src/derive2csh.f95:3): returns dt_omegak_new.
    ``omegak`` is (Ny, Nh) complex: row ky, column kx (Fortran omegak(Nh,Ny))."""
    ny, nh = omegak.shape
    nx = 2 * (nh - 1)
    w = _as_spectrum(omegak, nh, ny).copy()
    out = np.zeros_like(w)
    dummy = np.zeros_like(w)
    lib().derive2csh_(*_ints(nx, ny, nh), *_dbls(nu, time), _dp(w.view(np.float64)),
                      _dp(dummy.view(np.float64)), _dp(dummy.view(np.float64)),
                      _dp(out.view(np.float64)))
    _check(lib().tara_last_error())
    return out


def derive2css(omegak: np.ndarray, alpha: float, nu: float, time: float = 0.0) -> np.ndarray:
    """subroutine derive2css (src/derive2css.f95:6), defined mode."""
    ny, nh = omegak.shape
    nx = 2 * (nh - 1)
    w = _as_spectrum(omegak, nh, ny).copy()
    out = np.zeros_like(w)
    dummy = np.zeros_like(w)
    lib().derive2css_(*_ints(nx, ny, nh), *_dbls(alpha, nu, time), _dp(w.view(np.float64)),
                      _dp(dummy.view(np.float64)), _dp(dummy.view(np.float64)),
                      _dp(out.view(np.float64)))
    _check(lib().tara_last_error())
    return out


def ab2csh(omegak, dt_omegak_old, dt_omegak_new, dt: float, nu: float = 0.0, time: float = 0.0):
    """subroutine ab2csh (src/ab2csh.f95:3): returns omegak_new."""
    ny, nh = omegak.shape
    nx = 2 * (nh - 1)
    w = _as_spectrum(omegak, nh, ny)
    fo = _as_spectrum(dt_omegak_old, nh, ny)
    fn = _as_spectrum(dt_omegak_new, nh, ny)
    out = np.zeros_like(w)
    lib().ab2csh_(*_ints(nx, ny, nh), *_dbls(nu, time, dt), _dp(w.view(np.float64)),
                  _dp(out.view(np.float64)), _dp(fo.view(np.float64)), _dp(fn.view(np.float64)))
    _check(lib().tara_last_error())
    return out


def rk42css(omegak, alpha: float, nu: float, dt: float, time: float = 0.0):
    """subroutine rk42css (src/rk42css.f95:6) as a working classic RK4 step."""
    ny, nh = omegak.shape
    nx = 2 * (nh - 1)
    w = _as_spectrum(omegak, nh, ny).copy()
    out = np.zeros_like(w)
    dummy = np.zeros_like(w)
    lib().rk42css_(*_ints(nx, ny, nh), *_dbls(alpha, nu, time, dt), _dp(w.view(np.float64)),
                   _dp(out.view(np.float64)), _dp(dummy.view(np.float64)),
                   _dp(dummy.view(np.float64)))
    _check(lib().tara_last_error())
    return out


def set_css_params(lx: float, ly: float, lam: float) -> None:
    lib().tara_set_css_params(lx, ly, lam)


def finalize() -> None:
    """Free the device contexts the Fortran drop-ins keep per grid shape
    (tara_finalize); the next drop-in call creates them again."""
    _check(lib().tara_finalize())


def measure_dfma_rate(reps: int = 5) -> float:
    """FP64 FMA thread-instructions per second measured on the current device."""
    v = ctypes.c_double()
    _check(lib().tara_measure_dfma_rate(int(reps), ctypes.byref(v)))
    return v.value


def write_grid_records(path, xs, ys, fields) -> None:
    """A snapshot file in the reference drivers' fort.* format: one record per
    grid point (x outer, y inner) of xs[i], ys[j] and fields[k][j, i]
    (tara_write_grid_records; fields: (nfields, Ny, Nx) real arrays)."""
    xs = np.ascontiguousarray(xs, np.float64)
    ys = np.ascontiguousarray(ys, np.float64)
    f = np.ascontiguousarray(fields, np.float64)
    if f.ndim == 2:
        f = f[None]
    if f.shape[1:] != (ys.size, xs.size):
        raise ValueError(f"fields of shape {f.shape} do not match Ny = {ys.size}, Nx = {xs.size}")
    dptr = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    _check(lib().tara_write_grid_records(str(path).encode(), xs.size, ys.size, dptr(xs), dptr(ys), dptr(f),
                                         f.shape[0]))


def twiddle_table(n: int, precision: int = PREC_FP64) -> np.ndarray:
    """The transforms' twiddle table of length n as the device reads it, (count, 2)
    doubles (tara_twiddle_table; host only)."""
    cnt = ctypes.c_int()
    _check(lib().tara_twiddle_table(int(n), int(precision), None, 0, ctypes.byref(cnt)))
    out = np.zeros((cnt.value, 2))
    _check(lib().tara_twiddle_table(int(n), int(precision), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                    cnt.value, ctypes.byref(cnt)))
    return out


def fft2d_r2c(x: np.ndarray, precision: int = PREC_FP64) -> np.ndarray:
    """Unnormalised r2c of a real (Ny, Nx) field -> (Ny, Nh) complex (FFTW semantics)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    ny, nx = x.shape
    out = np.zeros((ny, nx // 2 + 1), np.complex128)
    _check(lib().tara_fft2d_r2c(nx, ny, precision, _dp(x), _dp(out.view(np.float64))))
    return out


def fft2d_c2r(c: np.ndarray, precision: int = PREC_FP64) -> np.ndarray:
    """Unnormalised c2r of a (Ny, Nh) half spectrum -> real (Ny, Nx) (FFTW semantics)."""
    c = np.ascontiguousarray(c, dtype=np.complex128)
    ny, nh = c.shape
    nx = 2 * (nh - 1)
    out = np.zeros((ny, nx), np.float64)
    _check(lib().tara_fft2d_c2r(nx, ny, precision, _dp(c.view(np.float64)), _dp(out)))
    return out


# ---------------------------------------------------------------------------
# Device-resident solver
# ---------------------------------------------------------------------------
class Solver2D:
    """Owns a tara2d handle: state in HBM, steps on the library's CUDA stream."""

    def __init__(self, nx: int, ny: int | None = None, *, rhs: int = RHS_PLAIN,
                 scheme: int = SCHEME_AB2, precision: int = PREC_FP64, nu: float = 0.01,
                 dt: float = 1e-4, alpha: float = 1.0, lam: float = 10.0,
                 lx: float | None = None, ly: float | None = None, kpi: float = PI_R4,
                 batch: int = 1):
        ny = nx if ny is None else ny
        cfg = Config2D()
        lib().tara2d_default_config(ctypes.byref(cfg), nx, ny)
        cfg.rhs, cfg.scheme, cfg.precision = rhs, scheme, precision
        cfg.batch = batch
        cfg.nu, cfg.dt, cfg.alpha, cfg.lam = nu, dt, alpha, lam
        cfg.kpi = kpi
        cfg.lx = 2.0 * kpi if lx is None else lx
        cfg.ly = 2.0 * kpi if ly is None else ly
        h = ctypes.c_void_p()
        _check(lib().tara2d_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.nx, self.ny, self.nh = nx, ny, nx // 2 + 1
        self.cfg = cfg

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().tara2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def launches_per_step(self) -> int:
        return lib().tara2d_launches_per_step(self._h)

    def set_state(self, omegak: np.ndarray, dt_old: np.ndarray | None = None) -> None:
        w = _as_spectrum(omegak, self.nh, self.ny)
        fo = None if dt_old is None else _as_spectrum(dt_old, self.nh, self.ny)
        _check(lib().tara2d_set_state(self._h, _dp(w.view(np.float64)),
                                      None if fo is None else _dp(fo.view(np.float64))))

    def get_state(self, with_history: bool = False):
        w = np.zeros((self.ny, self.nh), np.complex128)
        fo = np.zeros_like(w) if with_history else None
        _check(lib().tara2d_get_state(self._h, _dp(w.view(np.float64)),
                                      None if fo is None else _dp(fo.view(np.float64))))
        return (w, fo) if with_history else w

    def get_state_into(self, out: np.ndarray) -> None:
        """Copy the state into a caller-owned (Ny, Nh) complex128 array (e.g. pinned)."""
        if out.shape != (self.ny, self.nh) or out.dtype != np.complex128 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous (Ny, Nh) complex128 array")
        _check(lib().tara2d_get_state(self._h, _dp(out.view(np.float64)), None))

    def set_state_device(self, ptr: int, dt_old_ptr: int | None = None) -> None:
        _check(lib().tara2d_set_state_device(self._h, ctypes.c_void_p(ptr),
                                             ctypes.c_void_p(dt_old_ptr) if dt_old_ptr else None))

    def get_state_device(self, ptr: int) -> None:
        _check(lib().tara2d_get_state_device(self._h, ctypes.c_void_p(ptr)))

    def step(self, n: int = 1) -> None:
        _check(lib().tara2d_step(self._h, int(n)))

    KERNELS = ("k_col_inverse", "k_row_nl", "k_col_forward")

    def step_timed(self, n: int) -> dict:
        """Run n steps with CUDA events between launches; per-kernel-kind totals."""
        ms = (ctypes.c_double * 3)()
        cnt = (ctypes.c_int * 3)()
        tot = ctypes.c_double()
        _check(lib().tara2d_step_timed(self._h, int(n), ms, cnt, ctypes.byref(tot)))
        return {"total_ms": tot.value,
                "kernels": {k: {"ms": ms[i], "launches": cnt[i]} for i, k in enumerate(self.KERNELS)}}

    def rhs(self) -> np.ndarray:
        out = np.zeros((self.ny, self.nh), np.complex128)
        _check(lib().tara2d_rhs(self._h, _dp(out.view(np.float64))))
        return out

    def diag(self) -> tuple[float, float]:
        e, z = ctypes.c_double(), ctypes.c_double()
        _check(lib().tara2d_diag(self._h, ctypes.byref(e), ctypes.byref(z)))
        return e.value, z.value

    def synchronize(self) -> None:
        _check(lib().tara2d_synchronize(self._h))

    @property
    def stream(self) -> int:
        return lib().tara2d_stream(self._h) or 0

    def init_random(self, k0: float, energy: float, seed: int, run: int = 0) -> None:
        _check(lib().tara2d_init_random_run(self._h, run, k0, energy, seed))

    def autotune(self, trial_steps: int = 3) -> dict:
        """Pick the fastest tile variant per step kernel (state restored)."""
        v = (ctypes.c_int * 3)()
        ms = (ctypes.c_double * 24)()
        _check(lib().tara2d_autotune(self._h, int(trial_steps), v, ms))
        # per-launch ms in context: rows are the configurations 0-7 (tile variant +
        # 4 for the radix-8 path), columns the three kernels; 0 = not available
        return {"variants": list(v), "ms": [list(ms[3 * i:3 * i + 3]) for i in range(8)]}

    def set_variants(self, variants) -> None:
        v = (ctypes.c_int * 3)(*[int(x) for x in variants])
        _check(lib().tara2d_set_variants(self._h, v))

    def get_state_run(self, run: int) -> np.ndarray:
        w = np.zeros((self.ny, self.nh), np.complex128)
        _check(lib().tara2d_get_state_run(self._h, run, _dp(w.view(np.float64)), None))
        return w

    def set_state_run(self, run: int, omegak: np.ndarray) -> None:
        w = _as_spectrum(omegak, self.nh, self.ny)
        _check(lib().tara2d_set_state_run(self._h, run, _dp(w.view(np.float64)), None))

    def diag_run(self, run: int) -> tuple[float, float]:
        e, z = ctypes.c_double(), ctypes.c_double()
        _check(lib().tara2d_diag_run(self._h, run, ctypes.byref(e), ctypes.byref(z)))
        return e.value, z.value

    def filter(self, run: int, factor: int, omega_bar=0, flux=0, omega_bar64=0) -> None:
        """Box filter onto the grid coarsened by ``factor``; device pointers
        (FP32 omega_bar, FP32 (.., 2) flux, FP64 omega_bar64), 0 to skip."""
        _check(lib().tara2d_filter(self._h, run, factor, ctypes.c_void_p(omega_bar or None),
                                   ctypes.c_void_p(flux or None), ctypes.c_void_p(omega_bar64 or None)))

    def features(self, run: int, nf: int, out_ptr: int, scales=None) -> None:
        """Closure input features (FP32 (Ny, Nx, nf)) of run `run` at a device pointer."""
        sc = None if scales is None else np.ascontiguousarray(np.asarray(scales, np.float64))
        if sc is not None and sc.size < nf:
            raise ValueError(f"expected {nf} feature scales, got {sc.size}")
        _check(lib().tara2d_features(self._h, run, nf, None if sc is None else _dp(sc),
                                     ctypes.c_void_p(out_ptr)))

    def set_state_real_device(self, run: int, ptr: int) -> None:
        _check(lib().tara2d_set_state_real_device(self._h, run, ctypes.c_void_p(ptr)))

    def spectrum(self, run: int = 0, kmax: int | None = None) -> np.ndarray:
        kmax = self.nx // 2 if kmax is None else kmax
        out = np.zeros(kmax + 1)
        _check(lib().tara2d_spectrum(self._h, run, kmax, _dp(out)))
        return out


# ---------------------------------------------------------------------------
# 3D compressible MHD
# ---------------------------------------------------------------------------
def mhd_common() -> MhdCommon:
    """libtara's view of the Fortran common block /comm/ (read by derive3com_/ab3com_)."""
    return MhdCommon.in_dll(lib(), "comm_")


def _state8(a, shape=None) -> np.ndarray:
    """Eight 3D half spectra, C-contiguous complex128; `shape` = (Nz, Ny, Nh) of the
    handle they go to (the library reads exactly that many values)."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if a.ndim != 4 or a.shape[0] != 8 or (shape is not None and a.shape[1:] != tuple(shape)):
        raise ValueError(f"expected an (8, Nz, Ny, Nh) state{'' if shape is None else ' of ' + str(tuple(shape))}, "
                         f"got {a.shape}")
    return a


def derive3com(state, pi: float = 3.14159265358979323846, time: float = 0.0) -> np.ndarray:
    """subroutine derive3com (src/derive3com.f95:6): the eight d_*_k_dt_new arrays."""
    st = _state8(state)
    _, nz, ny, nh = st.shape
    out = np.zeros_like(st)
    old = np.zeros_like(st[0])
    args = []
    for f in range(8):
        args += [old.ctypes.data, out[f].ctypes.data]
    lib().derive3com_(*_ints(2 * (nh - 1), ny, nz, nh), *_dbls(pi, time),
                      *[st[f].ctypes.data for f in range(8)], *args)
    _check(lib().tara_last_error())
    return out


def ab3com(state, d_old, d_new, pi: float = 3.14159265358979323846, time: float = 0.0):
    """subroutine ab3com (src/ab3com.f95:6): the eight *_k_new arrays (dt from /comm/)."""
    st, do, dn = _state8(state), _state8(d_old), _state8(d_new)
    _, nz, ny, nh = st.shape
    out = np.zeros_like(st)
    pairs = []
    for f in range(8):
        pairs += [do[f].ctypes.data, dn[f].ctypes.data]
    lib().ab3com_(*_ints(2 * (nh - 1), ny, nz, nh), *_dbls(pi, time),
                  *[st[f].ctypes.data for f in range(8)], *[out[f].ctypes.data for f in range(8)],
                  *pairs)
    _check(lib().tara_last_error())
    return out


class Solver3D:
    """Device-resident 3D MHD state (tara3d handle)."""

    def __init__(self, nx: int, ny: int | None = None, nz: int | None = None, **kw):
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        cfg = Config3D()
        lib().tara3d_default_config(ctypes.byref(cfg), nx, ny, nz)
        for k, v in kw.items():
            setattr(cfg, k, v)
        h = ctypes.c_void_p()
        _check(lib().tara3d_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.shape = (nz, ny, nx // 2 + 1)
        self.cfg = cfg

    def close(self):
        if getattr(self, "_h", None):
            lib().tara3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, state, hist=None):
        st = _state8(state, self.shape)
        h = None if hist is None else _state8(hist, self.shape)
        _check(lib().tara3d_set_state(self._h, st.ctypes.data, None if h is None else h.ctypes.data))

    def set_state_real(self, real8):
        r = np.ascontiguousarray(real8, dtype=np.float64)
        nz, ny, nh = self.shape
        if r.shape != (8, nz, ny, 2 * (nh - 1)):
            raise ValueError(f"expected an (8, {nz}, {ny}, {2 * (nh - 1)}) real state, got {r.shape}")
        _check(lib().tara3d_set_state_real(self._h, r.ctypes.data))

    def init_orszag_tang(self, amp: float = 0.01, kmax: int = 4, seed: int = 3):
        """The 3D MHD benchmark's initial state (tara3d_init_orszag_tang): rho = 1,
        u = (-sin y, sin x, 0), B = (-sin y, sin 2x, 0), each plus a seeded
        random-phase solenoidal perturbation of relative r.m.s. `amp` on the modes
        0 < |k| <= kmax; E = 1 + |u|^2/2 + |B|^2/2; zero history."""
        _check(lib().tara3d_init_orszag_tang(self._h, float(amp), int(kmax), int(seed)))

    def get_state(self, with_history: bool = False):
        st = np.zeros((8,) + self.shape, np.complex128)
        h = np.zeros_like(st) if with_history else None
        _check(lib().tara3d_get_state(self._h, st.ctypes.data, None if h is None else h.ctypes.data))
        return (st, h) if with_history else st

    def step(self, n: int = 1):
        _check(lib().tara3d_step(self._h, int(n)))

    def rhs(self):
        out = np.zeros((8,) + self.shape, np.complex128)
        _check(lib().tara3d_rhs(self._h, out.ctypes.data))
        return out

    def synchronize(self):
        _check(lib().tara3d_synchronize(self._h))

    @property
    def stream(self) -> int:
        return lib().tara3d_stream(self._h) or 0

    def diag(self):
        out = (ctypes.c_double * 4)()
        _check(lib().tara3d_diag(self._h, out))
        return list(out)


# ---------------------------------------------------------------------------
# 2D compressible isothermal hydro
# ---------------------------------------------------------------------------
def coh_common() -> CohCommon:
    """libtara's /comm/ seen with the 2D compressible layout (read by derive2coh_/ab2coh_)."""
    return CohCommon.from_address(ctypes.addressof(MhdCommon.in_dll(lib(), "comm_")))


def _state3(a, shape=None) -> np.ndarray:
    """(nk, ukx, uky) half spectra; `shape` = (Ny, Nh) of the handle they go to."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if a.ndim != 3 or a.shape[0] != 3 or (shape is not None and a.shape[1:] != tuple(shape)):
        raise ValueError(f"expected a (3, Ny, Nh) state (nk, ukx, uky)"
                         f"{'' if shape is None else ' of ' + str(tuple(shape))}, got {a.shape}")
    return a


def derive2coh(state, pi: float = 3.14159265358979323846, time: float = 0.0) -> np.ndarray:
    """subroutine derive2coh (src/derive2coh.f95:6): (dn_dt_new, dux_dt_new, duy_dt_new)."""
    st = _state3(state)
    _, ny, nh = st.shape
    out = np.zeros_like(st)
    old = np.zeros_like(st[0])
    lib().derive2coh_(*_ints(2 * (nh - 1), ny, nh), *_dbls(pi, time),
                      *[st[f].ctypes.data for f in range(3)], *[old.ctypes.data] * 3,
                      *[out[f].ctypes.data for f in range(3)])
    _check(lib().tara_last_error())
    return out


def ab2coh(state, d_old, d_new, pi: float = 3.14159265358979323846, time: float = 0.0) -> np.ndarray:
    """subroutine ab2coh (src/ab2coh.f95:5): (nk_new, ukx_new, uky_new), dt from /comm/."""
    st, do, dn = _state3(state), _state3(d_old), _state3(d_new)
    _, ny, nh = st.shape
    out = np.zeros_like(st)
    lib().ab2coh_(*_ints(2 * (nh - 1), ny, nh), *_dbls(pi, time),
                  *[st[f].ctypes.data for f in range(3)], *[out[f].ctypes.data for f in range(3)],
                  *[do[f].ctypes.data for f in range(3)], *[dn[f].ctypes.data for f in range(3)])
    _check(lib().tara_last_error())
    return out


class Coh2D:
    """Device-resident 2D compressible isothermal hydro state (tara_coh2d handle)."""

    def __init__(self, nx: int, ny: int | None = None, **kw):
        ny = nx if ny is None else ny
        cfg = CohConfig()
        lib().tara_coh2d_default_config(ctypes.byref(cfg), nx, ny)
        for k, v in kw.items():
            setattr(cfg, k, v)
        h = ctypes.c_void_p()
        _check(lib().tara_coh2d_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.shape = (ny, nx // 2 + 1)
        self.nx, self.ny = nx, ny
        self.cfg = cfg

    def close(self):
        if getattr(self, "_h", None):
            lib().tara_coh2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, state, hist=None):
        st = _state3(state, self.shape)
        h = None if hist is None else _state3(hist, self.shape)
        _check(lib().tara_coh2d_set_state(self._h, st.ctypes.data, None if h is None else h.ctypes.data))

    def get_state(self, with_history: bool = False):
        st = np.zeros((3,) + self.shape, np.complex128)
        h = np.zeros_like(st) if with_history else None
        _check(lib().tara_coh2d_get_state(self._h, st.ctypes.data, None if h is None else h.ctypes.data))
        return (st, h) if with_history else st

    def get_state_into(self, out: np.ndarray) -> None:
        """Copy the state into a caller-owned (3, Ny, Nh) complex128 array (e.g. pinned)."""
        if out.shape != (3,) + self.shape or out.dtype != np.complex128 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous (3, Ny, Nh) complex128 array")
        _check(lib().tara_coh2d_get_state(self._h, out.ctypes.data, None))

    def init_vortices(self, lx_ini: float = 2.0, ly_ini: float = 2.0):
        _check(lib().tara_coh2d_init_vortices(self._h, lx_ini, ly_ini))

    def rhs(self):
        out = np.zeros((3,) + self.shape, np.complex128)
        _check(lib().tara_coh2d_rhs(self._h, out.ctypes.data))
        return out

    def step(self, n: int = 1):
        _check(lib().tara_coh2d_step(self._h, int(n)))

    def synchronize(self):
        _check(lib().tara_coh2d_synchronize(self._h))

    @property
    def stream(self) -> int:
        return lib().tara_coh2d_stream(self._h) or 0

    @property
    def launches_per_step(self) -> int:
        return lib().tara_coh2d_launches_per_step(self._h)


# ---------------------------------------------------------------------------
# 2D compressible MHD
# ---------------------------------------------------------------------------
def com_common() -> ComCommon:
    """libtara's /comm/ seen with the 2D compressible MHD layout (read by derive2com_/ab2com_)."""
    return ComCommon.from_address(ctypes.addressof(MhdCommon.in_dll(lib(), "comm_")))


def _state6(a, shape=None) -> np.ndarray:
    """(rho, rho ux, rho uy, E, Bx, By) half spectra; `shape` = (Ny, Nh) of the
    handle they go to."""
    a = np.ascontiguousarray(a, dtype=np.complex128)
    if a.ndim != 3 or a.shape[0] != 6 or (shape is not None and a.shape[1:] != tuple(shape)):
        raise ValueError(f"expected a (6, Ny, Nh) state (rho, rho ux, rho uy, E, Bx, By)"
                         f"{'' if shape is None else ' of ' + str(tuple(shape))}, got {a.shape}")
    return a


def derive2com(state, pi: float = 3.14159265358979323846, time: float = 0.0) -> np.ndarray:
    """subroutine derive2com (src/derive2com.f95:5): the six d_*_k_dt_new arrays."""
    st = _state6(state)
    _, ny, nh = st.shape
    out = np.zeros_like(st)
    old = np.zeros_like(st[0])
    args = []
    for f in range(6):
        args += [old.ctypes.data, out[f].ctypes.data]
    lib().derive2com_(*_ints(2 * (nh - 1), ny, nh), *_dbls(pi, time), *[st[f].ctypes.data for f in range(6)],
                      *args)
    _check(lib().tara_last_error())
    return out


def ab2com(state, d_old, d_new, pi: float = 3.14159265358979323846, time: float = 0.0) -> np.ndarray:
    """subroutine ab2com (src/ab2com.f95): the six *_k_new arrays, dt from /comm/."""
    st, do, dn = _state6(state), _state6(d_old), _state6(d_new)
    _, ny, nh = st.shape
    out = np.zeros_like(st)
    pairs = []
    for f in range(6):
        pairs += [do[f].ctypes.data, dn[f].ctypes.data]
    lib().ab2com_(*_ints(2 * (nh - 1), ny, nh), *_dbls(pi, time), *[st[f].ctypes.data for f in range(6)],
                  *[out[f].ctypes.data for f in range(6)], *pairs)
    _check(lib().tara_last_error())
    return out


class Com2D:
    """Device-resident 2D compressible MHD state (tara_com2d handle)."""

    def __init__(self, nx: int, ny: int | None = None, **kw):
        ny = nx if ny is None else ny
        cfg = ComConfig()
        lib().tara_com2d_default_config(ctypes.byref(cfg), nx, ny)
        for k, v in kw.items():
            setattr(cfg, k, v)
        h = ctypes.c_void_p()
        _check(lib().tara_com2d_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.shape = (ny, nx // 2 + 1)
        self.nx, self.ny = nx, ny
        self.cfg = cfg

    def close(self):
        if getattr(self, "_h", None):
            lib().tara_com2d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_state(self, state, hist=None):
        st = _state6(state, self.shape)
        h = None if hist is None else _state6(hist, self.shape)
        _check(lib().tara_com2d_set_state(self._h, st.ctypes.data, None if h is None else h.ctypes.data))

    def get_state(self, with_history: bool = False):
        st = np.zeros((6,) + self.shape, np.complex128)
        h = np.zeros_like(st) if with_history else None
        _check(lib().tara_com2d_get_state(self._h, st.ctypes.data, None if h is None else h.ctypes.data))
        return (st, h) if with_history else st

    def get_state_into(self, out: np.ndarray) -> None:
        """Copy the state into a caller-owned (6, Ny, Nh) complex128 array (e.g. pinned)."""
        if out.shape != (6,) + self.shape or out.dtype != np.complex128 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous (6, Ny, Nh) complex128 array")
        _check(lib().tara_com2d_get_state(self._h, out.ctypes.data, None))

    def init_reference(self, lx_ini: float = 2.0, ly_ini: float = 2.0, b0: float = 1.0):
        _check(lib().tara_com2d_init_reference(self._h, lx_ini, ly_ini, b0))

    def rhs(self):
        out = np.zeros((6,) + self.shape, np.complex128)
        _check(lib().tara_com2d_rhs(self._h, out.ctypes.data))
        return out

    def step(self, n: int = 1):
        _check(lib().tara_com2d_step(self._h, int(n)))

    def synchronize(self):
        _check(lib().tara_com2d_synchronize(self._h))

    @property
    def stream(self) -> int:
        return lib().tara_com2d_stream(self._h) or 0

    @property
    def launches_per_step(self) -> int:
        return lib().tara_com2d_launches_per_step(self._h)


# ---------------------------------------------------------------------------
# Ensembles of runs of uneven sizes
# ---------------------------------------------------------------------------
class EnsRun(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("k0", ctypes.c_double), ("seed", ctypes.c_uint64)]


class Ensemble:
    """tara_ens handle: runs grouped by size, one CUDA-graph launch per step."""

    def __init__(self, runs, *, precision=PREC_FP32, scheme=SCHEME_RK4, nu=1e-3, dt=1e-4,
                 energy=0.5):
        arr = (EnsRun * len(runs))(*[EnsRun(int(n), float(k0), int(seed)) for n, k0, seed in runs])
        h = ctypes.c_void_p()
        _check(lib().tara_ens_create(len(runs), ctypes.cast(arr, ctypes.c_void_p), precision, scheme,
                                     nu, dt, energy, ctypes.byref(h)))
        self._h = h
        self.runs = list(runs)

    def close(self):
        if getattr(self, "_h", None):
            lib().tara_ens_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def autotune(self, trial_steps: int = 3):
        _check(lib().tara_ens_autotune(self._h, int(trial_steps)))

    def step(self, n: int = 1):
        _check(lib().tara_ens_step(self._h, int(n)))

    def set_form(self, form: int) -> None:
        """ENS_GRAPH (one graph launch per step) or ENS_PERSISTENT4 / 8 (one
        cooperative launch per step() call, radix-4 or radix-8 transforms)."""
        _check(lib().tara_ens_set_form(self._h, int(form)))

    def form(self) -> dict:
        f = ctypes.c_int()
        ms = (ctypes.c_double * 3)()
        _check(lib().tara_ens_form(self._h, ctypes.byref(f), ms))
        return {"form": ["graph", "persistent radix-4", "persistent radix-8"][f.value],
                "ms_per_step": {"graph": ms[0], "persistent radix-4": ms[1], "persistent radix-8": ms[2]}}

    def synchronize(self):
        _check(lib().tara_ens_synchronize(self._h))

    @property
    def stream(self) -> int:
        return lib().tara_ens_stream(self._h) or 0

    @property
    def launches_per_step(self) -> int:
        return lib().tara_ens_launches_per_step(self._h)

    def get_state(self, run: int) -> np.ndarray:
        n = self.runs[run][0]
        out = np.zeros((n, n // 2 + 1), np.complex128)
        _check(lib().tara_ens_get_state(self._h, run, _dp(out.view(np.float64))))
        return out

    def set_state(self, run: int, w: np.ndarray) -> None:
        n = self.runs[run][0]
        w = _as_spectrum(w, n // 2 + 1, n)
        _check(lib().tara_ens_set_state(self._h, run, _dp(w.view(np.float64))))

    def diag(self, run: int):
        e, z = ctypes.c_double(), ctypes.c_double()
        _check(lib().tara_ens_diag(self._h, run, ctypes.byref(e), ctypes.byref(z)))
        return e.value, z.value

    def groups(self):
        out = []
        for g in range(lib().tara_ens_groups(self._h)):
            n, r = ctypes.c_int(), ctypes.c_int()
            v = (ctypes.c_int * 3)()
            ms = (ctypes.c_double * 24)()
            _check(lib().tara_ens_group_info(self._h, g, ctypes.byref(n), ctypes.byref(r), v, ms))
            out.append({"n": n.value, "runs": r.value, "variants": list(v), "tuned_ms": list(ms)})
        return out


# ---------------------------------------------------------------------------
# Learned subgrid closure
# ---------------------------------------------------------------------------
def fno_default_config(**kw) -> FnoConfig:
    c = FnoConfig()
    lib().tara_fno_default_config(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class FNO:
    """tara_fno handle: the library's Fourier neural operator (BF16 tensor-core
    GEMMs with FP32 accumulation, or FP32 for checks).  Data arguments are
    device pointers (e.g. ``torch_tensor.data_ptr()``) to FP32 NHWC arrays."""

    def __init__(self, cfg: FnoConfig | None = None, **kw):
        cfg = fno_default_config(**kw) if cfg is None else cfg
        h = ctypes.c_void_p()
        _check(lib().tara_fno_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self.cfg = cfg
        self.num_params = int(lib().tara_fno_num_params(h))

    def close(self):
        if getattr(self, "_h", None):
            lib().tara_fno_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        _check(lib().tara_fno_get_params(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.size}")
        _check(lib().tara_fno_set_params(self._h, p.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))

    def get_grads(self) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        _check(lib().tara_fno_get_grads(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def set_mode(self, mode: int) -> None:
        _check(lib().tara_fno_set_mode(self._h, mode))

    def set_fused(self, enable: bool) -> None:
        """Fused small-batch inference forward (default on; see tara_fno_set_fused)."""
        _check(lib().tara_fno_set_fused(self._h, int(bool(enable))))

    def forward(self, x_ptr: int, y_ptr: int, batch: int) -> None:
        _check(lib().tara_fno_forward(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), batch))

    def train_step(self, x_ptr: int, t_ptr: int, batch: int, lr: float = 0.0, idx_ptr: int = 0,
                   n_samples: int | None = None, want_loss: bool = True) -> float | None:
        """One forward/backward (+ Adam when lr > 0).  With idx_ptr, the batch is
        gathered from datasets of n_samples samples at x_ptr / t_ptr."""
        loss = ctypes.c_double()
        ns = batch if n_samples is None else n_samples
        _check(lib().tara_fno_train_step(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(t_ptr),
                                         ctypes.c_void_p(idx_ptr or None), ns, batch, lr,
                                         ctypes.byref(loss) if want_loss else None))
        return loss.value if want_loss else None

    @property
    def adam_steps(self) -> int:
        return int(lib().tara_fno_adam_steps(self._h))

    @property
    def stream(self) -> int:
        return lib().tara_fno_stream(self._h) or 0


def closure_augment(x_ptr: int, t_ptr: int, n_samples: int, n: int, nf: int, x_out: int, t_out: int) -> None:
    """Eight-fold symmetry augmentation of closure samples (device pointers; 0 skips)."""
    _check(lib().tara_closure_augment(ctypes.c_void_p(x_ptr or None), ctypes.c_void_p(t_ptr or None),
                                      n_samples, n, nf, ctypes.c_void_p(x_out or None),
                                      ctypes.c_void_p(t_out or None)))


class Closure:
    """tara_closure: a coarse Solver2D stepped with the FNO's subgrid flux."""

    def __init__(self, solver: Solver2D, fno: FNO, in_scale, out_scale: float):
        """in_scale: one value per input feature channel (a scalar for one channel)."""
        sc = np.atleast_1d(np.asarray(in_scale, np.float64))
        if sc.size != int(fno.cfg.ci):
            raise ValueError(f"expected {int(fno.cfg.ci)} input scales, got {sc.size}")
        h = ctypes.c_void_p()
        _check(lib().tara_closure_create(solver._h, fno._h, _dp(np.ascontiguousarray(sc)), out_scale,
                                         ctypes.byref(h)))
        self._h = h
        self.solver, self.fno = solver, fno  # keep both alive

    def close(self):
        if getattr(self, "_h", None):
            lib().tara_closure_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, n: int = 1) -> None:
        _check(lib().tara_closure_step(self._h, int(n)))


# ---------------------------------------------------------------------------
# Lagrangian passive particles (plain driver)
# ---------------------------------------------------------------------------
class Particles:
    """tara_particles: passive particles moved by a Solver2D's velocity (run 0)
    with the plain driver's interpolation, Euler step and wrap."""

    def __init__(self, solver: Solver2D, xp, yp, lx: float, ly: float, kpi: float = math.pi):
        xp = np.ascontiguousarray(xp, np.float64)
        yp = np.ascontiguousarray(yp, np.float64)
        if xp.shape != yp.shape or xp.ndim != 1:
            raise ValueError("xp and yp must be 1-D arrays of equal length")
        h = ctypes.c_void_p()
        _check(lib().tara_particles_create(solver._h, kpi, lx, ly, xp.size, _dp(xp), _dp(yp), ctypes.byref(h)))
        self._h = h
        self.np = xp.size
        self.solver = solver

    def close(self):
        if getattr(self, "_h", None):
            lib().tara_particles_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def advance(self, dt: float) -> None:
        _check(lib().tara_particles_advance(self._h, dt))

    def positions(self):
        x, y = np.zeros(self.np), np.zeros(self.np)
        _check(lib().tara_particles_get(self._h, _dp(x), _dp(y)))
        return x, y


def park_miller(n: int, state: int = 1):
    """n draws of the driver's RAND generator (minimal-standard LCG) and the final state."""
    st = ctypes.c_uint64(state)
    out = np.array([lib().tara_park_miller_rand(ctypes.byref(st)) for _ in range(n)], np.float32)
    return out, st.value
