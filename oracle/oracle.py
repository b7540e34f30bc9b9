"""ctypes binding of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module, and only as the oracle.  ``load()`` returns the own-FFT
restatement (liboracle.so, builds anywhere); ``load(fftw=True)`` returns the
same restatement over FFTW 3.3.9 compiled from the reference's vendored sources
(oracle/_ref/liboracle_fftw.so), which exists only where the reference tree was
available at build time.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT = HERE / "liboracle.so"
REF = HERE / "_ref" / "liboracle_fftw.so"
PI_R4 = float(np.float32(3.1428))
PI_R8 = 3.14159265358979323846

_cache: dict = {}


def available(fftw: bool = False) -> bool:
    return (REF if fftw else PORT).exists()


def load(fftw: bool = False) -> "Oracle":
    key = bool(fftw)
    if key not in _cache:
        path = REF if fftw else PORT
        if not path.exists():
            raise FileNotFoundError(f"{path} missing (make -C oracle {'ref' if fftw else 'port'})")
        _cache[key] = Oracle(ctypes.CDLL(str(path)))
    return _cache[key]


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(v):
    return ctypes.byref(ctypes.c_int(int(v)))


def _d(v):
    return ctypes.byref(ctypes.c_double(float(v)))


class MhdParams(ctypes.Structure):
    """oracle_mhd_params (oracle/tara_oracle.h)."""
    _fields_ = [("lx", ctypes.c_double), ("ly", ctypes.c_double), ("lz", ctypes.c_double),
                ("mu", ctypes.c_double), ("eta", ctypes.c_double), ("cs", ctypes.c_double),
                ("defined", ctypes.c_int), ("nu_u", ctypes.c_double), ("eta_b", ctypes.c_double)]


class CohParams(ctypes.Structure):
    """oracle_coh_params (oracle/tara_oracle.h)."""
    _fields_ = [("pi", ctypes.c_double), ("lx", ctypes.c_double), ("ly", ctypes.c_double),
                ("mux", ctypes.c_double), ("muy", ctypes.c_double), ("cs", ctypes.c_double)]


def coh_params(pi=PI_R8, lx=2 * PI_R8, ly=2 * PI_R8, mux=2e-4, muy=2e-4, cs=3.77) -> CohParams:
    """Defaults: the values src/main2coh.f95 sets (Lx = Ly = 2 pi, mux = muy =
    0.0002, CS = U0/M = 1.885/0.5)."""
    return CohParams(pi, lx, ly, mux, muy, cs)


class ComParams(ctypes.Structure):
    """oracle_com_params (oracle/tara_oracle.h)."""
    _fields_ = [(n, ctypes.c_double) for n in ("pi", "lx", "ly", "mu", "eta", "cs", "kf", "a")] + [
        ("defined", ctypes.c_int)]


def com_params(pi=PI_R8, lx=2 * PI_R8, ly=2 * PI_R8, mu=1e-3, eta=1e-4, cs=100.0, kf=1.0, a=1.0,
               defined=0) -> ComParams:
    """Defaults: src/main2com.f95 (eta = 1e-4, CS = 1/M = 100, kf = A = 1; mu is the
    ini's nu, 1e-3 here)."""
    return ComParams(pi, lx, ly, mu, eta, cs, kf, a, defined)


def mhd_params(lx=2 * PI_R8, ly=2 * PI_R8, lz=2 * PI_R8, mu=0.01, eta=0.005, cs=10.0,
               defined=0, nu_u=0.0, eta_b=0.0) -> MhdParams:
    return MhdParams(lx, ly, lz, mu, eta, cs, defined, nu_u, eta_b)


class Oracle:
    def __init__(self, L):
        self.L = L
        c_int, c_double, vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        L.oracle_run.argtypes = [c_int, c_int, c_int, c_int, c_double, c_double, c_double, c_int,
                                 vp, vp]
        L.oracle_ic_shear.argtypes = [c_int, c_int, c_double, c_double, c_double, c_double,
                                      c_double, c_int, vp]
        L.oracle_ic_random.argtypes = [c_int, c_int, c_double, c_double, ctypes.c_uint64, vp]
        L.oracle_energy_enstrophy.argtypes = [c_int, c_int, c_double, c_double, vp, vp]
        L.oracle_diag_css.argtypes = [c_int, c_int, c_double, c_double, c_double, vp, vp]
        L.oracle_set_css_params.argtypes = [c_double, c_double, c_double]
        L.oracle_r2c_2d.argtypes = [c_int, c_int, vp, vp]
        L.oracle_c2r_2d.argtypes = [c_int, c_int, vp, vp]
        L.oracle_set_threads.argtypes = [c_int]
        L.oracle_r2c_3d.argtypes = [c_int, c_int, c_int, vp, vp]
        L.oracle_c2r_3d.argtypes = [c_int, c_int, c_int, vp, vp]
        L.oracle_derive3com.argtypes = [c_int, c_int, c_int, vp, vp, vp]
        L.oracle_ab3com.argtypes = [c_int, c_int, c_int, c_double, vp, vp, vp, vp]
        L.oracle_run3d.argtypes = [c_int, c_int, c_int, vp, c_double, c_int, vp, vp]
        L.oracle_ic3d_abc.argtypes = [c_int, c_int, c_int, c_double, c_double, c_double, vp]
        L.oracle_ic3d_ot.argtypes = [c_int, c_int, c_int, c_double, c_int, ctypes.c_uint64, vp]
        L.oracle_driver_velocity.argtypes = [c_int, c_int, c_double, c_double, vp, vp, vp]
        L.oracle_particles_step.argtypes = [c_int, c_int, c_double, c_double, vp, vp, c_int, vp, vp,
                                            c_double]
        L.oracle_derive2coh.argtypes = [c_int, c_int, vp, vp, vp]
        L.oracle_ab2coh.argtypes = [c_int, c_int, c_double, vp, vp, vp, vp]
        L.oracle_run_coh.argtypes = [c_int, c_int, vp, c_double, c_int, vp, vp]
        L.oracle_ic_coh.argtypes = [c_int, c_int, c_double, c_double, vp]
        L.oracle_derive2com.argtypes = [c_int, c_int, vp, vp, vp]
        L.oracle_ab2com.argtypes = [c_int, c_int, c_double, vp, vp, vp, vp]
        L.oracle_run_com.argtypes = [c_int, c_int, vp, c_double, c_int, vp, vp]
        L.oracle_ic_com.argtypes = [c_int, c_int, c_double, c_double, c_double, c_double, c_double, vp]
        self.is_fftw = bool(L.oracle_backend_is_fftw())

    def set_threads(self, n: int) -> None:
        self.L.oracle_set_threads(int(n))

    def threads(self) -> int:
        return int(self.L.oracle_get_threads())

    # transforms (unnormalised, FFTW semantics)
    def r2c(self, x):
        x = np.ascontiguousarray(x, np.float64)
        ny, nx = x.shape
        out = np.zeros((ny, nx // 2 + 1), np.complex128)
        self.L.oracle_r2c_2d(nx, ny, x.ctypes.data, out.ctypes.data)
        return out

    def c2r(self, c, nx=None):
        """Unnormalised c2r of a (Ny, Nh) half spectrum; nx defaults to the even
        length 2 (Nh - 1) (an odd nx = 2 Nh - 1 has the same Nh)."""
        c = np.ascontiguousarray(c, np.complex128)
        ny, nh = c.shape
        nx = 2 * (nh - 1) if nx is None else int(nx)
        if nx // 2 + 1 != nh:
            raise ValueError(f"nx = {nx} does not match Nh = {nh}")
        out = np.zeros((ny, nx), np.float64)
        self.L.oracle_c2r_2d(nx, ny, c.ctypes.data, out.ctypes.data)
        return out

    # reference subroutines
    def derive2csh(self, w, nu):
        w = np.ascontiguousarray(w, np.complex128).copy()
        ny, nh = w.shape
        out = np.zeros_like(w)
        self.L.oracle_derive2csh(_i(2 * (nh - 1)), _i(ny), _i(nh), _d(nu), _d(0.0),
                                 _dp(w.view(np.float64)), None, None, _dp(out.view(np.float64)))
        return out

    def derive2css(self, w, alpha, nu):
        w = np.ascontiguousarray(w, np.complex128).copy()
        ny, nh = w.shape
        out = np.zeros_like(w)
        self.L.oracle_derive2css(_i(2 * (nh - 1)), _i(ny), _i(nh), _d(alpha), _d(nu), _d(0.0),
                                 _dp(w.view(np.float64)), None, None, _dp(out.view(np.float64)))
        return out

    def ab2(self, w, fo, fn, dt):
        w, fo, fn = (np.ascontiguousarray(a, np.complex128) for a in (w, fo, fn))
        ny, nh = w.shape
        out = np.zeros_like(w)
        self.L.oracle_ab2csh(_i(2 * (nh - 1)), _i(ny), _i(nh), _d(0.0), _d(0.0), _d(dt),
                             _dp(w.view(np.float64)), _dp(out.view(np.float64)),
                             _dp(fo.view(np.float64)), _dp(fn.view(np.float64)))
        return out

    def rk42css(self, w, alpha, nu, dt):
        w = np.ascontiguousarray(w, np.complex128).copy()
        ny, nh = w.shape
        out = np.zeros_like(w)
        self.L.oracle_rk42css(_i(2 * (nh - 1)), _i(ny), _i(nh), _d(alpha), _d(nu), _d(0.0), _d(dt),
                              _dp(w.view(np.float64)), _dp(out.view(np.float64)), None, None)
        return out

    def set_css_params(self, lx, ly, lam):
        self.L.oracle_set_css_params(lx, ly, lam)

    def run(self, w, *, rhs=0, scheme=0, alpha=1.0, nu=0.01, dt=1e-4, steps=1, dt_old=None):
        w = np.ascontiguousarray(w, np.complex128).copy()
        fo = np.zeros_like(w) if dt_old is None else np.ascontiguousarray(dt_old, np.complex128).copy()
        ny, nh = w.shape
        self.L.oracle_run(2 * (nh - 1), ny, rhs, scheme, alpha, nu, dt, int(steps), w.ctypes.data,
                          fo.ctypes.data)
        return w, fo

    # initial conditions and diagnostics
    def ic_shear(self, nx, ny, lx_ini=2.0, ly_ini=2.0, w0=25.0, m0=2.0, d_ini=0.0234375, variant=0):
        out = np.zeros((ny, nx), np.float64)
        self.L.oracle_ic_shear(nx, ny, lx_ini, ly_ini, w0, m0, d_ini, variant, out.ctypes.data)
        return out

    def ic_random(self, nx, ny, k0, energy, seed):
        out = np.zeros((ny, nx // 2 + 1), np.complex128)
        self.L.oracle_ic_random(nx, ny, k0, energy, seed, out.ctypes.data)
        return out

    def energy_enstrophy(self, w, lx=2 * PI_R8, ly=2 * PI_R8):
        w = np.ascontiguousarray(w, np.complex128)
        ny, nh = w.shape
        out = np.zeros(2)
        self.L.oracle_energy_enstrophy(2 * (nh - 1), ny, lx, ly, w.ctypes.data, out.ctypes.data)
        return float(out[0]), float(out[1])

    def diag_css(self, w, lx, ly, lam=10.0):
        w = np.ascontiguousarray(w, np.complex128)
        ny, nh = w.shape
        out = np.zeros(6)
        self.L.oracle_diag_css(2 * (nh - 1), ny, lx, ly, lam, w.ctypes.data, out.ctypes.data)
        return out

    # Lagrangian particles of the plain driver
    def driver_velocity(self, w, lx, ly):
        w = np.ascontiguousarray(w, np.complex128)
        ny, nh = w.shape
        nx = 2 * (nh - 1)
        ux, uy = np.zeros((ny, nx)), np.zeros((ny, nx))
        self.L.oracle_driver_velocity(nx, ny, lx, ly, w.ctypes.data, ux.ctypes.data, uy.ctypes.data)
        return ux, uy

    def particles_step(self, ux, uy, xp, yp, lx, ly, dt):
        ux, uy = np.ascontiguousarray(ux, np.float64), np.ascontiguousarray(uy, np.float64)
        xp, yp = np.array(xp, np.float64), np.array(yp, np.float64)
        ny, nx = ux.shape
        self.L.oracle_particles_step(nx, ny, lx, ly, ux.ctypes.data, uy.ctypes.data, xp.size,
                                     xp.ctypes.data, yp.ctypes.data, dt)
        return xp, yp

    # 3D MHD: arrays are (Nz, Ny, Nh) complex / (Nz, Ny, Nx) real; a state is (8, Nz, Ny, Nh)
    def r2c3(self, x):
        x = np.ascontiguousarray(x, np.float64)
        nz, ny, nx = x.shape
        out = np.zeros((nz, ny, nx // 2 + 1), np.complex128)
        self.L.oracle_r2c_3d(nx, ny, nz, x.ctypes.data, out.ctypes.data)
        return out

    def c2r3(self, c):
        c = np.ascontiguousarray(c, np.complex128)
        nz, ny, nh = c.shape
        nx = 2 * (nh - 1)
        out = np.zeros((nz, ny, nx), np.float64)
        self.L.oracle_c2r_3d(nx, ny, nz, c.ctypes.data, out.ctypes.data)
        return out

    # 2D compressible isothermal hydro: state (3, Ny, Nh) = (nk, ukx, uky)
    def derive2coh(self, state, params):
        state = np.ascontiguousarray(state, np.complex128)
        _, ny, nh = state.shape
        out = np.zeros_like(state)
        self.L.oracle_derive2coh(2 * (nh - 1), ny, ctypes.addressof(params), state.ctypes.data,
                                 out.ctypes.data)
        return out

    def ab2coh(self, state, d_old, d_new, dt):
        state, d_old, d_new = (np.ascontiguousarray(a, np.complex128) for a in (state, d_old, d_new))
        _, ny, nh = state.shape
        out = np.zeros_like(state)
        self.L.oracle_ab2coh(2 * (nh - 1), ny, dt, state.ctypes.data, out.ctypes.data,
                             d_old.ctypes.data, d_new.ctypes.data)
        return out

    def run_coh(self, state, params, dt, steps, hist=None):
        st = np.ascontiguousarray(state, np.complex128).copy()
        h = np.zeros_like(st) if hist is None else np.ascontiguousarray(hist, np.complex128).copy()
        _, ny, nh = st.shape
        self.L.oracle_run_coh(2 * (nh - 1), ny, ctypes.addressof(params), dt, int(steps),
                              st.ctypes.data, h.ctypes.data)
        return st, h

    def ic_coh(self, nx, ny, l_ini=2.0):
        out = np.zeros((3, ny, nx // 2 + 1), np.complex128)
        self.L.oracle_ic_coh(nx, ny, l_ini, l_ini, out.ctypes.data)
        return out

    # 2D compressible MHD: state (6, Ny, Nh) = (rho, rho ux, rho uy, E, Bx, By)
    def derive2com(self, state, params):
        state = np.ascontiguousarray(state, np.complex128)
        _, ny, nh = state.shape
        out = np.zeros_like(state)
        self.L.oracle_derive2com(2 * (nh - 1), ny, ctypes.addressof(params), state.ctypes.data,
                                 out.ctypes.data)
        return out

    def ab2com(self, state, d_old, d_new, dt):
        state, d_old, d_new = (np.ascontiguousarray(a, np.complex128) for a in (state, d_old, d_new))
        _, ny, nh = state.shape
        out = np.zeros_like(state)
        self.L.oracle_ab2com(2 * (nh - 1), ny, dt, state.ctypes.data, out.ctypes.data,
                             d_old.ctypes.data, d_new.ctypes.data)
        return out

    def run_com(self, state, params, dt, steps, hist=None):
        st = np.ascontiguousarray(state, np.complex128).copy()
        h = np.zeros_like(st) if hist is None else np.ascontiguousarray(hist, np.complex128).copy()
        _, ny, nh = st.shape
        self.L.oracle_run_com(2 * (nh - 1), ny, ctypes.addressof(params), dt, int(steps),
                              st.ctypes.data, h.ctypes.data)
        return st, h

    def ic_com(self, nx, ny, l_ini=2.0, cs=100.0, kf=1.0, b0=1.0):
        out = np.zeros((6, ny, nx // 2 + 1), np.complex128)
        self.L.oracle_ic_com(nx, ny, l_ini, l_ini, cs, kf, b0, out.ctypes.data)
        return out

    def derive3com(self, state, params):
        state = np.ascontiguousarray(state, np.complex128)
        _, nz, ny, nh = state.shape
        out = np.zeros_like(state)
        self.L.oracle_derive3com(2 * (nh - 1), ny, nz, ctypes.addressof(params), state.ctypes.data,
                                 out.ctypes.data)
        return out

    def ab3com(self, state, d_old, d_new, dt):
        state, d_old, d_new = (np.ascontiguousarray(a, np.complex128) for a in (state, d_old, d_new))
        _, nz, ny, nh = state.shape
        out = np.zeros_like(state)
        self.L.oracle_ab3com(2 * (nh - 1), ny, nz, dt, state.ctypes.data, out.ctypes.data,
                             d_old.ctypes.data, d_new.ctypes.data)
        return out

    def run3d(self, state, params, dt, steps, hist=None):
        st = np.ascontiguousarray(state, np.complex128).copy()
        h = np.zeros_like(st) if hist is None else np.ascontiguousarray(hist, np.complex128).copy()
        _, nz, ny, nh = st.shape
        self.L.oracle_run3d(2 * (nh - 1), ny, nz, ctypes.addressof(params), dt, int(steps),
                            st.ctypes.data, h.ctypes.data)
        return st, h

    def ic3d_abc(self, nx, ny, nz, l_ini=2.0):
        out = np.zeros((8, nz, ny, nx), np.float64)
        self.L.oracle_ic3d_abc(nx, ny, nz, l_ini, l_ini, l_ini, out.ctypes.data)
        return out

    def ic3d_ot(self, nx, ny=None, nz=None, amp=0.01, kmax=4, seed=3):
        """The 3D MHD benchmark's initial state as a spectral state (8, Nz, Ny, Nh)."""
        ny = nx if ny is None else ny
        nz = nx if nz is None else nz
        out = np.zeros((8, nz, ny, nx // 2 + 1), np.complex128)
        self.L.oracle_ic3d_ot(nx, ny, nz, amp, kmax, seed, out.ctypes.data)
        return out

    def state_from_real(self, real8):
        return np.stack([self.r2c3(f) for f in real8])

    def philox(self, ctr, key):
        out = (ctypes.c_uint32 * 4)()
        self.L.oracle_philox4x32_10((ctypes.c_uint32 * 4)(*ctr), (ctypes.c_uint32 * 2)(*key), out)
        return [int(v) for v in out]
