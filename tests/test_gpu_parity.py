"""GPU parity tests: libtara's CUDA path, called through the C ABI, against the
CPU oracle and the FFTW-generated golden vectors.

Tolerances (relative L2 over the half spectrum, FP64 path):
  transforms 1e-14, one RHS evaluation 1e-12, 2000 AB2 steps 1e-10.
The FP32-transform mode is checked against the FP64 path with 1e-5.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

pytestmark = pytest.mark.gpu

PI_R4 = tg.PI_R4
PI_R8 = 3.14159265358979323846


@pytest.fixture(autouse=True)
def _reset_css():
    tg.set_css_params(2 * PI_R4, 2 * PI_R4, 10.0)
    yield
    tg.set_css_params(2 * PI_R4, 2 * PI_R4, 10.0)


# ---------------------------------------------------------------- transforms
def test_fft_golden_vectors(golden):
    assert rel_l2(tg.fft2d_r2c(golden["fft_r2c_in"]), golden["fft_r2c_out"]) < 1e-14
    # non-Hermitian input: Im of the kx = 0 and kx = Nx/2 bins is discarded after the y pass
    assert rel_l2(tg.fft2d_c2r(golden["fft_c2r_in"]), golden["fft_c2r_out"]) < 1e-14


@pytest.mark.parametrize("ny,nx", [(16, 16), (32, 64), (64, 16), (128, 128), (256, 512),
                                   (1024, 1024), (2048, 2048), (16, 2048), (2048, 16), (4096, 4096),
                                   (16, 4096), (4096, 32)])
def test_fft_vs_oracle(oracle, ny, nx):
    rng = np.random.default_rng(nx * 7 + ny)
    x = rng.standard_normal((ny, nx))
    assert rel_l2(tg.fft2d_r2c(x), oracle.r2c(x)) < 1e-14
    c = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
    assert rel_l2(tg.fft2d_c2r(c), oracle.c2r(c)) < 1e-14


@pytest.mark.parametrize("n", [64, 512])
def test_fft_fp32_mode(oracle, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, n))
    assert rel_l2(tg.fft2d_r2c(x, tg.PREC_FP32), oracle.r2c(x)) < 1e-6
    c = oracle.r2c(x)
    assert rel_l2(tg.fft2d_c2r(c, tg.PREC_FP32), oracle.c2r(c)) < 1e-6


# ---------------------------------------------------------------- drop-ins
def test_derive2csh_golden(golden):
    f = tg.derive2csh(golden["ic_spec"], 0.01)
    assert rel_l2(f, golden["rhs_plain"]) < 1e-12


def test_derive2css_golden(golden):
    assert rel_l2(tg.derive2css(golden["ic_spec"], 1.0, 0.01), golden["rhs_screen"]) < 1e-12
    tg.set_css_params(2.0 * PI_R8, 2.0 * PI_R8, 10.0)  # the driver's Lx = Lx_ini*pi
    assert rel_l2(tg.derive2css(golden["ic_spec"], 1.0, 0.01), golden["rhs_screen_driverL"]) < 1e-12


@pytest.mark.parametrize("ny,nx", [(64, 128), (256, 64), (512, 512), (2048, 2048), (16, 2048), (2048, 16),
                                   (4096, 4096), (4096, 64), (32, 4096)])
def test_derive_vs_oracle_sizes(oracle, ny, nx):
    w = oracle.ic_random(nx, ny, 6.0, 0.5, 11) if nx == ny else None
    if w is None:
        rng = np.random.default_rng(5)
        w = oracle.r2c(rng.standard_normal((ny, nx)))
    assert rel_l2(tg.derive2csh(w, 1e-3), oracle.derive2csh(w, 1e-3)) < 1e-12
    oracle.set_css_params(2 * PI_R4, 2 * PI_R4, 10.0)
    assert rel_l2(tg.derive2css(w, 0.7, 1e-3), oracle.derive2css(w, 0.7, 1e-3)) < 1e-12


def test_finalize_frees_and_recreates_dropin_contexts(golden):
    """tara_finalize drops the per-shape contexts of the 2D and compressible
    drop-ins; the next calls build them again and give the same results."""
    a = tg.derive2csh(golden["ic_spec"], 0.01)
    c = tg.coh_common()
    c.Lx, c.Ly, c.mux, c.muy, c.ms, c.CS, c.dt = 2 * PI_R8, 2 * PI_R8, 2e-4, 2e-4, 1.0, 3.77, 1e-3
    st = np.zeros((3, 32, 17), np.complex128)
    st[0, 0, 0] = 32 * 32
    st[1, 1, 2] = 40.0 + 3.0j
    d0 = tg.derive2coh(st)
    tg.finalize()
    assert rel_l2(tg.derive2csh(golden["ic_spec"], 0.01), a) < 1e-15
    assert rel_l2(tg.derive2coh(st), d0) < 1e-15
    tg.finalize()


def test_ab2_dropin_exact(oracle):
    rng = np.random.default_rng(2)
    shp = (32, 17)
    w, fo, fn = (rng.standard_normal(shp) + 1j * rng.standard_normal(shp) for _ in range(3))
    assert rel_l2(tg.ab2csh(w, fo, fn, 1e-3), oracle.ab2(w, fo, fn, 1e-3)) < 1e-15


def test_reference_loop_2000_steps_through_dropins(golden):
    """The reference driver loop (src/main2csh.f95:114-126): derive2csh, ab2csh,
    then rotate the history and state on the host, 2000 times at 64^2."""
    w = golden["ic_spec"].copy()
    fo = np.zeros_like(w)
    for _ in range(2000):
        fn = tg.derive2csh(w, 0.01)
        w = tg.ab2csh(w, fo, fn, 1e-4)
        fo = fn
    assert rel_l2(w, golden["ab2_plain_2000"]) < 1e-10
    assert rel_l2(fo, golden["ab2_plain_2000_hist"]) < 1e-10


def test_rk42css_golden(golden):
    assert rel_l2(tg.rk42css(golden["ic_spec"], 1.0, 0.01, 1e-4), golden["rk42css_1"]) < 1e-12


# ---------------------------------------------------------------- resident solver
@pytest.mark.parametrize("steps", [1, 10, 2000])
def test_solver_ab2_plain_golden(oracle, golden, steps):
    with tg.Solver2D(64, nu=0.01, dt=1e-4) as s:
        s.set_state(golden["ic_spec"])
        s.step(steps)
        w, fo = s.get_state(with_history=True)
    assert rel_l2(w, golden[f"ab2_plain_{steps}"]) < 1e-10
    assert rel_l2(fo, golden[f"ab2_plain_{steps}_hist"]) < 1e-10
    # the parity bar is stated for the vorticity in real space
    assert rel_l2(oracle.c2r(w), oracle.c2r(golden[f"ab2_plain_{steps}"])) < 1e-10


def test_solver_ab2_screen_golden(golden):
    with tg.Solver2D(64, rhs=tg.RHS_SCREEN, nu=0.01, dt=1e-4, alpha=1.0, lam=10.0) as s:
        s.set_state(golden["ic_spec"])
        s.step(2000)
        w = s.get_state()
    assert rel_l2(w, golden["ab2_screen_2000"]) < 1e-10


def test_solver_rk4_plain_golden(golden):
    with tg.Solver2D(64, scheme=tg.SCHEME_RK4, nu=1e-4, dt=5e-5) as s:
        s.set_state(golden["ic_random"])
        s.step(10)
        w = s.get_state()
    assert rel_l2(w, golden["rk4_plain_10"]) < 1e-12


def test_solver_rk4_512_vs_oracle(oracle):
    """Config-2 physics (512^2, nu=1e-4, dt=5e-5, RK4) for 5 steps."""
    w0 = oracle.ic_random(512, 512, 6.0, 0.5, 20240512)
    ref, _ = oracle.run(w0, rhs=0, scheme=1, nu=1e-4, dt=5e-5, steps=5)
    with tg.Solver2D(512, scheme=tg.SCHEME_RK4, nu=1e-4, dt=5e-5) as s:
        s.set_state(w0)
        s.step(5)
        w = s.get_state()
    assert rel_l2(w, ref) < 1e-12


def test_init_random_matches_oracle(oracle):
    for n, seed in ((64, 20240512), (512, 20240512), (2048, 20242048)):
        with tg.Solver2D(n) as s:
            s.init_random(6.0, 0.5, seed)
            w = s.get_state()
            e, _ = s.diag()
        assert rel_l2(w, oracle.ic_random(n, n, 6.0, 0.5, seed)) < 1e-13
        assert abs(e - 0.5) < 1e-13


def test_diag_matches_oracle(oracle, golden):
    with tg.Solver2D(64) as s:
        s.set_state(golden["ic_spec"])
        e, z = s.diag()
    eo, zo = oracle.energy_enstrophy(golden["ic_spec"])
    assert abs(e - eo) < 1e-12 * eo and abs(z - zo) < 1e-12 * zo


def test_2048_rk4_properties(oracle):
    """Full-size checks where a long oracle run is too slow: one RHS against the
    oracle, then RK4 steps conserve Hermitian symmetry and dissipate energy at
    the rate dE/dt = -2 nu Z."""
    n, nu, dt = 2048, 1e-4, 5e-5
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=nu, dt=dt) as s:
        s.init_random(6.0, 0.5, 20242048)
        w0 = s.get_state()
        assert rel_l2(s.rhs(), oracle.derive2csh(w0, nu)) < 1e-12
        e0, z0 = s.diag()
        s.step(4)
        e1, z1 = s.diag()
        w1 = s.get_state()
    assert e1 < e0 and z1 < z0
    rate = (e1 - e0) / (4 * dt)
    assert abs(rate + 2 * nu * 0.5 * (z0 + z1)) < 1e-3 * abs(rate)
    col = w1[:, 0]
    assert np.allclose(col[1:], np.conj(col[1:][::-1]), atol=1e-12 * np.abs(col).max())


def test_fp32_mode_error_vs_fp64(oracle):
    """FP32 transforms and products with FP64 state: relative error vs FP64."""
    w0 = oracle.ic_random(256, 256, 6.0, 0.5, 4000)
    out = []
    for prec in (tg.PREC_FP64, tg.PREC_FP32):
        with tg.Solver2D(256, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-4, precision=prec) as s:
            s.set_state(w0)
            s.step(50)
            out.append(s.get_state())
    assert rel_l2(out[1], out[0]) < 1e-5


def test_nonfinite_state_is_reported(golden):
    w = golden["ic_spec"].copy()
    w[3, 4] = np.nan
    with tg.Solver2D(64) as s:
        s.set_state(w)
        s.step(1)
        with pytest.raises(tg.TaraError) as e:
            s.synchronize()
        assert e.value.code == tg.TARA_ERR_NONFINITE


def test_rhs_does_not_touch_input(golden):
    w = golden["ic_spec"].copy()
    before = w.copy()
    L = tg.lib()
    out = np.zeros_like(w)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    ints = [ctypes.byref(ctypes.c_int(v)) for v in (64, 64, 33)]
    dbl = [ctypes.byref(ctypes.c_double(v)) for v in (0.01, 0.0)]
    L.derive2csh_(*ints, *dbl, dp(w.view(np.float64)), None, None, dp(out.view(np.float64)))
    assert tg.last_error()[0] == tg.TARA_OK
    assert np.array_equal(w, before)


def test_pinned_host_round_trip():
    """Page-locked host arrays take the contiguous staged copy; pageable ones the
    pitched copy: both give the same state, bit for bit."""
    torch = pytest.importorskip("torch")
    n = 512
    rng = np.random.default_rng(77)
    w = rng.standard_normal((n, n // 2 + 1)) + 1j * rng.standard_normal((n, n // 2 + 1))
    pin_in = torch.empty((n, n // 2 + 1), dtype=torch.complex128, pin_memory=True).numpy()
    pin_out = torch.empty((n, n // 2 + 1), dtype=torch.complex128, pin_memory=True).numpy()
    pin_in[:] = w
    with tg.Solver2D(n) as s:
        s.set_state(pin_in)
        s.get_state_into(pin_out)
        assert np.array_equal(pin_out, w)
        assert np.array_equal(s.get_state(), w)  # pageable read of the pinned write
        s.set_state(w)                           # pageable write
        s.get_state_into(pin_out)
        assert np.array_equal(pin_out, w)


def test_4096_rk4_steps_and_configurations(oracle):
    """4096^2 (a grid the reference's input.ini can name): the resident RK4
    solver's right-hand side against the oracle, every configuration the
    autotuner may pick (tile variants that fit a CTA, both radix paths) giving
    the default's result (bitwise on one radix path), and RK4 steps that keep
    Hermitian symmetry and dissipate energy at dE/dt = -2 nu Z."""
    n, nu, dt = 4096, 1e-4, 2.5e-5
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=nu, dt=dt) as s:
        s.init_random(6.0, 0.5, 4096)
        w0 = s.get_state()
        assert rel_l2(s.rhs(), oracle.derive2csh(w0, nu)) < 1e-12
        e0, z0 = s.diag()
        s.step(2)
        e1, z1 = s.diag()
        w1 = s.get_state()
        r = s.autotune(1)
    assert e1 < e0 and z1 < z0
    rate = (e1 - e0) / (2 * dt)
    assert abs(rate + 2 * nu * 0.5 * (z0 + z1)) < 1e-3 * abs(rate)
    col = w1[:, 0]
    assert np.allclose(col[1:], np.conj(col[1:][::-1]), atol=1e-12 * np.abs(col).max())
    # the FP64 row pass fits one CTA only in the three-slot tile at 4096 points
    assert r["variants"][1] & 3 == 3
    for c in range(8):
        assert r["ms"][c][1] > 0 if c & 3 == 3 else r["ms"][c][1] == 0
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=nu, dt=dt) as s:
        s.set_state(w0)
        s.set_variants(r["variants"])
        s.step(2)
        w2 = s.get_state()
    if all(v & 4 == 0 for v in r["variants"]):
        assert np.array_equal(w2, w1)
    else:
        assert rel_l2(w2, w1) < 1e-13
