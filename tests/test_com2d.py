"""2D compressible MHD (src/derive2com.f95, src/ab2com.f95).

CPU: the own-FFT oracle against the FFTW-oracle golden vectors
(tests/golden/golden_com.npz, tests/golden/make_golden.py).
GPU: the drop-ins derive2com_ / ab2com_ (common block /comm/ through libtara's
comm_) and the device-resident Com2D solver, faithful and defined curl B.

Tolerances (relative L2).  The reference state at Mach 0.01 carries a pressure
CS^2 rho = 1e4 whose gradients nearly cancel, so its right-hand side is
ill-conditioned: two correct FFTs (own radix-2 and FFTW) give RHS that differ by
1e-11 at the initial state and by 1e-8 after 500 steps, while the states agree to
3e-14.  Hence: states 1e-11; the RHS of the well-conditioned smooth state 1e-12;
the RHS at the reference state 1e-9; histories after many steps 1e-6.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from oracle import oracle as orc

GOLDEN_COM = ROOT / "tests" / "golden" / "golden_com.npz"
PI = orc.PI_R8


@pytest.fixture(scope="module")
def gcom():
    return dict(np.load(GOLDEN_COM))


# ------------------------------------------------------------------ CPU (oracle)
def test_oracle_ic_golden(oracle, gcom):
    assert rel_l2(oracle.ic_com(64, 64), gcom["ic"]) < 1e-14


def test_oracle_derive2com_golden(oracle, gcom):
    assert rel_l2(oracle.derive2com(gcom["ic"], orc.com_params()), gcom["rhs_ic"]) < 1e-9
    assert rel_l2(oracle.derive2com(gcom["smooth"], orc.com_params()), gcom["rhs_smooth"]) < 1e-13
    assert rel_l2(oracle.derive2com(gcom["smooth"], orc.com_params(defined=1)),
                  gcom["rhs_smooth_defined"]) < 1e-13


def test_oracle_run_golden(oracle, gcom):
    st, h = oracle.run_com(gcom["ic"], orc.com_params(), 2e-4, 500)
    assert rel_l2(st, gcom["ab2_500"]) < 1e-11
    assert rel_l2(h, gcom["ab2_500_hist"]) < 1e-6


def test_oracle_reference_defect_is_kept(oracle, gcom):
    """The faithful curl B (from d_ux_dx, d_uy_dy / (Nx Ny)) differs from the
    defined one once B varies; at the uniform-B, divergence-free initial state
    both vanish up to rounding."""
    assert rel_l2(gcom["rhs_smooth"], gcom["rhs_smooth_defined"]) > 1e-10
    a = oracle.derive2com(gcom["ic"], orc.com_params())
    b = oracle.derive2com(gcom["ic"], orc.com_params(defined=1))
    assert rel_l2(a, b) < 1e-14


# ------------------------------------------------------------------ GPU
gpu = pytest.mark.gpu


def _tg():
    import tara_gb300 as tg

    return tg


def _set_common(tg, lx=2 * PI, ly=2 * PI, mu=1e-3, eta=1e-4, cs=100.0, dt=2e-4, kf=1.0, a=1.0):
    c = tg.com_common()
    c.Lx, c.Ly, c.spheat, c.mu, c.ms, c.CS = lx, ly, 5.0 / 3.0, mu, 1.0, cs
    c.mu_0, c.eta, c.dt, c.kf, c.A = 1.0, eta, dt, kf, a


@gpu
def test_gpu_derive2com_golden(gcom):
    tg = _tg()
    _set_common(tg)
    assert rel_l2(tg.derive2com(gcom["ic"]), gcom["rhs_ic"]) < 1e-9
    assert rel_l2(tg.derive2com(gcom["smooth"]), gcom["rhs_smooth"]) < 1e-12


@gpu
def test_gpu_reference_loop_golden(gcom):
    """The driver loop of src/main2com.f95:352-414 through the two drop-ins."""
    tg = _tg()
    _set_common(tg, dt=2e-4)
    st = gcom["ic"].copy()
    old = np.zeros_like(st)
    for _ in range(10):
        new = tg.derive2com(st)
        st = tg.ab2com(st, old, new)
        old = new
    assert rel_l2(st, gcom["ab2_10"]) < 1e-11
    assert rel_l2(old, gcom["ab2_10_hist"]) < 1e-6


@gpu
@pytest.mark.parametrize("steps", [1, 10, 500])
def test_gpu_solver_ab2_golden(gcom, steps):
    tg = _tg()
    with tg.Com2D(64, dt=2e-4) as s:
        s.set_state(gcom["ic"])
        s.step(steps)
        st, h = s.get_state(with_history=True)
    assert rel_l2(st, gcom[f"ab2_{steps}"]) < 1e-11
    assert rel_l2(h, gcom[f"ab2_{steps}_hist"]) < 1e-6


@gpu
def test_gpu_defined_mode_golden(gcom):
    tg = _tg()
    with tg.Com2D(64, dt=2e-4, defined=1) as s:
        s.set_state(gcom["smooth"])
        assert rel_l2(s.rhs(), gcom["rhs_smooth_defined"]) < 1e-12
        s.step(50)
        st = s.get_state()
    assert rel_l2(st, gcom["ab2_smooth_defined_50"]) < 1e-11


@gpu
def test_gpu_init_reference_golden(gcom):
    tg = _tg()
    with tg.Com2D(64) as s:
        s.init_reference(2.0, 2.0, 1.0)
        st, h = s.get_state(with_history=True)
    assert rel_l2(st, gcom["ic"]) < 1e-14
    assert np.abs(h).max() == 0.0


@gpu
@pytest.mark.parametrize("ny,nx,a", [(32, 64, 1.0), (64, 16, 0.0), (128, 256, 0.5), (16, 2048, 1.0),
                                      (2048, 16, 1.0),
                                      (96, 96, 1.0), (80, 48, 0.5), (60, 120, 1.0)])  # (mixed-radix lengths)
def test_gpu_rhs_rectangular_vs_oracle(oracle, ny, nx, a):
    """Rectangular grids and boxes, forcing on and off, against the oracle."""
    tg = _tg()
    sm = np.stack([np.zeros((ny, nx // 2 + 1), np.complex128)] * 6)
    rng = np.random.default_rng(nx * ny)
    xs, ys = np.meshgrid(np.arange(nx) * (2 * PI / nx), np.arange(ny) * (4 * PI / ny))
    base = [1.0, 0.0, 0.0, 1.5e4, 1.0, 1.0]
    amp = [0.05, 0.3, 0.3, 50.0, 0.3, 0.3]
    for f in range(6):
        g = base[f] + amp[f] * np.cos(rng.integers(1, 4) * xs + 0.5 * rng.integers(1, 4) * ys + rng.uniform(0, 6))
        sm[f] = oracle.r2c(g)
    p = orc.com_params(lx=2 * PI, ly=4 * PI, mu=2e-3, eta=5e-4, cs=100.0, kf=2.0, a=a)
    ref = oracle.derive2com(sm, p)
    with tg.Com2D(nx, ny, lx=2 * PI, ly=4 * PI, mu=2e-3, eta=5e-4, cs=100.0, kf=2.0, a=a) as s:
        s.set_state(sm)
        d = s.rhs()
    assert rel_l2(d, ref) < 1e-12


@gpu
def test_gpu_1024_rhs_and_steps_vs_oracle(oracle):
    """Full-size check from the driver's initial state at 1024^2: the state after
    20 AB2 steps against the oracle."""
    tg = _tg()
    st0 = oracle.ic_com(1024, 1024)
    p = orc.com_params()
    with tg.Com2D(1024, dt=2e-5) as s:
        s.init_reference(2.0, 2.0, 1.0)
        assert rel_l2(s.get_state(), st0) < 1e-13
        s.step(20)
        st = s.get_state()
    ref, _ = oracle.run_com(st0, p, 2e-5, 20)
    assert rel_l2(st, ref) < 1e-11


@gpu
def test_gpu_mixed_radix_96_steps_vs_oracle(oracle):
    """A 96^2 grid (mixed-radix transforms) from the driver's initial state: the
    state after 20 AB2 steps against the oracle (its direct DFT at this length)."""
    tg = _tg()
    st0 = oracle.ic_com(96, 96)
    p = orc.com_params()
    with tg.Com2D(96, dt=2e-5) as s:
        s.init_reference(2.0, 2.0, 1.0)
        assert rel_l2(s.get_state(), st0) < 1e-13
        s.step(20)
        st = s.get_state()
    ref, _ = oracle.run_com(st0, p, 2e-5, 20)
    assert rel_l2(st, ref) < 1e-11


@gpu
def test_gpu_nonfinite_is_reported(gcom):
    tg = _tg()
    st = gcom["smooth"].copy()
    st[4, 3, 4] = np.nan
    with tg.Com2D(64) as s:
        s.set_state(st)
        s.step(1)
        with pytest.raises(tg.TaraError) as e:
            s.synchronize()
        assert e.value.code == tg.TARA_ERR_NONFINITE
