"""3D compressible MHD (derive3com / ab3com): oracle pinning on CPU and GPU parity.

Tolerances (relative L2 over all eight spectra): transforms 1e-14; one RHS 1e-11
(the momentum flux carries P = CS^2 rho = 100 rho, whose gradient nearly cancels,
so rounding is amplified relative to the result); 5 AB2 steps 1e-11.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from oracle import oracle as orc

GOLDEN3D = ROOT / "tests" / "golden" / "golden3d.npz"


@pytest.fixture(scope="module")
def golden3d():
    return dict(np.load(GOLDEN3D))


def smooth_state(nx, ny, nz, seed, amp=0.05):
    """A deterministic smooth MHD state: rho ~ 1, |u|, |B| ~ 0.1 plus low-mode noise."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*(np.arange(n) * 2 * np.pi / n for n in (nz, ny, nx)), indexing="ij")
    fields = [1.0 + amp * np.cos(x + 2 * y) * np.sin(z),
              0.1 * np.sin(z) + amp * np.cos(y), 0.1 * np.sin(x) + amp * np.sin(z + x),
              0.1 * np.cos(y), 2.0 + 0 * x, 0.1 + amp * np.sin(y), 0.1 * np.cos(2 * x),
              0.1 + amp * np.cos(z)]
    out = []
    for f in fields:
        noise = rng.standard_normal(f.shape)
        spec = np.fft.rfftn(noise)
        kz, ky, kx = np.meshgrid(np.fft.fftfreq(nz, 1 / nz), np.fft.fftfreq(ny, 1 / ny),
                                 np.arange(nx // 2 + 1), indexing="ij")
        spec[(kx**2 + ky**2 + kz**2) > 9] = 0
        out.append(f + 1e-3 * np.fft.irfftn(spec, s=(nz, ny, nx), axes=(0, 1, 2)))
    return np.stack(out)


# ------------------------------------------------------------------ CPU: oracle
def test_fft3d_matches_numpy(oracle):
    rng = np.random.default_rng(1)
    x = rng.standard_normal((16, 32, 64))
    assert rel_l2(oracle.r2c3(x), np.fft.rfftn(x, axes=(0, 1, 2))) < 1e-15
    c = np.fft.rfftn(x, axes=(0, 1, 2)) + 0.3j * rng.standard_normal((16, 32, 33))
    ref = np.fft.irfftn(c, s=(16, 32, 64), axes=(0, 1, 2)) * x.size
    assert rel_l2(oracle.c2r3(c), ref) < 1e-15


def test_derive3com_oracle_golden(oracle, golden3d):
    p = orc.mhd_params()
    assert rel_l2(oracle.derive3com(golden3d["state0"], p), golden3d["derive_faithful"]) < 1e-12
    st, _ = oracle.run3d(golden3d["state0"], p, 1e-3, 5)
    assert rel_l2(st, golden3d["ab2_5"]) < 1e-12


def test_ic3d_spectrum_golden(oracle, golden3d):
    st = oracle.state_from_real(oracle.ic3d_abc(16, 16, 16))
    assert rel_l2(st, golden3d["state0"]) < 1e-15


@pytest.mark.skipif(not orc.available(fftw=True), reason="needs oracle/_ref (reference tree)")
def test_derive3com_own_fft_vs_fftw_defined_mode():
    own, ref = orc.load(), orc.load(fftw=True)
    real = smooth_state(16, 32, 16, 3)
    st = ref.state_from_real(real)
    p = orc.mhd_params(defined=1, nu_u=0.01, eta_b=0.01)
    assert rel_l2(own.derive3com(st, p), ref.derive3com(st, p)) < 1e-12


def test_ab3com_freezes_energy(oracle, golden3d):
    st = golden3d["state0"]
    d = oracle.derive3com(st, orc.mhd_params())
    new = oracle.ab3com(st, np.zeros_like(st), d, 1e-3)
    assert np.array_equal(new[4], st[4])
    assert rel_l2(new[1], st[1] + 1.5e-3 * d[1]) < 1e-15


# ------------------------------------------------------------------ GPU
gpu = pytest.mark.gpu


def _tg():
    import tara_gb300 as tg

    return tg


def _set_common(tg, lx=2 * orc.PI_R8, mu=0.01, eta=0.005, cs=10.0, dt=1e-3):
    c = tg.mhd_common()
    c.Lx = c.Ly = c.Lz = lx
    c.mu, c.eta, c.CS, c.dt = mu, eta, cs, dt


@gpu
def test_gpu_derive3com_golden(golden3d):
    tg = _tg()
    _set_common(tg)
    d = tg.derive3com(golden3d["state0"])
    assert rel_l2(d, golden3d["derive_faithful"]) < 1e-11


@gpu
def test_gpu_reference_loop_derive3com_ab3com(golden3d):
    """The reference loop of src/main3com.f95:536-614 through the drop-ins."""
    tg = _tg()
    _set_common(tg, dt=1e-3)
    st = golden3d["state0"].copy()
    old = np.zeros_like(st)
    for _ in range(5):
        new_d = tg.derive3com(st)
        st = tg.ab3com(st, old, new_d)
        old = new_d
    assert rel_l2(st, golden3d["ab2_5"]) < 1e-11


@gpu
def test_gpu_resident_ab2_golden(golden3d):
    tg = _tg()
    with tg.Solver3D(16, dt=1e-3) as s:
        s.set_state(golden3d["state0"])
        s.step(5)
        st = s.get_state()
    assert rel_l2(st, golden3d["ab2_5"]) < 1e-11


@gpu
@pytest.mark.parametrize("shape,defined", [((32, 32, 32), 0), ((16, 32, 64), 1), ((64, 16, 32), 1)])
def test_gpu_rhs_vs_oracle(oracle, shape, defined):
    tg = _tg()
    nz, ny, nx = shape
    real = smooth_state(nx, ny, nz, 7)
    st = oracle.state_from_real(real)
    p = orc.mhd_params(defined=defined, nu_u=0.01, eta_b=0.01)
    kw = dict(defined=defined, nu_u=0.01, eta_b=0.01)
    with tg.Solver3D(nx, ny, nz, **kw) as s:
        s.set_state(st)
        d = s.rhs()
    assert rel_l2(d, oracle.derive3com(st, p)) < 1e-11


@gpu
def test_gpu_set_state_real_matches_oracle_r2c(oracle):
    tg = _tg()
    real = smooth_state(32, 16, 16, 9)
    with tg.Solver3D(32, 16, 16) as s:
        s.set_state_real(real)
        st = s.get_state()
    assert rel_l2(st, oracle.state_from_real(real)) < 1e-14


@gpu
def test_gpu_128_cubed_rhs_and_steps(oracle):
    """Config-3 size (128^3): one full RHS against the oracle, then AB2 steps keep
    the state finite and conserve the mean density (k = 0 of d rho/dt is zero)."""
    tg = _tg()
    real = smooth_state(128, 128, 128, 3)
    st = oracle.state_from_real(real)
    p = orc.mhd_params(defined=1, nu_u=0.01, eta_b=0.01)
    with tg.Solver3D(128, defined=1, nu_u=0.01, eta_b=0.01, dt=1e-3) as s:
        s.set_state(st)
        assert rel_l2(s.rhs(), oracle.derive3com(st, p)) < 1e-11
        s.step(5)
        s.synchronize()
        out = s.get_state()
    assert np.all(np.isfinite(out.view(np.float64)))
    assert abs(out[0, 0, 0, 0] - st[0, 0, 0, 0]) < 1e-12 * abs(st[0, 0, 0, 0])


@gpu
@pytest.mark.parametrize("shape", [(512, 16, 16), (16, 512, 16), (16, 16, 512)])
def test_gpu_512_lines_rhs_vs_oracle(oracle, shape):
    """512-point transforms along each axis (the rows along x, the strided
    line passes along y and z) in a full right-hand side against the oracle,
    from the Orszag-Tang-type state (kmax 4 fits every axis of 16)."""
    tg = _tg()
    p = orc.mhd_params(defined=1, nu_u=0.01, eta_b=0.01)
    with tg.Solver3D(*shape, defined=1, nu_u=0.01, eta_b=0.01, dt=1e-3) as s:
        s.init_orszag_tang(0.01, 4, 3)
        st = s.get_state()
        d = s.rhs()
    assert rel_l2(st, oracle.ic3d_ot(*shape, amp=0.01, kmax=4, seed=3)) < 1e-13
    assert rel_l2(d, oracle.derive3com(st, p)) < 1e-11


@gpu
def test_gpu_512_cubed_steps():
    """512^3 (the largest 3D grid here, about 85 GB on the GPU): the
    benchmark's initial state, then AB2 steps stay finite and keep the mean
    density (the k = 0 mode of d rho/dt vanishes), and the magnetic and
    kinetic energies move by what a few steps of nu = eta = 0.01 allow."""
    tg = _tg()
    with tg.Solver3D(512, defined=1, nu_u=0.01, eta_b=0.01, dt=1e-3) as s:
        s.init_orszag_tang(0.01, 4, 3)
        d0 = s.diag()
        s.step(3)
        s.synchronize()
        d1 = s.diag()
        st = s.get_state()
        assert np.all(np.isfinite(st[:, ::7, ::7, ::7]))
        assert abs(st[0, 0, 0, 0] / 512.0**3 - 1.0) < 1e-12
        del st
    assert all(np.isfinite(d1))
    assert abs(d1[1] - d0[1]) < 0.05 * d0[1] and abs(d1[3] - d0[3]) < 0.05 * d0[3]
