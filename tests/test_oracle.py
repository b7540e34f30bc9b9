"""CPU tests of the oracle: pinned against the FFTW-generated golden vectors and
against closed-form known answers (no GPU)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel_l2


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for philox4x32-10
    assert oracle.philox((0, 0, 0, 0), (0, 0)) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2) == [
        0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle.philox((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344),
                         (0xA4093822, 0x299F31D0)) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_fft_matches_fftw_golden(oracle, golden):
    assert rel_l2(oracle.r2c(golden["fft_r2c_in"]), golden["fft_r2c_out"]) < 1e-15
    # c2r of a non-Hermitian spectrum: FFTW discards Im at kx = 0 and kx = Nx/2
    assert rel_l2(oracle.c2r(golden["fft_c2r_in"]), golden["fft_c2r_out"]) < 1e-15


@pytest.mark.parametrize("shape", [(16, 16), (64, 32), (32, 128), (256, 256)])
def test_fft_matches_numpy(oracle, shape):
    rng = np.random.default_rng(3)
    ny, nx = shape
    x = rng.standard_normal((ny, nx))
    assert rel_l2(oracle.r2c(x), np.fft.rfft2(x)) < 1e-15
    c = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
    # numpy's irfft2 uses the same rank-2 c2r order and discard rule
    assert rel_l2(oracle.c2r(c), np.fft.irfft2(c, s=(ny, nx)) * nx * ny) < 1e-15


def test_c2r_discards_imag_of_edge_bins(oracle):
    ny, nx = 16, 16
    c = np.zeros((ny, nx // 2 + 1), np.complex128)
    c[0, 0] = 1.0 + 5.0j        # imaginary part dropped after the y pass
    c[0, nx // 2] = 2.0 - 3.0j  # likewise at kx = Nx/2
    x = oracle.c2r(c)
    ref = np.full((ny, nx), 1.0) + 2.0 * np.cos(np.pi * np.arange(nx))[None, :]
    assert np.allclose(x, ref, atol=1e-13)


def test_ic_shear_and_spectrum(oracle, golden):
    w = oracle.ic_shear(64, 64, 2.0, 2.0, 25.0, 2.0, 0.0234375, variant=0)
    assert np.array_equal(w, golden["ic_real"])  # same libm, same expression order
    assert rel_l2(oracle.r2c(w), golden["ic_spec"]) < 1e-15


def test_rhs_matches_fftw_golden(oracle, golden):
    w0 = golden["ic_spec"]
    assert rel_l2(oracle.derive2csh(w0, 0.01), golden["rhs_plain"]) < 1e-13
    oracle.set_css_params(2 * np.float32(3.1428), 2 * np.float32(3.1428), 10.0)
    assert rel_l2(oracle.derive2css(w0, 1.0, 0.01), golden["rhs_screen"]) < 1e-13


@pytest.mark.parametrize("steps", [1, 10, 2000])
def test_ab2_run_matches_fftw_golden(oracle, golden, steps):
    w, fo = oracle.run(golden["ic_spec"], rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=steps)
    assert rel_l2(w, golden[f"ab2_plain_{steps}"]) < 1e-12
    assert rel_l2(fo, golden[f"ab2_plain_{steps}_hist"]) < 1e-12


def test_rk4_and_random_ic_match_fftw_golden(oracle, golden):
    wr = oracle.ic_random(64, 64, 6.0, 0.5, 20240512)
    assert rel_l2(wr, golden["ic_random"]) < 1e-14
    w, _ = oracle.run(golden["ic_random"], rhs=0, scheme=1, nu=1e-4, dt=5e-5, steps=10)
    assert rel_l2(w, golden["rk4_plain_10"]) < 1e-13
    oracle.set_css_params(2 * np.float32(3.1428), 2 * np.float32(3.1428), 10.0)
    assert rel_l2(oracle.rk42css(golden["ic_spec"], 1.0, 0.01, 1e-4), golden["rk42css_1"]) < 1e-13


def test_random_ic_energy_and_hermitian(oracle):
    w = oracle.ic_random(64, 64, 6.0, 0.5, 7)
    e, _ = oracle.energy_enstrophy(w)
    assert abs(e - 0.5) < 1e-13
    assert w[0, 0] == 0
    # kx = 0 column Hermitian in ky after the round-trip projection
    col = w[:, 0]
    assert np.allclose(col[1:], np.conj(col[1:][::-1]), atol=1e-14 * np.abs(col).max())


def test_single_mode_rhs_is_pure_viscous(oracle):
    # A single Fourier mode has u . grad(omega) = 0: dt omega_hat = -nu k^2 omega_hat.
    n = 32
    y, x = np.mgrid[0:n, 0:n] * (2 * np.pi / n)
    w = oracle.r2c(np.cos(3 * x + 2 * y))
    f = oracle.derive2csh(w, 0.05)
    ref = -0.05 * 13.0 * w
    assert np.abs(f - ref).max() < 1e-10 * np.abs(w).max()


def test_taylor_green_ab2_recurrence(oracle):
    # omega = 2 sin x cos y is an eigenmode (k^2 = 2) whose nonlinear term
    # vanishes, so AB2 reduces to the scalar recurrence w' = -2 nu w.
    n, nu, dt, steps = 32, 0.05, 1e-3, 50
    y, x = np.mgrid[0:n, 0:n] * (2 * np.pi / n)
    w0 = oracle.r2c(2 * np.sin(x) * np.cos(y))
    w, _ = oracle.run(w0, rhs=0, scheme=0, nu=nu, dt=dt, steps=steps)
    a, fo = 1.0, 0.0
    for _ in range(steps):
        f = -2 * nu * a
        a, fo = a + (1.5 * f - 0.5 * fo) * dt, f
    assert rel_l2(w, a * w0) < 1e-12
    # the zero history makes step 1 a 3/2-weighted Euler step: O(dt) start error
    assert abs(a - np.exp(-2 * nu * dt * steps)) < 1e-4


def test_parseval_energy(oracle, golden):
    e, z = oracle.energy_enstrophy(golden["ic_spec"])
    assert np.allclose([e, z], golden["energy_enstrophy_ic"], rtol=1e-13)
    w = golden["ic_spec"]
    n = 64
    ky = np.fft.fftfreq(n, 1.0 / n)[:, None]
    kx = np.arange(n // 2 + 1)[None, :]
    k2 = kx**2 + ky**2
    wt = np.where((kx == 0) | (kx == n // 2), 1.0, 2.0)
    k2s = np.where(k2 == 0, 1.0, k2)
    e_spec = 0.5 * np.sum(wt * np.abs(w) ** 2 / k2s * (k2 != 0)) / n**4
    z_spec = 0.5 * np.sum(wt * np.abs(w) ** 2) / n**4
    assert abs(e - e_spec) < 1e-12 * e and abs(z - z_spec) < 1e-12 * z


def grid_energy_rule(w):
    """Parseval with the c2r discard rule of the reference's transforms (the rule
    libtara's reduction implements): u_y of the kx = Nx/2 column and u_x of the
    ky = -Ny/2 row in the kx = 0 and kx = Nx/2 columns vanish on the grid."""
    ny, nh = w.shape
    nx = 2 * (nh - 1)
    ky = np.fft.fftfreq(ny, 1.0 / ny)[:, None]
    kx = np.arange(nh)[None, :].astype(float)
    k2 = kx**2 + ky**2
    edge = (kx == 0) | (kx == nx // 2)
    wt = np.where(edge, 1.0, 2.0)
    keep_ux = np.where(edge & (ky == -ny // 2), 0.0, ky**2)
    keep_uy = np.where(kx == nx // 2, 0.0, kx**2)
    k2s = np.where(k2 == 0, 1.0, k2)
    e = 0.5 * np.sum(wt * np.abs(w) ** 2 * (keep_ux + keep_uy) / k2s**2 * (k2 != 0)) / (nx * ny) ** 2
    z = 0.5 * np.sum(wt * np.abs(w) ** 2) / (nx * ny) ** 2
    return e, z


@pytest.mark.parametrize("n,seed", [(64, 20240512), (128, 3), (32, 9)])
def test_grid_energy_rule_matches_physical_space(oracle, n, seed):
    w = oracle.ic_random(n, n, 6.0 if n > 32 else 12.0, 0.5, seed)
    e, z = oracle.energy_enstrophy(w)
    er, zr = grid_energy_rule(w)
    assert abs(er - e) < 1e-14 * e and abs(zr - z) < 1e-14 * z
