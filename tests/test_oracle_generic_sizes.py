"""CPU: the oracle's own transform at lengths that are not powers of two (its
direct DFT over the long-double root table) against the FFTW-backed fixtures
of tests/golden/make_generic_sizes.py -- the reference's shear layer at 96^2,
seeded random states at 48 x 80 and 56 x 84 (factors 3, 5 and 7).  This pins
the oracle the GPU's mixed-radix path is tested against.  Tolerances (relative
L2): one RHS 1e-14, runs 1e-13."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

GOLD = Path(__file__).resolve().parent / "golden" / "generic_sizes.npz"


@pytest.fixture(scope="module")
def gen():
    return np.load(GOLD)


@pytest.mark.parametrize("key,nu", [("s96", 0.01), ("r48x80", 1e-3), ("r56x84", 1e-3)])
def test_oracle_rhs_matches_fftw_fixture(oracle, gen, key, nu):
    assert rel_l2(oracle.derive2csh(gen[f"{key}_w0"], nu), gen[f"{key}_rhs"]) < 1e-14


def test_oracle_runs_match_fftw_fixtures(oracle, gen):
    w, _ = oracle.run(gen["s96_w0"], rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=500)
    assert rel_l2(w, gen["s96_w500"]) < 1e-13
    w, _ = oracle.run(gen["r48x80_w0"], rhs=0, scheme=1, nu=1e-3, dt=1e-3, steps=200)
    assert rel_l2(w, gen["r48x80_w200"]) < 1e-13
    w, _ = oracle.run(gen["r56x84_w0"], rhs=0, scheme=1, nu=1e-3, dt=1e-3, steps=100)
    assert rel_l2(w, gen["r56x84_w100"]) < 1e-13


@pytest.mark.parametrize("ny,nx", [(84, 56), (70, 42), (112, 112)])
def test_oracle_transforms_invert_at_factor_7_lengths(oracle, ny, nx):
    rng = np.random.default_rng(nx + ny)
    x = rng.standard_normal((ny, nx))
    assert rel_l2(oracle.c2r(oracle.r2c(x)) / (nx * ny), x) < 1e-14
    k = np.fft.rfft2(x)
    assert rel_l2(oracle.r2c(x), k) < 1e-14


@pytest.mark.parametrize("ny,nx", [(45, 45), (27, 50), (50, 27), (33, 35), (64, 63)])
def test_oracle_transforms_at_odd_lengths(oracle, ny, nx):
    """Odd lengths (which the reference's FFTW takes and the GPU path refuses):
    the oracle's r2c and c2r against numpy's pocketfft, whose c2r keeps FFTW's
    semantics (a complex inverse along y, then a c2r along x that reads only the
    real part of the self-conjugate bins: kx = 0, and kx = Nx/2 for even Nx)."""
    rng = np.random.default_rng(nx * 100 + ny)
    x = rng.standard_normal((ny, nx))
    assert rel_l2(oracle.r2c(x), np.fft.rfft2(x)) < 1e-14
    c = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
    assert rel_l2(oracle.c2r(c, nx), np.fft.irfft2(c, s=(ny, nx)) * (nx * ny)) < 1e-14
