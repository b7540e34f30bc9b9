"""GPU tests of the mixed-radix FP64 path: the grid sizes the reference accepts
beyond powers of two (src/main2csh.f95:35-38 reads any Nx, Ny; FFTW transforms
any length), here even lengths up to 3600 whose prime factors are 2, 3, 5 and 7.

Against the FFTW-backed fixtures (tests/golden/make_generic_sizes.py): the RHS
and 500 AB2 steps from the reference's shear layer at 96^2, the RHS and 200 RK4
steps from a seeded random-phase state at 48 x 80, the RHS and 100 RK4 steps
at 56 x 84 (a factor 7 on both axes).  Against the oracle (its
direct DFT at these lengths, itself pinned to the same fixtures on the CPU):
transforms, one RHS of both kinds, and steps at several shapes.  At sizes the
oracle's direct DFT would take long, properties: the c2r of the r2c returns
Nx Ny times the field, and the energy decays with the RHS's viscous term only.
Tolerances as for the power-of-two path: transforms 1e-14, one RHS 1e-12, runs
1e-10 (relative L2)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

pytestmark = pytest.mark.gpu
PI_R4 = tg.PI_R4
GOLD = Path(__file__).resolve().parent / "golden" / "generic_sizes.npz"


@pytest.fixture(scope="module")
def gen():
    return np.load(GOLD)


@pytest.fixture(autouse=True)
def _reset_css():
    tg.set_css_params(2 * PI_R4, 2 * PI_R4, 10.0)
    yield
    tg.set_css_params(2 * PI_R4, 2 * PI_R4, 10.0)


def test_fixtures_rhs_and_runs(gen):
    assert rel_l2(tg.derive2csh(gen["s96_w0"], 0.01), gen["s96_rhs"]) < 1e-12
    assert rel_l2(tg.derive2csh(gen["r48x80_w0"], 1e-3), gen["r48x80_rhs"]) < 1e-12
    with tg.Solver2D(96, nu=0.01, dt=1e-4) as s:
        s.set_state(gen["s96_w0"])
        s.step(500)
        assert rel_l2(s.get_state(), gen["s96_w500"]) < 1e-10
    with tg.Solver2D(48, 80, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as s:
        s.set_state(gen["r48x80_w0"])
        s.step(200)
        assert rel_l2(s.get_state(), gen["r48x80_w200"]) < 1e-10
    assert rel_l2(tg.derive2csh(gen["r56x84_w0"], 1e-3), gen["r56x84_rhs"]) < 1e-12
    with tg.Solver2D(56, 84, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as s:
        s.set_state(gen["r56x84_w0"])
        s.step(100)
        assert rel_l2(s.get_state(), gen["r56x84_w100"]) < 1e-10


@pytest.mark.parametrize("ny,nx", [(96, 96), (80, 48), (40, 30), (90, 120), (384, 384), (50, 200), (8, 12),
                                   (84, 56), (70, 42), (14, 28), (448, 336)])
def test_transforms_vs_oracle(oracle, ny, nx):
    rng = np.random.default_rng(nx * 3 + ny)
    x = rng.standard_normal((ny, nx))
    assert rel_l2(tg.fft2d_r2c(x), oracle.r2c(x)) < 1e-14
    c = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
    assert rel_l2(tg.fft2d_c2r(c), oracle.c2r(c)) < 1e-14


@pytest.mark.parametrize("ny,nx", [(96, 96), (80, 48), (40, 30), (90, 120), (384, 384), (64, 96), (96, 64),
                                   (84, 56), (112, 112), (64, 98)])
def test_rhs_vs_oracle(oracle, ny, nx):
    """One RHS of each kind; (64, 96) and (96, 64) mix a power-of-two axis with
    a mixed-radix one (the whole grid takes the mixed-radix path)."""
    rng = np.random.default_rng(7 * nx + ny)
    w = oracle.r2c(rng.standard_normal((ny, nx)))
    assert rel_l2(tg.derive2csh(w, 1e-3), oracle.derive2csh(w, 1e-3)) < 1e-12
    oracle.set_css_params(2 * PI_R4, 2 * PI_R4, 10.0)
    assert rel_l2(tg.derive2css(w, 0.7, 1e-3), oracle.derive2css(w, 0.7, 1e-3)) < 1e-12


@pytest.mark.parametrize("scheme,rhs", [(tg.SCHEME_AB2, tg.RHS_PLAIN), (tg.SCHEME_RK4, tg.RHS_PLAIN),
                                        (tg.SCHEME_AB2, tg.RHS_SCREEN)])
def test_solver_steps_vs_oracle(oracle, scheme, rhs):
    w0 = oracle.ic_random(120, 90, 5.0, 0.5, 31)
    ref, _ = oracle.run(w0, rhs=rhs, scheme=1 if scheme == tg.SCHEME_RK4 else 0, alpha=1.0, nu=1e-3, dt=1e-3,
                        steps=50)
    with tg.Solver2D(120, 90, scheme=scheme, rhs=rhs, nu=1e-3, dt=1e-3, alpha=1.0, lam=10.0) as s:
        s.set_state(w0)
        s.step(50)
        assert rel_l2(s.get_state(), ref) < 1e-10


def test_dropins_and_rk4_dropin(gen, oracle):
    w = gen["s96_w0"]
    fn = tg.derive2csh(w, 0.01)
    fo = oracle.derive2csh(oracle.run(w, rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=1)[0], 0.01)
    assert rel_l2(tg.ab2csh(w, fo, fn, 1e-4), oracle.ab2(w, fo, fn, 1e-4)) < 1e-14
    assert rel_l2(tg.rk42css(w, 1.0, 0.01, 1e-4), oracle.rk42css(w, 1.0, 0.01, 1e-4)) < 1e-12


@pytest.mark.parametrize("n", [1536, 2000, 1792, 3000, 3600])
def test_large_mixed_radix_properties(n):
    """Lengths whose oracle DFT would take minutes: the c2r of the r2c is Nx Ny
    times the field, and a plain RK4 run keeps the mean vorticity and loses
    energy at a rate the viscous term bounds."""
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n // 2, n))
    back = tg.fft2d_c2r(tg.fft2d_r2c(x)) / (x.shape[0] * x.shape[1])
    assert rel_l2(back, x) < 1e-14
    with tg.Solver2D(n, n // 2, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as s:
        s.init_random(6.0, 0.5, 99)
        e0, _ = s.diag()
        w0 = s.get_state()
        s.step(20)
        e1, _ = s.diag()
        w1 = s.get_state()
    # (the spectrum is unnormalised: the mean mode moves by rounding only, far
    # below the state's norm)
    assert abs(w1[0, 0] - w0[0, 0]) < 1e-15 * np.linalg.norm(w0)
    assert 0.0 < e1 < e0


def test_driver_runs_a_96_grid(tmp_path, oracle):
    """The `tara` driver accepts Nx = Ny = 96 and its first-step snapshot matches
    the oracle's run of the reference's initial state."""
    ini = """[dimension]
dim = 2
[architecture]
arch = cpu
[parallel]
mode = serial
[type]
domain = hydro
[problem]
hydrotype = bare
[particle]
Np = 0
[grid]
Nx = 96
Ny = 96
Nz = 64
[length]
Lx = 2.0d0
Ly = 2.0d0
Lz = 2.0d0
[resistivity]
nu = 0.010d0
eta = 0.0d0
[time]
time_min = 0.0d0
time_max = 2.0d0
dt = 0.00010d0
[initialProfile]
W0 = 25.0d0
m0 = 2.0d0
d = 0.0234375d0
"""
    (tmp_path / "input.ini").write_text(ini)
    out = tmp_path / "output"
    rc = tg.lib().tara_run_ini(str(tmp_path / "input.ini").encode(), str(out).encode(), 3)
    assert rc == tg.TARA_OK, tg.last_error()
    snap = np.array([[float(v) for v in line.split()] for line in (out / "fort.00000100").read_text().splitlines()])
    assert snap.shape == (96 * 96, 5)
    w0 = oracle.r2c(oracle.ic_shear(96, 96, 2.0, 2.0, 25.0, 2.0, 0.0234375, variant=1))
    w, _ = oracle.run(w0, rhs=0, scheme=0, nu=0.01, dt=1e-4, steps=1)
    om = oracle.c2r(w) / (96 * 96)
    assert np.abs(snap[:, 2] - om.T.ravel()).max() < 1e-10 * np.abs(om).max()
