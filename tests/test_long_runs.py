"""Parity at the benchmark configurations' full step counts, against fixtures made
by the FFTW-backed oracle (tests/golden/make_long_runs.py):

* plain 2D RK4, 1000 steps at 512^2 and 2048^2 (nu = 1e-4, dt = 5e-5, seeded
  random-phase vorticity): the vorticity on a 128^2 sub-lattice of the grid
  after 100 and 1000 steps within 1e-10 relative L2, energy and enstrophy within
  1e-10 relative;
* 3D compressible MHD, 500 AB2 steps at 64^3 and 128^3 from the Orszag-Tang-type
  initial state (nu = eta = 0.01, dt = 1e-3): each of the eight fields on a 16^3
  sub-lattice after 100 and 500 steps within 1e-10 relative L2;
* the 384-run ensemble: six of its runs (two per size) after 2000 RK4 steps,
  the FP64 batched path within 1e-10 and the FP32 form's error against the FP64
  oracle stated and bounded (1e-5).

The sub-lattice of a field is a linear function of its spectrum, so an error in
the state shows in it at about the same relative size.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ROOT, rel_l2

GOLD = ROOT / "tests" / "golden"
gpu = pytest.mark.gpu


def _load(name):
    path = GOLD / name
    if not path.exists():
        pytest.skip(f"{name} not generated")
    return dict(np.load(path))


def _omega_sub(w, n):
    """omega on the 128^2 sub-lattice of the grid from a half spectrum (the
    fixture's c2r / n^2; numpy's inverse drops the same imaginary parts)."""
    stride = n // 128
    return np.fft.irfft2(w, s=(n, n))[::stride, ::stride]


# the six ensemble runs of the fixture (tests/golden/make_long_runs.py)
ENS_RUNS, ENS_STEPS = (0, 1, 128, 129, 256, 257), 2000


def ensemble_run(r: int) -> tuple[int, float, int]:
    """(n, k0, seed) of run r of the 384-run ensemble (bench.py's run list)."""
    k0 = np.random.default_rng(4000).uniform(4.0, 10.0, 384)
    return (128, 256, 512)[r // 128], float(k0[r]), 4000 + r


# ---------------------------------------------------------------- CPU checks
def test_long_fixtures_are_consistent():
    """The fixtures decay as the physics says: energy and enstrophy fall, the
    vorticity stays finite, and the 3D density keeps its mean."""
    g = _load("long_rk4.npz")
    for n in (512, 2048):
        if f"n{n}_energy_1000" not in g:
            continue
        e = [float(g[f"n{n}_energy_{s}"]) for s in (0, 100, 1000)]
        z = [float(g[f"n{n}_enstrophy_{s}"]) for s in (0, 100, 1000)]
        assert abs(e[0] - 0.5) < 1e-12 and e[0] > e[1] > e[2] and z[0] > z[1] > z[2]
        assert np.all(np.isfinite(g[f"n{n}_omega_1000"]))
    g3 = _load("long_mhd3d.npz")
    for n in (64, 128):
        if f"mhd{n}_fields_500" not in g3:
            continue
        f0, f1 = g3[f"mhd{n}_fields_0"], g3[f"mhd{n}_fields_500"]
        assert np.allclose(f0[0], 1.0)
        assert np.all(np.isfinite(f1))


# ---------------------------------------------------------------- GPU parity
@gpu
@pytest.mark.parametrize("n", [512, 2048])
def test_rk4_1000_steps_vs_fftw_oracle(n):
    import tara_gb300 as tg

    g = _load("long_rk4.npz")
    if f"n{n}_omega_1000" not in g:
        pytest.skip(f"{n}^2 fixture not generated")
    seed = {512: 20240512, 2048: 20242048}[n]
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-4, dt=5e-5) as s:
        s.init_random(6.0, 0.5, seed)
        done = 0
        for step in (100, 1000):
            s.step(step - done)
            done = step
            e, z = s.diag()
            assert abs(e - float(g[f"n{n}_energy_{step}"])) < 1e-10 * abs(e)
            assert abs(z - float(g[f"n{n}_enstrophy_{step}"])) < 1e-10 * abs(z)
            err = rel_l2(_omega_sub(s.get_state(), n), g[f"n{n}_omega_{step}"])
            assert err < 1e-10, f"{n}^2 after {step} RK4 steps: {err:.3e}"


@gpu
def test_mhd3d_initial_state_matches_oracle(oracle):
    import tara_gb300 as tg

    for shape in ((32, 32, 32), (64, 32, 16)):
        with tg.Solver3D(*shape) as s:
            s.init_orszag_tang(0.01, 4, 3)
            st = s.get_state()
        ref = oracle.ic3d_ot(*shape, amp=0.01, kmax=4, seed=3)
        assert rel_l2(st, ref) < 1e-13


@gpu
@pytest.mark.parametrize("n", [64, 128])
def test_mhd3d_500_steps_vs_fftw_oracle(n):
    import tara_gb300 as tg

    g = _load("long_mhd3d.npz")
    if f"mhd{n}_fields_500" not in g:
        pytest.skip(f"{n}^3 fixture not generated")
    stride = n // 16
    names = ("rho", "rho ux", "rho uy", "rho uz", "E", "Bx", "By", "Bz")
    with tg.Solver3D(n, defined=1, nu_u=0.01, eta_b=0.01, dt=1e-3) as s:
        s.init_orszag_tang(0.01, 4, 3)
        done = 0
        for step in (0, 100, 500):
            s.step(step - done)
            done = step
            s.synchronize()
            st = s.get_state()
            fields = np.stack([np.fft.irfftn(f, s=(n, n, n), axes=(0, 1, 2))
                               for f in st])[:, ::stride, ::stride, ::stride]
            ref = g[f"mhd{n}_fields_{step}"]
            for f, name in enumerate(names):
                err = rel_l2(fields[f], ref[f])
                assert err < 1e-10, f"{n}^3 {name} after {step} AB2 steps: {err:.3e}"


@gpu
def test_ensemble_2000_steps_vs_fftw_oracle():
    """Six runs of the 384-run ensemble after 2000 RK4 steps: the batched FP64
    path matches the FP64 oracle to 1e-10; the FP32 form (FP32 transforms and
    products, FP64 state) states its error against the same oracle."""
    import tara_gb300 as tg

    g = _load("long_ensemble.npz")
    runs = [ensemble_run(r) for r in ENS_RUNS]
    errs = {}
    for prec in (tg.PREC_FP64, tg.PREC_FP32):
        with tg.Ensemble(runs, precision=prec, nu=1e-3, dt=1e-4) as e:
            e.step(ENS_STEPS)
            e.synchronize()
            for i, (r, (n, _, _)) in enumerate(zip(ENS_RUNS, runs)):
                errs[(prec, r)] = rel_l2(_omega_sub(e.get_state(i), n), g[f"run{r}_omega"])
    for r in ENS_RUNS:
        assert errs[(tg.PREC_FP64, r)] < 1e-10, (r, errs[(tg.PREC_FP64, r)])
        assert errs[(tg.PREC_FP32, r)] < 1e-5, (r, errs[(tg.PREC_FP32, r)])
    print({f"run {r} fp32 vs fp64 oracle": f"{errs[(tg.PREC_FP32, r)]:.2e}" for r in ENS_RUNS})
