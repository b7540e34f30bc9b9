"""2D compressible isothermal hydro (src/derive2coh.f95, src/ab2coh.f95).

CPU: the own-FFT oracle against the FFTW-oracle golden vectors
(tests/golden/golden_coh.npz, tests/golden/make_golden.py).
GPU: the drop-ins derive2coh_ / ab2coh_ (common block /comm/ set through
libtara's comm_) and the device-resident Coh2D solver against the same vectors
and the oracle.  Tolerances (relative L2): one RHS 1e-12, 2000 AB2 steps 1e-10,
the initial state 1e-13.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import ROOT, rel_l2
from oracle import oracle as orc

GOLDEN_COH = ROOT / "tests" / "golden" / "golden_coh.npz"
PI = orc.PI_R8


@pytest.fixture(scope="module")
def gcoh():
    return dict(np.load(GOLDEN_COH))


def _smooth(n_y, n_x, seed, amp=40.0):
    rng = np.random.default_rng(seed)
    nh = n_x // 2 + 1
    ky = np.fft.fftfreq(n_y, 1.0 / n_y)[:, None]
    kx = np.arange(nh)[None, :]
    env = np.exp(-(kx**2 + ky**2) / 18.0)
    st = np.stack([env * (rng.standard_normal((n_y, nh)) + 1j * rng.standard_normal((n_y, nh)))
                   for _ in range(3)]) * amp
    st[0, 0, 0] = n_x * n_y
    return st


# ------------------------------------------------------------------ CPU (oracle)
def test_oracle_ic_golden(oracle, gcoh):
    assert rel_l2(oracle.ic_coh(64, 64), gcoh["ic"]) < 1e-13


def test_oracle_derive2coh_golden(oracle, gcoh):
    assert rel_l2(oracle.derive2coh(gcoh["ic"], orc.coh_params()), gcoh["rhs_ic"]) < 1e-13
    p = orc.coh_params(mux=1e-3, muy=5e-4, cs=2.0)
    assert rel_l2(oracle.derive2coh(gcoh["smooth"], p), gcoh["rhs_smooth"]) < 1e-13


def test_oracle_run_golden(oracle, gcoh):
    for steps in (10, 2000):
        st, h = oracle.run_coh(gcoh["ic"], orc.coh_params(), 1e-3, steps)
        assert rel_l2(st, gcoh[f"ab2_{steps}"]) < 1e-11
        assert rel_l2(h, gcoh[f"ab2_{steps}_hist"]) < 1e-11


def test_oracle_rhs_properties(oracle):
    """A uniform state at rest has no tendency; a uniform flow only advects."""
    n = 32
    st = np.zeros((3, n, n // 2 + 1), np.complex128)
    st[0, 0, 0] = n * n
    assert np.abs(oracle.derive2coh(st, orc.coh_params())).max() == 0.0
    st[1, 0, 0] = 0.5 * n * n  # ux = 0.5 everywhere
    d = oracle.derive2coh(st, orc.coh_params())
    assert np.abs(d).max() < 1e-9


# ------------------------------------------------------------------ GPU
gpu = pytest.mark.gpu


def _tg():
    import tara_gb300 as tg

    return tg


def _set_common(tg, lx=2 * PI, ly=2 * PI, mux=2e-4, muy=2e-4, cs=3.77, dt=1e-3):
    c = tg.coh_common()
    c.Lx, c.Ly, c.mux, c.muy, c.ms, c.CS, c.dt = lx, ly, mux, muy, 1.0, cs, dt


@gpu
def test_gpu_derive2coh_golden(gcoh):
    tg = _tg()
    _set_common(tg)
    assert rel_l2(tg.derive2coh(gcoh["ic"]), gcoh["rhs_ic"]) < 1e-12
    _set_common(tg, mux=1e-3, muy=5e-4, cs=2.0)
    assert rel_l2(tg.derive2coh(gcoh["smooth"]), gcoh["rhs_smooth"]) < 1e-12


@gpu
def test_gpu_reference_loop_golden(gcoh):
    """The driver loop of src/main2coh.f95:263-298 through the two drop-ins."""
    tg = _tg()
    _set_common(tg, dt=1e-3)
    st = gcoh["ic"].copy()
    old = np.zeros_like(st)
    for _ in range(10):
        new = tg.derive2coh(st)
        st = tg.ab2coh(st, old, new)
        old = new
    assert rel_l2(st, gcoh["ab2_10"]) < 1e-12
    assert rel_l2(old, gcoh["ab2_10_hist"]) < 1e-12


@gpu
def test_gpu_ab2coh_matches_oracle(oracle, gcoh):
    tg = _tg()
    _set_common(tg, dt=2.5e-3)
    st = gcoh["smooth"]
    d_old = _smooth(64, 64, 5, amp=3.0)
    d_new = _smooth(64, 64, 6, amp=3.0)
    ref = oracle.ab2coh(st, d_old, d_new, 2.5e-3)
    assert rel_l2(tg.ab2coh(st, d_old, d_new), ref) < 1e-15


@gpu
@pytest.mark.parametrize("steps", [1, 10, 2000])
def test_gpu_solver_ab2_golden(gcoh, steps):
    tg = _tg()
    with tg.Coh2D(64, dt=1e-3) as s:
        s.set_state(gcoh["ic"])
        s.step(steps)
        st, h = s.get_state(with_history=True)
    assert rel_l2(st, gcoh[f"ab2_{steps}"]) < 1e-10
    assert rel_l2(h, gcoh[f"ab2_{steps}_hist"]) < 1e-10


@gpu
def test_gpu_init_vortices_golden(gcoh):
    tg = _tg()
    with tg.Coh2D(64) as s:
        s.init_vortices(2.0, 2.0)
        st, h = s.get_state(with_history=True)
    assert rel_l2(st, gcoh["ic"]) < 1e-13
    assert np.abs(h).max() == 0.0


@gpu
@pytest.mark.parametrize("ny,nx", [(32, 64), (64, 16), (128, 256), (16, 2048), (2048, 16),
                                   (96, 96), (80, 48), (60, 120)])  # (mixed-radix lengths)
def test_gpu_rhs_rectangular_vs_oracle(oracle, ny, nx):
    tg = _tg()
    st = _smooth(ny, nx, nx + ny)
    p = orc.coh_params(lx=2 * PI, ly=4 * PI, mux=5e-4, muy=1e-3, cs=3.0)
    ref = oracle.derive2coh(st, p)
    with tg.Coh2D(nx, ny, lx=2 * PI, ly=4 * PI, mux=5e-4, muy=1e-3, cs=3.0) as s:
        s.set_state(st)
        d = s.rhs()
    assert rel_l2(d, ref) < 1e-12


@gpu
def test_gpu_1024_rhs_and_steps_vs_oracle(oracle):
    """Full-size check: the driver's initial state at 1024^2, one RHS and 20 AB2
    steps against the oracle."""
    tg = _tg()
    st0 = oracle.ic_coh(1024, 1024)
    p = orc.coh_params()
    with tg.Coh2D(1024, dt=5e-4) as s:
        s.init_vortices(2.0, 2.0)
        assert rel_l2(s.get_state(), st0) < 1e-13
        assert rel_l2(s.rhs(), oracle.derive2coh(st0, p)) < 1e-12
        s.step(20)
        st = s.get_state()
    ref, _ = oracle.run_coh(st0, p, 5e-4, 20)
    assert rel_l2(st, ref) < 1e-11


@gpu
def test_gpu_nonfinite_is_reported(gcoh):
    tg = _tg()
    st = gcoh["ic"].copy()
    st[1, 3, 4] = np.nan
    with tg.Coh2D(64) as s:
        s.set_state(st)
        s.step(1)
        with pytest.raises(tg.TaraError) as e:
            s.synchronize()
        assert e.value.code == tg.TARA_ERR_NONFINITE


@gpu
def test_gpu_dropin_rejects_bad_common():
    tg = _tg()
    _set_common(tg, lx=0.0)
    with pytest.raises(tg.TaraError):
        tg.derive2coh(np.zeros((3, 32, 17), np.complex128))
    _set_common(tg)


@gpu
def test_gpu_mixed_radix_96_steps_vs_oracle(oracle):
    """A 96^2 grid (mixed-radix transforms): the driver's initial state and 20
    AB2 steps against the oracle (its direct DFT at this length)."""
    tg = _tg()
    st0 = oracle.ic_coh(96, 96)
    p = orc.coh_params()
    with tg.Coh2D(96, dt=5e-4) as s:
        s.init_vortices(2.0, 2.0)
        assert rel_l2(s.get_state(), st0) < 1e-13
        assert rel_l2(s.rhs(), oracle.derive2coh(st0, p)) < 1e-12
        s.step(20)
        st = s.get_state()
    ref, _ = oracle.run_coh(st0, p, 5e-4, 20)
    assert rel_l2(st, ref) < 1e-11
