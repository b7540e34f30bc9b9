"""GPU tests of the double-float form (TARA_PREC_DF64): transforms and spectral
products in pairs of FP32 numbers (about 48 significant bits), state, update and
reductions in FP64.  It is held to the FP64 path's own bars against the oracle:
2000 AB2 steps within 1e-10, one RHS and a few RK4 steps within 1e-12; against
the FP64 path within 1e-12 after 50 RK4 steps; tile variants and batched runs
bitwise equal to one another."""
from __future__ import annotations

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

pytestmark = pytest.mark.gpu

DF = tg.PREC_DF64


@pytest.fixture(autouse=True)
def _reset_css():
    tg.set_css_params(2 * tg.PI_R4, 2 * tg.PI_R4, 10.0)
    yield
    tg.set_css_params(2 * tg.PI_R4, 2 * tg.PI_R4, 10.0)


@pytest.mark.parametrize("steps", [10, 2000])
def test_df64_ab2_plain_golden(golden, steps):
    with tg.Solver2D(64, nu=0.01, dt=1e-4, precision=DF) as s:
        s.set_state(golden["ic_spec"])
        s.step(steps)
        w, fo = s.get_state(with_history=True)
    assert rel_l2(w, golden[f"ab2_plain_{steps}"]) < 1e-10
    assert rel_l2(fo, golden[f"ab2_plain_{steps}_hist"]) < 1e-10


def test_df64_ab2_screen_golden(golden):
    with tg.Solver2D(64, rhs=tg.RHS_SCREEN, nu=0.01, dt=1e-4, alpha=1.0, lam=10.0, precision=DF) as s:
        s.set_state(golden["ic_spec"])
        s.step(2000)
        w = s.get_state()
    assert rel_l2(w, golden["ab2_screen_2000"]) < 1e-10


def test_df64_rk4_512_vs_oracle(oracle):
    w0 = oracle.ic_random(512, 512, 6.0, 0.5, 20240512)
    ref, _ = oracle.run(w0, rhs=0, scheme=1, nu=1e-4, dt=5e-5, steps=5)
    with tg.Solver2D(512, scheme=tg.SCHEME_RK4, nu=1e-4, dt=5e-5, precision=DF) as s:
        s.set_state(w0)
        s.step(5)
        w = s.get_state()
    assert rel_l2(w, ref) < 1e-12


def test_df64_rhs_2048_vs_oracle(oracle):
    with tg.Solver2D(2048, scheme=tg.SCHEME_RK4, nu=1e-4, dt=5e-5, precision=DF) as s:
        s.init_random(6.0, 0.5, 20242048)
        w0 = s.get_state()
        f = s.rhs()
    assert rel_l2(f, oracle.derive2csh(w0, 1e-4)) < 1e-12


def test_df64_error_vs_fp64(oracle):
    """The double-float form tracks the FP64 path to 1e-12 (the FP32 form: 1e-5)."""
    w0 = oracle.ic_random(256, 256, 6.0, 0.5, 4000)
    out = []
    for prec in (tg.PREC_FP64, DF):
        with tg.Solver2D(256, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-4, precision=prec) as s:
            s.set_state(w0)
            s.step(50)
            out.append(s.get_state())
    err = rel_l2(out[1], out[0])
    assert 0.0 < err < 1e-12


@pytest.mark.parametrize("n", [64, 256, 128])
def test_df64_tile_variants_are_bitwise_equal(n):
    out = []
    for v in ((0, 0, 0), (1, 1, 1), (2, 2, 2), (2, 0, 1), (0, 3, 0)):
        with tg.Solver2D(n, scheme=tg.SCHEME_RK4, precision=DF, nu=1e-3, dt=1e-4) as s:
            s.init_random(6.0, 0.5, 4100)
            s.set_variants(v)
            s.step(3)
            s.synchronize()
            out.append(s.get_state())
    for o in out[1:]:
        assert np.array_equal(o, out[0])


def test_df64_ensemble_equals_single_runs():
    runs = [(64, 4.0, 4000), (32, 6.0, 4001), (128, 8.5, 4002), (64, 10.0, 4003)]
    with tg.Ensemble(runs, precision=DF, nu=1e-3, dt=1e-4) as e:
        e.step(7)
        e.synchronize()
        got = [e.get_state(r) for r in range(len(runs))]
    for r, (n, k0, seed) in enumerate(runs):
        with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-4, precision=DF) as s:
            s.init_random(k0, 0.5, seed)
            s.step(7)
            ref = s.get_state()
        assert np.array_equal(got[r], ref), r


@pytest.mark.parametrize("value", [np.nan, np.inf])
def test_df64_nonfinite_state_is_reported(golden, value):
    w = golden["ic_spec"].copy()
    w[3, 4] = value
    with tg.Solver2D(64, precision=DF) as s:
        s.set_state(w)
        s.step(1)
        with pytest.raises(tg.TaraError) as e:
            s.synchronize()
        assert e.value.code == tg.TARA_ERR_NONFINITE


def test_df64_tiny_and_huge_spectra(oracle):
    """States scaled by 1e-10 and 1e+10 keep the FP64 bars.  (The double-float
    form has FP32's exponent range: the unnormalised products, about
    N^4 |u| |grad w|, must stay below 3e38, and parts below 2^-126 flush.)"""
    w0 = oracle.ic_random(64, 64, 6.0, 0.5, 4200)
    for scale in (1e-10, 1e10):
        ref, _ = oracle.run(w0 * scale, rhs=0, scheme=1, nu=1e-3, dt=1e-4 / max(1.0, scale), steps=3)
        with tg.Solver2D(64, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-4 / max(1.0, scale), precision=DF) as s:
            s.set_state(w0 * scale)
            s.step(3)
            w = s.get_state()
        assert rel_l2(w, ref) < 1e-12, scale
