"""GPU tests of batched ensembles of uneven grid sizes (tara_ens_*): a batched
run equals the same run advanced alone, the FP32-transform mode stays within
1e-5 of FP64 per run, the autotuner leaves the state untouched, and a run
matches the oracle."""
from __future__ import annotations

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2

pytestmark = pytest.mark.gpu

RUNS = [(64, 4.0, 4000), (32, 6.0, 4001), (128, 8.5, 4002), (64, 10.0, 4003), (32, 5.0, 4004),
        (128, 4.5, 4005)]


def test_batched_runs_equal_single_runs():
    steps = 7
    with tg.Ensemble(RUNS, precision=tg.PREC_FP64, nu=1e-3, dt=1e-4) as e:
        e.step(steps)
        e.synchronize()
        got = [e.get_state(r) for r in range(len(RUNS))]
    for r, (n, k0, seed) in enumerate(RUNS):
        with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-4) as s:
            s.init_random(k0, 0.5, seed)
            s.step(steps)
            ref = s.get_state()
        assert rel_l2(got[r], ref) < 1e-14, r


def test_fp32_ensemble_error_vs_fp64():
    steps = 50
    out = {}
    for prec in (tg.PREC_FP64, tg.PREC_FP32):
        with tg.Ensemble(RUNS, precision=prec, nu=1e-3, dt=1e-4) as e:
            e.step(steps)
            e.synchronize()
            out[prec] = [e.get_state(r) for r in range(len(RUNS))]
    errs = [rel_l2(a, b) for a, b in zip(out[tg.PREC_FP32], out[tg.PREC_FP64])]
    assert max(errs) < 1e-5, errs
    assert min(errs) > 0.0


def test_autotune_keeps_state_and_picks_variants():
    with tg.Ensemble(RUNS, precision=tg.PREC_FP32) as e:
        before = [e.get_state(r) for r in range(len(RUNS))]
        e.autotune(2)
        after = [e.get_state(r) for r in range(len(RUNS))]
        for a, b in zip(before, after):
            assert np.array_equal(a, b)
        groups = e.groups()
        assert sorted(g["n"] for g in groups) == [32, 64, 128]
        for g in groups:
            assert all(v in (0, 1, 2) for v in g["variants"])
            assert len(g["tuned_ms"]) == 9 and all(t > 0 for t in g["tuned_ms"])
        e.step(3)  # graph captured with the chosen variants
        e.synchronize()
        assert e.launches_per_step == 3 * 12


def test_ensemble_run_matches_oracle(oracle):
    with tg.Ensemble([(64, 6.0, 20240512)], precision=tg.PREC_FP64, nu=1e-4, dt=5e-5) as e:
        w0 = e.get_state(0)
        e.step(10)
        e.synchronize()
        w = e.get_state(0)
    assert rel_l2(w0, oracle.ic_random(64, 64, 6.0, 0.5, 20240512)) < 1e-13
    ref, _ = oracle.run(w0, rhs=0, scheme=1, nu=1e-4, dt=5e-5, steps=10)
    assert rel_l2(w, ref) < 1e-12


@pytest.mark.parametrize("n", [64, 256, 32, 128])
@pytest.mark.parametrize("prec", [tg.PREC_FP64, tg.PREC_FP32])
def test_tile_variants_are_bitwise_equal(n, prec):
    """Every tile variant runs the same per-column / per-row arithmetic (odd
    log2 n adds the final radix-2 stage)."""
    out = []
    for v in ((0, 0, 0), (1, 1, 1), (2, 2, 2), (2, 0, 1)):
        with tg.Solver2D(n, scheme=tg.SCHEME_RK4, precision=prec, nu=1e-3, dt=1e-4) as s:
            s.init_random(6.0, 0.5, 4100)
            s.set_variants(v)
            s.step(3)
            s.synchronize()
            out.append(s.get_state())
    for o in out[1:]:
        assert np.array_equal(o, out[0])


def test_tile_variants_at_2048_are_bitwise_equal():
    """At the bench's 2048^2 FP64 RK4 workload the autotuner picks per-kernel
    variants such as (1, 0, 2); they give the default tiles' results bit for bit."""
    out = []
    for v in ((0, 0, 0), (1, 0, 2), (2, 2, 2)):
        with tg.Solver2D(2048, scheme=tg.SCHEME_RK4, nu=1e-4, dt=5e-5) as s:
            s.init_random(6.0, 0.5, 20242048)
            s.set_variants(v)
            s.step(1)
            s.synchronize()
            out.append(s.get_state())
    for o in out[1:]:
        assert np.array_equal(o, out[0])


def test_solver_autotune_restores_state():
    with tg.Solver2D(128, scheme=tg.SCHEME_AB2, nu=1e-3, dt=1e-4) as s:
        s.init_random(6.0, 0.5, 4101)
        s.step(2)
        w, fo = s.get_state(with_history=True)
        r = s.autotune(2)
        w2, fo2 = s.get_state(with_history=True)
        assert np.array_equal(w, w2) and np.array_equal(fo, fo2)
        assert all(v in (0, 1, 2) for v in r["variants"])
        assert all(t > 0 for row in r["ms"] for t in row)
