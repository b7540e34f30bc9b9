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
            assert g["variants"][0] & 3 in (0, 1, 2) and g["variants"][1] & 3 in (0, 1, 2, 3)
            assert g["variants"][2] & 3 in (0, 1, 2)
            ms = np.array(g["tuned_ms"]).reshape(8, 3)
            for c in range(8):  # no tile variant 3 of the column passes
                assert (ms[c] > 0).tolist() == [c & 3 < 3, True, c & 3 < 3]
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
    for v in ((0, 0, 0), (1, 1, 1), (2, 2, 2), (2, 0, 1), (0, 3, 0)):
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
    for v in ((0, 0, 0), (1, 0, 2), (2, 2, 2), (1, 3, 0)):
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
        assert all(0 <= v < 8 for v in r["variants"])
        for c, row in enumerate(r["ms"]):  # the column passes have no tile variant 3
            assert [t > 0 for t in row] == [c & 3 < 3, True, c & 3 < 3], (c, row)


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512, 1024, 2048])
def test_radix8_path_rhs_matches_oracle(n, oracle):
    """The radix-8 path (configuration index + 4) of all three step kernels:
    one right-hand side against the oracle at every supported length (each
    length has its own mix of radix-8 and radix-4 stages)."""
    w0 = oracle.ic_random(n, n, 6.0, 0.5, 20240512 + n)
    ref = oracle.derive2csh(w0, 1e-3)
    for v in ((4, 4, 4), (5, 7, 6)):
        with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-4) as s:
            s.set_state(w0)
            s.set_variants(v)
            assert rel_l2(s.rhs(), ref) < 1e-12, (n, v)


@pytest.mark.parametrize("prec", [tg.PREC_FP64, tg.PREC_FP32])
def test_radix8_tiles_bitwise_and_close_to_radix4(prec):
    """On the radix-8 path every tile variant gives the same bits; against the
    radix-4 path the results differ only by rounding."""
    n = 256
    out = {}
    for v in ((0, 0, 0), (4, 4, 4), (5, 5, 5), (6, 6, 6), (4, 7, 4)):
        with tg.Solver2D(n, scheme=tg.SCHEME_RK4, precision=prec, nu=1e-3, dt=1e-4) as s:
            s.init_random(6.0, 0.5, 4100)
            s.set_variants(v)
            s.step(5)
            s.synchronize()
            out[v] = s.get_state()
    for v in ((5, 5, 5), (6, 6, 6), (4, 7, 4)):
        assert np.array_equal(out[v], out[(4, 4, 4)]), v
    tol = 1e-13 if prec == tg.PREC_FP64 else 1e-5
    assert rel_l2(out[(4, 4, 4)], out[(0, 0, 0)]) < tol


def test_radix8_rejected_for_double_float():
    with tg.Solver2D(64, precision=tg.PREC_DF64) as s:
        with pytest.raises(tg.TaraError):
            s.set_variants((4, 0, 0))


PRUNS = [(128, 4.0, 4000), (256, 6.0, 4001), (512, 8.5, 4002), (128, 10.0, 4003), (256, 5.0, 4004)]


def test_persistent_form_equals_graph_and_single_runs():
    """The persistent form (one cooperative launch for all steps of all sizes)
    runs the same CTA bodies as the per-pass kernels: on the radix-4 path it
    equals the graph form bit for bit, on the radix-8 path it equals single
    runs advanced with the radix-8 configurations bit for bit."""
    steps = 6
    out = {}
    for form in (tg.ENS_GRAPH, tg.ENS_PERSISTENT4, tg.ENS_PERSISTENT8):
        with tg.Ensemble(PRUNS, precision=tg.PREC_FP32, nu=1e-3, dt=1e-4) as e:
            e.set_form(form)
            e.step(steps - 2)  # two calls: the counter and descriptors are reset per launch
            e.step(2)
            e.synchronize()
            out[form] = [e.get_state(r) for r in range(len(PRUNS))]
            assert e.form()["form"] == ["graph", "persistent radix-4", "persistent radix-8"][form]
    for a, b in zip(out[tg.ENS_PERSISTENT4], out[tg.ENS_GRAPH]):
        assert np.array_equal(a, b)
    for r, (n, k0, seed) in enumerate(PRUNS):
        with tg.Solver2D(n, scheme=tg.SCHEME_RK4, precision=tg.PREC_FP32, nu=1e-3, dt=1e-4) as s:
            s.init_random(k0, 0.5, seed)
            s.set_variants((4, 4, 4))
            s.step(steps)
            s.synchronize()
            assert np.array_equal(out[tg.ENS_PERSISTENT8][r], s.get_state()), r
        assert rel_l2(out[tg.ENS_PERSISTENT8][r], out[tg.ENS_GRAPH][r]) < 1e-5


def test_persistent_form_refused_where_unsupported():
    with tg.Ensemble([(32, 5.0, 1), (128, 6.0, 2)], precision=tg.PREC_FP32) as e:
        with pytest.raises(tg.TaraError):
            e.set_form(tg.ENS_PERSISTENT4)  # 32^2 has no 256-thread tiles
    with tg.Ensemble([(128, 5.0, 1)], precision=tg.PREC_FP64) as e:
        with pytest.raises(tg.TaraError):
            e.set_form(tg.ENS_PERSISTENT4)  # FP32 form only


def test_autotune_times_every_form():
    with tg.Ensemble(PRUNS, precision=tg.PREC_FP32, nu=1e-3, dt=1e-4) as e:
        before = [e.get_state(r) for r in range(len(PRUNS))]
        e.autotune(2)
        f = e.form()
        assert all(v > 0 for v in f["ms_per_step"].values()), f
        after = [e.get_state(r) for r in range(len(PRUNS))]
        for a, b in zip(before, after):
            assert np.array_equal(a, b)
