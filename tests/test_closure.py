"""GPU tests of the learned-closure pieces around the plain solver: the box
filter and subgrid flux, shell spectra, real-space state input, and the
closure stepper (FNO flux -> -div flux added to every RK4 stage) against the
CPU oracles (oracle/oracle.py for the RHS, oracle/fno_oracle.py for the
network, filter and spectrum)."""
from __future__ import annotations

import numpy as np
import pytest

import tara_gb300 as tg
from conftest import rel_l2
from oracle import fno_oracle as fo

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _real(w, n):
    return np.fft.irfft2(w, s=(n, n))


def test_filter_matches_oracle():
    n, f = 256, 8
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-4, dt=1e-4, batch=2) as s:
        s.init_random(8.0, 0.5, 77, run=0)
        s.init_random(6.0, 0.5, 78, run=1)
        w = s.get_state_run(1)
        nc = n // f
        wb = torch.zeros((nc, nc), dtype=torch.float32, device="cuda")
        fl = torch.zeros((nc, nc, 2), dtype=torch.float32, device="cuda")
        wb64 = torch.zeros((nc, nc), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()  # the solver's stream does not wait on torch's stream
        s.filter(1, f, wb.data_ptr(), fl.data_ptr(), wb64.data_ptr())
        ref_wb, ref_fl = fo.box_filter(_real(w, n), f)
        assert rel_l2(wb64.cpu().numpy(), ref_wb) < 1e-13
        assert rel_l2(wb.cpu().numpy(), ref_wb) < 1e-6
        assert rel_l2(fl.cpu().numpy(), ref_fl) < 1e-6


def test_spectrum_matches_oracle_and_energy():
    n = 128
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-4, dt=1e-4) as s:
        s.init_random(8.0, 0.5, 79)
        E = s.spectrum(0, kmax=n)  # covers |k| <= sqrt(2) n/2
        ref = fo.shell_spectrum(_real(s.get_state(), n), n)
        assert rel_l2(E, ref) < 1e-12
        e, _ = s.diag()
        assert abs(E.sum() - e) < 1e-10 * e


def test_set_state_real_round_trip(oracle):
    n = 64
    rng = np.random.default_rng(80)
    w = rng.standard_normal((n, n))
    with tg.Solver2D(n) as s:
        wd = torch.from_numpy(w).cuda()
        torch.cuda.synchronize()
        s.set_state_real_device(0, wd.data_ptr())
        got = s.get_state()
    assert rel_l2(got, oracle.r2c(w)) < 1e-14


def _closure_net(n, mode, zero=False):
    cfg = tg.fno_default_config(h=n, w=n, c=8, mx=8, my=16, layers=2, p=16, max_batch=1, seed=3)
    cfg.mode = mode
    net = tg.FNO(cfg)
    p = net.get_params()
    net.set_params(np.zeros_like(p) if zero else 0.5 * p)
    return net


def test_zero_network_closure_equals_plain():
    n = 64
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as a, \
            tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as b, \
            _closure_net(n, tg.FNO_BF16, zero=True) as net:
        a.init_random(6.0, 0.5, 81)
        b.init_random(6.0, 0.5, 81)
        with tg.Closure(b, net, 1.0, 1.0) as c:
            c.step(5)  # one eager step, then graph replays
            b.synchronize()
        a.step(5)
        a.synchronize()
        assert np.array_equal(a.get_state(), b.get_state())


def _forcing_ref(w, n, params, s, in_scale, out_scale):
    """-div(out_scale * FNO(in_scale * omega)), 2/3-truncated, in the state's normalisation."""
    omega = _real(w, n)
    x = torch.tensor((in_scale * omega).astype(np.float32).astype(np.float64))[None, :, :, None]
    y = fo.forward(torch.tensor(params, dtype=torch.float64), x, s)[0].numpy()
    flux = out_scale * y
    fx, fy = np.fft.rfft2(flux[..., 0]), np.fft.rfft2(flux[..., 1])
    ky = np.fft.fftfreq(n, 1.0 / n)[:, None]
    ky[n // 2] = -n // 2
    kx = np.arange(n // 2 + 1)[None, :]
    keep = np.sqrt(kx * kx + ky * ky) < n / 3.0
    return np.where(keep, -1j * (kx * fx + ky * fy), 0.0)


def test_closure_steps_match_oracle(oracle):
    n, nu, dt, in_s, out_s = 64, 1e-3, 1e-3, 0.3, 300.0
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=nu, dt=dt) as sol, _closure_net(n, tg.FNO_FP32) as net:
        sol.init_random(6.0, 0.5, 82)
        w = sol.get_state()
        params = net.get_params()
        s = fo.FnoShape.of(net.cfg)
        with tg.Closure(sol, net, in_s, out_s) as c:
            got = []
            for _ in range(3):  # eager step, then two graph replays
                c.step(1)
                sol.synchronize()
                got.append(sol.get_state())
    for k in range(3):
        F = _forcing_ref(w, n, params, s, in_s, out_s)
        rhs = lambda v: oracle.derive2csh(v, nu) + F  # noqa: E731
        k1 = rhs(w)
        k2 = rhs(w + dt / 2 * k1)
        k3 = rhs(w + dt / 2 * k2)
        k4 = rhs(w + dt * k3)
        w1 = w + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        assert rel_l2(got[k] - w, w1 - w) < 1e-5, k
        assert np.linalg.norm(F) > 0.02 * np.linalg.norm(k1)  # the closure term is not negligible
        w = got[k]


def test_features_match_numpy():
    n = 64
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as s:
        s.init_random(6.0, 0.5, 83)
        w = s.get_state()
        out = torch.empty((n, n, 6), dtype=torch.float32, device="cuda")
        sc = np.array([1.0, 0.5, 0.25, 2.0, 3.0, 4.0])
        torch.cuda.synchronize()
        s.features(0, 6, out.data_ptr(), sc)
        got = out.cpu().numpy()
    ky = np.fft.fftfreq(n, 1.0 / n)[:, None]
    kx = np.arange(n // 2 + 1)[None, :]
    k2 = (kx * kx + ky * ky).astype(float)
    inv = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    psi = w * inv
    nyq = np.zeros(w.shape, bool)
    nyq[n // 2, :] = True
    nyq[:, n // 2] = True
    specs = [w, 1j * kx * w, 1j * ky * w, -kx * ky * psi, -ky * ky * psi, kx * kx * psi]
    specs = [specs[0]] + [np.where(nyq, 0.0, sp) for sp in specs[1:]]  # odd derivatives: no Nyquist
    for c, sp in enumerate(specs):
        ref = sc[c] * _real(sp, n)
        assert rel_l2(got[..., c], ref) < 1e-6, c


def _d4(a, g):
    """Symmetry g (bit 0 x-flip, bit 1 y-flip, bit 2 transpose) of a real vorticity
    field on a (y, x) grid: w' = -w at the reflected point for each reflection."""
    if g & 1:
        a = -a[:, ::-1]
    if g & 2:
        a = -a[::-1, :]
    if g & 4:
        a = -a.T
    return np.ascontiguousarray(a)


def test_augment_equals_filtered_transformed_field():
    """Symmetry g of (features, flux) of a filtered field equals the features
    and flux of the filtered transformed fine field."""
    n, f = 64, 4
    nc = n // f
    with tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as fine, \
            tg.Solver2D(nc, scheme=tg.SCHEME_RK4, nu=1e-3, dt=1e-3) as coarse:
        fine.init_random(5.0, 0.5, 84)
        wf = _real(fine.get_state(), n)
        X = torch.empty((8, nc, nc, 6), dtype=torch.float32, device="cuda")
        T = torch.empty((8, nc, nc, 2), dtype=torch.float32, device="cuda")
        wb = torch.empty((nc, nc), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        for g in range(8):
            src = torch.from_numpy(_d4(wf, g)).cuda()
            torch.cuda.synchronize()
            fine.set_state_real_device(0, src.data_ptr())
            fine.filter(0, f, 0, T[g].data_ptr(), wb.data_ptr())
            coarse.set_state_real_device(0, wb.data_ptr())
            coarse.features(0, 6, X[g].data_ptr())
        Xa = torch.empty((8, nc, nc, 6), dtype=torch.float32, device="cuda")
        Ta = torch.empty((8, nc, nc, 2), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        tg.closure_augment(X[0:1].data_ptr(), T[0:1].data_ptr(), 1, nc, 6, Xa.data_ptr(), Ta.data_ptr())
        for g in range(8):
            assert rel_l2(Xa[g].cpu().numpy(), X[g].cpu().numpy()) < 1e-5, g
            assert rel_l2(Ta[g].cpu().numpy(), T[g].cpu().numpy()) < 1e-5, g


def test_trained_closure_gains_over_no_closure():
    """What the trained network gains over the coarse run without it, on a
    small setup (256^2 -> 64^2, nu 1e-4, 0.5 eddy times): a-priori it predicts
    the subgrid flux of held-out runs (r2 > 0.3 against the zero flux of the
    method without a closure), and a-posteriori its coarse runs from held-out
    seeds have a lower time-averaged spectrum error against the filtered fine
    run than the coarse runs without it, without falling back."""
    from tara_gb300 import closure as cl

    s = cl.ClosureSetup(n_fine=256, factor=4, nu=1e-4, pairs=256, train_runs=2, val_runs=1, epochs=4,
                        eval_runs=2, samples=5, eddy_times=0.5, calibrate=False)
    out = cl.run_all(s, log=lambda m: None)
    assert out["train"]["val"]["r2"] > 0.3
    ev = out["eval"]
    assert ev["fallback"] is None
    assert ev["err_avg_closure"] < 0.95 * ev["err_avg_plain"], (ev["err_avg_closure"], ev["err_avg_plain"])
    assert out["throughput"]["closure_speedup"] > 1.0
