"""Learned subgrid closure on libtara: training data from the plain fine-grid
solver, FNO training with the library's own kernels, and the coarse-grid runs
measured against the box-filtered fine-grid run.

Everything numeric runs in libtara's CUDA kernels (tara2d_*, tara_fno_*,
tara_closure_*); torch only holds device buffers.  The workflow:

* ``generate_pairs``: decaying-turbulence runs of the plain FP64 solver on the
  fine grid; every few steps each run is box-filtered (block means) onto the
  coarse grid, giving the filtered vorticity (network input) and the exact
  subgrid vorticity flux bar(u w) - bar(u) bar(w) (2-channel target).
* ``train``: Adam on shuffled mini-batches through ``tara_fno_train_step``.
* ``evaluate``: from a held-out seed, the fine-grid plain run (the arbiter of the spectrum error) and
  coarse runs with and without the closure; relative L2 errors of the shell
  energy spectra (shells 1..kmax) against the filtered fine run, averaged over
  the samples of the whole interval, and the simulated time per wall-second of
  each solver on the same GPU.  A closure run whose energy grows (decaying
  turbulence cannot gain energy) or turns non-finite is replaced by the plain
  fine-grid run, which is the fallback.
"""
from __future__ import annotations

import math
import time
from dataclasses import asdict, dataclass, field

import numpy as np

from . import (FNO, PREC_FP32, PREC_FP64, SCHEME_RK4, Closure, FnoConfig, Solver2D, TaraError,
               closure_augment, fno_default_config)


@dataclass
class ClosureSetup:
    n_fine: int = 1024
    factor: int = 8            # coarse grid n_fine / factor
    nu: float = 5e-5
    k0: float = 8.0
    energy: float = 0.5
    dt_fine: float = 5e-4
    coarse_dt_ratio: int = 8   # coarse dt = ratio * fine dt (equal CFL number at factor 8)
    eddy_times: float = 5.0
    train_runs: int = 8
    pairs: int = 2000          # training pairs (train_runs runs, evenly spaced snapshots)
    val_runs: int = 1          # held-out runs for the a-priori validation loss
    seed0: int = 5000
    eval_seed: int = 9000
    batch: int = 32
    lr: float = 1e-3
    epochs: int = 20
    coarse_precision: int = PREC_FP32
    kmax: int | None = None    # spectrum shells 1..kmax (default: the coarse 2/3 cutoff)
    samples: int = 40          # spectrum samples over the evaluation interval
    eval_runs: int = 32        # held-out evaluation runs (seeds eval_seed..)
    cal_runs: int = 16         # validation runs of the a-posteriori calibration (seeds seed0 + 200..)
    features: int = 6          # input channels: w, dw/dx, dw/dy, du/dx, du/dy, dv/dx (first n)
    augment: bool = True       # train on the 8 grid symmetries of every pair
    calibrate: bool = True     # pick the flux amplitude on validation seeds (a-posteriori)
    alphas: tuple = (3.0, 4.0, 5.0, 6.0, 7.0)
    # extra coarse-grid viscosities calibrated jointly with alpha: a constant
    # eddy viscosity beside the learned flux drains what the flux injects at the
    # large scales (0 = the learned flux alone)
    eddy_nus: tuple = (0.0, 5e-5, 1e-4, 2e-4)
    fno: dict = field(default_factory=dict)  # overrides of the FNO config

    @property
    def n_coarse(self) -> int:
        return self.n_fine // self.factor

    @property
    def dt_coarse(self) -> float:
        return self.dt_fine * self.coarse_dt_ratio

    @property
    def tau(self) -> float:
        """Eddy-turnover time (2 pi / k0) / u_rms(0), u_rms = sqrt(<|u|^2>) = sqrt(2 E)."""
        return (2.0 * math.pi / self.k0) / math.sqrt(2.0 * self.energy)

    @property
    def fine_steps(self) -> int:
        """Fine steps over the interval, a multiple of the coarse/fine dt ratio."""
        r = self.coarse_dt_ratio
        return int(round(self.eddy_times * self.tau / self.dt_fine / r)) * r

    @property
    def shells(self) -> int:
        return self.kmax if self.kmax is not None else int(math.ceil(self.n_coarse / 3.0)) - 1


def _torch():
    import torch

    return torch


def _solver(n, s: ClosureSetup, dt, precision=PREC_FP64, batch=1, nu_extra: float = 0.0) -> Solver2D:
    # true pi and a 2 pi box: integer wavenumbers
    return Solver2D(n, scheme=SCHEME_RK4, precision=precision, nu=s.nu + nu_extra, dt=dt, batch=batch,
                    kpi=math.pi, lx=2 * math.pi, ly=2 * math.pi)


def fno_config(s: ClosureSetup, max_batch: int) -> FnoConfig:
    nc = s.n_coarse
    kw = dict(h=nc, w=nc, ci=s.features, co=2, max_batch=max_batch)
    kw.update(s.fno)
    return fno_default_config(**kw)


# ---------------------------------------------------------------------------
# training data
# ---------------------------------------------------------------------------
def generate_pairs(s: ClosureSetup, runs: int, seed0: int, pairs_per_run: int, autotune: bool = True):
    """Network inputs (N, nc, nc, features) and subgrid flux targets (N, nc, nc, 2)
    on the device (FP32), from `runs` fine runs with seeds seed0.. sampled evenly
    over the evaluation interval (snapshot at the end of each stride).  The
    inputs are the closure features of the box-filtered vorticity computed on
    the coarse grid, exactly as the closure computes them at run time."""
    torch = _torch()
    nc, nf = s.n_coarse, s.features
    N = runs * pairs_per_run
    X = torch.empty((N, nc, nc, nf), dtype=torch.float32, device="cuda")
    T = torch.empty((N, nc, nc, 2), dtype=torch.float32, device="cuda")
    wbar = torch.empty((nc, nc), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    stride = max(1, s.fine_steps // pairs_per_run)
    with _solver(s.n_fine, s, s.dt_fine, batch=runs) as fine, _solver(nc, s, s.dt_coarse) as coarse:
        for r in range(runs):
            fine.init_random(s.k0, s.energy, seed0 + r, run=r)
        if autotune:
            fine.autotune(2)
        t0 = time.perf_counter()
        for j in range(pairs_per_run):
            fine.step(stride)
            for r in range(runs):
                i = r * pairs_per_run + j
                fine.filter(r, s.factor, 0, T[i].data_ptr(), wbar.data_ptr())
                coarse.set_state_real_device(0, wbar.data_ptr())
                coarse.features(0, nf, X[i].data_ptr())
        fine.synchronize()
        wall = time.perf_counter() - t0
    return X, T, {"runs": runs, "pairs": N, "stride_steps": stride, "wall_s": wall}


def augment(X, T, nf: int):
    """The eight symmetry images of every pair (tara_closure_augment)."""
    torch = _torch()
    N, n = X.shape[0], X.shape[1]
    Xa = torch.empty((8 * N,) + tuple(X.shape[1:]), dtype=torch.float32, device="cuda")
    Ta = torch.empty((8 * N,) + tuple(T.shape[1:]), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    closure_augment(X.data_ptr(), T.data_ptr(), N, n, nf, Xa.data_ptr(), Ta.data_ptr())
    return Xa, Ta


def scales(X, T):
    """Per-channel in_scales = 1/rms(input channel), out_scale = rms(target)."""
    torch = _torch()
    xs = torch.sqrt(torch.mean(X.double() ** 2, dim=(0, 1, 2))).cpu().numpy()
    ts = float(torch.sqrt(torch.mean(T.double() ** 2)))
    return 1.0 / xs, ts


# ---------------------------------------------------------------------------
# training
# ---------------------------------------------------------------------------
def train(net: FNO, X, T, in_scale, out_scale: float, *, epochs: int, batch: int, lr: float,
          seed: int = 0, Xv=None, Tv=None, log=None) -> dict:
    """Adam on shuffled batches of the normalised pairs.  With validation pairs,
    the parameters of the epoch with the lowest validation loss are kept (early
    stopping).  Returns the loss history and the validation loss of the model
    against the zero prediction (the method without a closure)."""
    torch = _torch()
    sc = torch.as_tensor(np.asarray(in_scale, np.float32), device="cuda")
    Xn = (X * sc).contiguous()
    Tn = (T / out_scale).contiguous()
    N = X.shape[0]
    rng = np.random.default_rng(seed)
    hist, vhist = [], []
    best = (float("inf"), None, -1)
    t0 = time.perf_counter()
    steps = 0
    for ep in range(epochs):
        perm = torch.from_numpy(rng.permutation(N).astype(np.int32)).cuda()
        torch.cuda.synchronize()
        tot, cnt = 0.0, 0
        for b0 in range(0, N - batch + 1, batch):
            idx = perm[b0:b0 + batch]
            loss = net.train_step(Xn.data_ptr(), Tn.data_ptr(), batch, lr=lr, idx_ptr=idx.data_ptr(),
                                  n_samples=N)
            tot += loss
            cnt += 1
            steps += 1
        hist.append(tot / max(cnt, 1))
        msg = f"epoch {ep + 1}/{epochs} loss {hist[-1]:.4e}"
        if Xv is not None:
            v = validate(net, Xv, Tv, in_scale, out_scale)
            vhist.append(v["mse"])
            msg += f" val {v['mse']:.4e} (zero {v['mse_zero']:.4e})"
            if v["mse"] < best[0]:
                best = (v["mse"], net.get_params(), ep)
        if log:
            log(msg)
    wall = time.perf_counter() - t0
    out = {"loss": hist, "val_loss": vhist, "train_steps": steps, "wall_s": wall}
    if best[1] is not None:
        net.set_params(best[1])
        out["best_epoch"] = best[2] + 1
    if Xv is not None:
        out["val"] = validate(net, Xv, Tv, in_scale, out_scale)
    return out


def validate(net: FNO, Xv, Tv, in_scale: float, out_scale: float) -> dict:
    """Mean squared error of the normalised flux prediction on held-out pairs,
    against the zero prediction (no closure): r2 = 1 - mse / mse_zero."""
    torch = _torch()
    sc = torch.as_tensor(np.asarray(in_scale, np.float32), device="cuda")
    Xn = (Xv * sc).contiguous()
    Tn = (Tv / out_scale).contiguous()
    B = int(net.cfg.max_batch)
    Y = torch.empty_like(Tn)
    torch.cuda.synchronize()
    for b0 in range(0, Xn.shape[0], B):
        nb = min(B, Xn.shape[0] - b0)
        net.forward(Xn[b0:b0 + nb].data_ptr(), Y[b0:b0 + nb].data_ptr(), nb)
    torch.cuda.synchronize()
    mse = float(torch.mean((Y.double() - Tn.double()) ** 2))
    mse0 = float(torch.mean(Tn.double() ** 2))
    return {"mse": mse, "mse_zero": mse0, "r2": 1.0 - mse / mse0}


# ---------------------------------------------------------------------------
# evaluation
# ---------------------------------------------------------------------------
def _events_ms(stream_ptr: int, fn, n: int) -> float:
    torch = _torch()
    st = torch.cuda.ExternalStream(stream_ptr)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(st)
    fn(n)
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / n


def spectrum_error(E, Eref, kmax: int) -> float:
    a, b = np.asarray(E[1:kmax + 1]), np.asarray(Eref[1:kmax + 1])
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def evaluate(s: ClosureSetup, net: FNO | None = None, in_scale=1.0, out_scale: float = 1.0,
             nu_extra: float = 0.0, *, closures: dict | None = None, seed: int | None = None,
             runs: int | None = None) -> dict:
    """Held-out runs (seeds seed..seed+eval_runs, default eval_seed) of the fine
    plain solver (the arbiter) and of the coarse solver without a closure and with
    each closure, from the box-filtered fine initial state.  `closures` maps a
    name to (net, in_scale, out_scale[, nu_extra]), each net a separate handle
    whose batch holds eval_runs, nu_extra an eddy viscosity added to the coarse
    solver of that closure; `net` alone stands for {"closure": (net, in_scale,
    out_scale, nu_extra)}.
    `runs` overrides eval_runs.  Spectra (shells 1..kmax) are sampled `samples`
    times over the interval.
    Reported errors, each a relative L2 over the shells against the filtered
    fine run:
      * err_avg_*: of the spectra averaged over the samples and runs (the
        statistical comparison), and
      * mean_err_*: the mean over samples and runs of the per-sample errors
        (which saturates at the run-to-run spread once the coarse and fine
        trajectories have decorrelated).
    A closure run whose energy exceeds 1.05 x its initial energy or turns
    non-finite falls back to the plain fine-grid run from then on (recorded)."""
    torch = _torch()
    if closures is None:
        closures = {"closure": (net, in_scale, out_scale, nu_extra)} if net is not None else {}
    seed = s.eval_seed if seed is None else seed
    nc, kmax, R = s.n_coarse, s.shells, (s.eval_runs if runs is None else runs)
    ratio = s.coarse_dt_ratio
    steps_f = s.fine_steps
    ns = max(1, min(s.samples, steps_f // ratio))
    stride_c = (steps_f // ratio) // ns          # coarse steps between samples
    stride_f = stride_c * ratio
    wbar = torch.empty((nc, nc), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    res = {"setup": {k: v for k, v in asdict(s).items()}, "tau": s.tau, "fine_steps": steps_f,
           "samples": ns, "kmax": kmax, "eval_runs": R, "seed": seed}
    names = list(closures)
    kinds = ["fine", "plain"] + names
    spec_sum = {k: np.zeros(kmax + 1) for k in kinds}
    inst = {k: [] for k in kinds if k != "fine"}
    energy = {k: np.zeros(ns) for k in kinds}
    fallback = {k: None for k in names}
    handles = {}
    objs = {}
    try:
        fine = handles["fine"] = _solver(s.n_fine, s, s.dt_fine, batch=R)
        # coarse-grid handle that holds the filtered fine state to measure its spectrum
        meter = handles["meter"] = _solver(nc, s, s.dt_coarse, precision=s.coarse_precision, batch=R)
        coarse = {"plain": _solver(nc, s, s.dt_coarse, precision=s.coarse_precision, batch=R)}
        for k in names:
            nu_e = closures[k][3] if len(closures[k]) > 3 else 0.0
            coarse[k] = _solver(nc, s, s.dt_coarse, precision=s.coarse_precision, batch=R, nu_extra=nu_e)
        handles.update({"c_" + k: v for k, v in coarse.items()})
        for r in range(R):
            fine.init_random(s.k0, s.energy, seed + r, run=r)
        fine.autotune(2)
        for c in coarse.values():
            c.autotune(2)
        for r in range(R):
            fine.filter(r, s.factor, 0, 0, wbar.data_ptr())
            for c in [meter] + list(coarse.values()):
                c.set_state_real_device(r, wbar.data_ptr())
        e_init = [meter.diag_run(r)[0] for r in range(R)]
        for k in names:
            nk, ik, ok = closures[k][:3]
            objs[k] = Closure(coarse[k], nk, ik, ok)
        for j in range(ns):
            fine.step(stride_f)
            coarse["plain"].step(stride_c)
            for k in names:
                if fallback[k] is None:
                    objs[k].step(stride_c)
            for r in range(R):
                fine.filter(r, s.factor, 0, 0, wbar.data_ptr())
                meter.set_state_real_device(r, wbar.data_ptr())
                Ef = meter.spectrum(r, kmax)
                ef = meter.diag_run(r)[0]
                spec_sum["fine"] += Ef
                energy["fine"][j] += ef / R
                for k in ["plain"] + names:
                    if k != "plain" and fallback[k] is None:
                        try:
                            ec = coarse[k].diag_run(r)[0]
                        except TaraError as ex:
                            ec = float("nan")
                            fallback[k] = f"run {r}: non-finite closure state at sample {j}: {ex}"
                        if fallback[k] is None and not ec <= 1.05 * e_init[r]:
                            fallback[k] = (f"run {r}: closure energy {ec:.4g} above 1.05 x the initial "
                                           f"{e_init[r]:.4g} at sample {j}")
                    if k != "plain" and fallback[k] is not None:
                        Ec, ec = Ef, ef  # the plain fine-grid solver stands in from here on
                    else:
                        Ec, ec = coarse[k].spectrum(r, kmax), coarse[k].diag_run(r)[0]
                    spec_sum[k] += Ec
                    inst[k].append(spectrum_error(Ec, Ef, kmax))
                    energy[k][j] += ec / R
    finally:
        for o in objs.values():
            o.close()
        for h in handles.values():
            h.close()
    avg = {k: v / (ns * R) for k, v in spec_sum.items()}
    res["times"] = [(j + 1) * stride_f * s.dt_fine for j in range(ns)]
    res["fallback"] = fallback.get("closure") if list(fallback) == ["closure"] else fallback
    for k in inst:
        res[f"err_avg_{k}"] = spectrum_error(avg[k], avg["fine"], kmax)
        res[f"mean_err_{k}"] = float(np.mean(inst[k]))
        res[f"err_{k}"] = inst[k]
    res["spectrum_avg"] = {k: list(v) for k, v in avg.items()}
    res["energy"] = {k: list(v) for k, v in energy.items()}
    return res


def calibrate(s: ClosureSetup, params, in_scale, out_scale: float, alphas=(1.0, 1.5, 2.0, 3.0),
              seed: int | None = None, eddy_nus=(0.0,)) -> dict:
    """A-posteriori calibration of the flux amplitude alpha and the extra
    coarse viscosity nu_e on held-out validation seeds (never the evaluation
    seeds): the closure with out_scale * alpha on a coarse solver of viscosity
    nu + nu_e, for every pair, runs beside one fine run; returns the errors and,
    among the pairs whose runs needed no fallback, the one whose time-averaged
    spectrum error is lowest ("best": alpha, "best_nu": nu_e)."""
    seed = s.seed0 + 200 if seed is None else seed
    R = max(1, s.cal_runs)
    grid = [(a, v) for v in eddy_nus for a in alphas]
    name = {(a, v): f"a{a:g}" if v == 0.0 else f"a{a:g}_nu{v:g}" for a, v in grid}
    nets = {}
    try:
        for a, v in grid:
            n = FNO(fno_config(s, R))
            n.set_params(params)
            nets[name[a, v]] = (n, in_scale, out_scale * a, v)
        ev = evaluate(s, closures=nets, seed=seed, runs=R)
    finally:
        for n in nets.values():
            n[0].close()
    errs = {name[g]: ev[f"err_avg_{name[g]}"] for g in grid}
    fell = {name[g]: ev["fallback"][name[g]] for g in grid}
    ok = [g for g in grid if fell[name[g]] is None] or [min(grid)]
    best = min(ok, key=lambda g: errs[name[g]])
    return {"alphas": list(alphas), "eddy_nus": list(eddy_nus), "err_avg": errs, "fallback": fell,
            "err_avg_plain": ev["err_avg_plain"], "best": best[0], "best_nu": best[1],
            "energy": ev["energy"], "seed": seed, "runs": R}


def throughput(s: ClosureSetup, net: FNO | None, in_scale=1.0, out_scale: float = 1.0,
               steps: int = 200, nu_extra: float = 0.0) -> dict:
    """Simulated time per wall-second of one fine plain run and of one coarse run
    with the closure (and without), on the same GPU: CUDA events around `steps`
    steps on each solver's stream, after autotuning and warm-up."""
    torch = _torch()
    nc = s.n_coarse
    out = {}
    with _solver(s.n_fine, s, s.dt_fine) as fine, \
            _solver(nc, s, s.dt_coarse, precision=s.coarse_precision) as plain_c, \
            _solver(nc, s, s.dt_coarse, precision=s.coarse_precision, nu_extra=nu_extra) as clos_c:
        fine.init_random(s.k0, s.energy, s.eval_seed)
        wbar = torch.empty((nc, nc), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        fine.filter(0, s.factor, 0, 0, wbar.data_ptr())
        for c in (plain_c, clos_c):
            c.set_state_real_device(0, wbar.data_ptr())
        for h in (fine, plain_c, clos_c):
            h.autotune(2)
            h.step(3)
        ms_f = _events_ms(fine.stream, fine.step, steps)
        ms_p = _events_ms(plain_c.stream, plain_c.step, steps)
        out["fine_ms_per_step"] = ms_f
        out["plain_coarse_ms_per_step"] = ms_p
        out["fine_simtime_per_s"] = s.dt_fine / (ms_f * 1e-3)
        out["plain_coarse_simtime_per_s"] = s.dt_coarse / (ms_p * 1e-3)
        out["plain_coarse_speedup"] = out["plain_coarse_simtime_per_s"] / out["fine_simtime_per_s"]
        if net is not None:
            with Closure(clos_c, net, in_scale, out_scale) as closure:
                closure.step(3)
                ms_c = _events_ms(clos_c.stream, closure.step, steps)
            out["closure_ms_per_step"] = ms_c
            out["closure_simtime_per_s"] = s.dt_coarse / (ms_c * 1e-3)
            out["closure_speedup"] = out["closure_simtime_per_s"] / out["fine_simtime_per_s"]
    return out


def run_all(s: ClosureSetup, log=print) -> dict:
    """Data generation, training and evaluation; returns every figure."""
    out = {}
    X, T, gi = generate_pairs(s, s.train_runs, s.seed0, s.pairs // s.train_runs)
    log(f"train pairs {gi}")
    Xv, Tv, vi = generate_pairs(s, s.val_runs, s.seed0 + 100, max(1, s.pairs // (4 * s.train_runs)))
    log(f"validation pairs {vi}")
    if s.augment:
        X, T = augment(X, T, s.features)
    ins, outs = scales(X, T)
    out["data"] = {"train": gi, "val": vi, "in_scale": list(map(float, ins)), "out_scale": outs}
    with FNO(fno_config(s, s.batch)) as net:
        out["train"] = train(net, X, T, ins, outs, epochs=s.epochs, batch=s.batch, lr=s.lr, Xv=Xv, Tv=Tv,
                             log=log)
        log(f"validation {out['train']['val']}")
        params = net.get_params()
    alpha, nu_e = 1.0, 0.0
    if s.calibrate:
        out["calibration"] = calibrate(s, params, ins, outs, s.alphas, eddy_nus=s.eddy_nus)
        alpha, nu_e = out["calibration"]["best"], out["calibration"]["best_nu"]
        log(f"calibration {out['calibration']['err_avg']} -> alpha {alpha}, nu_e {nu_e}")
    out["alpha"] = alpha
    out["nu_e"] = nu_e
    with FNO(fno_config(s, max(1, s.eval_runs))) as neval:
        neval.set_params(params)
        out["eval"] = evaluate(s, neval, ins, outs * alpha, nu_e)
    with FNO(fno_config(s, 1)) as net1:
        net1.set_params(params)
        out["throughput"] = throughput(s, net1, ins, outs * alpha, nu_extra=nu_e)
    out["params"] = params
    return out
