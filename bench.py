"""Benchmark: grid-pt*steps/s of TARA's plain 2D vorticity solver, FP64, RK4.

Workload (one "step" = one classic RK4 step = 4 RHS evaluations): Nx = Ny = 2048,
2*pi box, nu = 1e-4, dt = 5e-5, seeded random-phase initial vorticity with
E(k) ~ k^4 exp(-(k/6)^2) normalised to energy 0.5 (seed 20242048).  The working
set (about 340 MB) is larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 2048]

Our arm prints one JSON line with value (device-resident state, CUDA events on
the solver stream), e2e (host buffers through tara2d_set_state / step /
get_state, copies inside the timed region), the roofline of the dominant kernel,
clocks sampled during the timed region and a CPU baseline (the oracle's C
restatement on the host cores, a bounded sample).  ``--impl reference`` times
the CPU restatement alone (the reference Fortran cannot be built on either
machine: no Fortran compiler) with all host threads.

Multi-GPU: the path does not shard (one grid is one FFT problem); N ranks run N
independent replicas, value = all ranks' grid-pt*steps / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "grid-pt*steps/s at 2048^2 FP64 (plain 2D vorticity RHS + RK4)"
UNIT = "grid-pt*steps/s"
SEED = {512: 20240512, 2048: 20242048}
NU, DT, K0, ENERGY = 1e-4, 5e-5, 6.0, 0.5


def workload(n: int) -> str:
    """The workload string both arms print in config.workload."""
    return (f"2D vorticity plain RHS (derive2csh), classic RK4, {n}x{n}, "
            f"2pi box, nu={NU}, dt={DT}, k0={K0}, E=0.5, seed {SEED.get(n, 1)}")


def peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def from_profiles(key: str, kernel: str, n: int) -> float | None:
    """A per-kernel figure recorded from an ncu capture: a profiles/*.txt line
    '<key> <kernel> <n> <value>' (e.g. traffic_bytes_per_launch), or None."""
    for f in sorted((ROOT / "profiles").glob("*.txt")):
        for line in f.read_text().splitlines():
            parts = line.split()
            if len(parts) == 4 and parts[0] == key and parts[1] == kernel and parts[2] == str(n):
                return float(parts[3])
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return self

        def rd():
            for line in self.proc.stdout:
                self.rows.append((time.time(), [c.strip() for c in line.split(",")]))

        self.thread = threading.Thread(target=rd, daemon=True)
        self.thread.start()
        return self

    def mark(self, which: str) -> None:
        setattr(self, "t_" + which, time.time())

    def stop(self) -> dict:
        time.sleep(0.1)
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        t0, t1 = getattr(self, "t_start", 0.0), getattr(self, "t_end", float("inf"))
        window = [r for t, r in self.rows if t0 <= t <= t1 + 0.05]
        if not window:  # a timed region shorter than the sampling period: nearest samples
            window = [r for t, r in self.rows if t >= t0][:2]
        for r in window:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(n: int, budget_s: float = 15.0, threads: int | None = None) -> dict:
    """The oracle's C restatement (own FFT, OpenMP over rows/columns) on the
    host cores: RK4 steps at n^2 until about budget_s of work."""
    from oracle import oracle as orc

    O = orc.load()
    O.set_threads(threads or os.cpu_count() or 1)
    w0 = O.ic_random(n, n, K0, ENERGY, SEED.get(n, 1))
    steps, elapsed, w = 0, 0.0, w0
    while elapsed < budget_s and steps < 1000:
        t0 = time.perf_counter()
        w, _ = O.run(w, rhs=0, scheme=1, nu=NU, dt=DT, steps=1)
        elapsed += time.perf_counter() - t0
        steps += 1
    return {"value": n * n * steps / elapsed, "unit": UNIT, "cores": O.threads(), "kind": "port",
            "sample": f"{steps} RK4 step(s) at {n}^2 in {elapsed:.2f} s (oracle C restatement, "
                      f"own radix-2 FFT, {O.threads()} OpenMP thread{'s' if O.threads() != 1 else ''})"}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        # NCCL on the GPUs; gloo only where no GPU is visible (the CPU tests of the
        # multi-rank host logic)
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
        return rank, ws, dist
    return 0, 1, None


def run_reference(args) -> None:
    rank, ws, dist = 0, int(os.environ.get("WORLD_SIZE", "1")), None
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle as orc

    O = orc.load()
    O.set_threads(os.cpu_count() or 1)
    n = args.n
    w = O.ic_random(n, n, K0, ENERGY, SEED.get(n, 1))
    for _ in range(args.warmup):
        w, _ = O.run(w, rhs=0, scheme=1, nu=NU, dt=DT, steps=1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w, _ = O.run(w, rhs=0, scheme=1, nu=NU, dt=DT, steps=1)
    el = time.perf_counter() - t0
    value = n * n * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded random-phase spectrum)",
        "config": {"workload": workload(n), "l2": "working set > L2 (no flush)",
                   "parallelism": "host CPU cores, rank 0 only"},
        "note": "reference Fortran not buildable (no Fortran compiler); CPU restatement",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": O.threads(), "kind": "port",
                         "sample": f"{args.steps} timed RK4 steps at {n}^2 after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def fft_fp64_inst(n: int, radix8: bool = False) -> int:
    """FP64 instructions of one length-n transform of fft.cuh, counted from its
    butterflies.  Radix-4 path: an untwiddled radix-4 first stage (16 adds per
    butterfly) or, for odd log2 n, an untwiddled radix-8 first stage (52 per
    butterfly), then twiddled radix-4 stages on ratio-form twiddles (22 FMAs per
    butterfly).  Radix-8 path: an untwiddled radix-8 first stage (52 per butterfly), twiddled
    radix-8 stages (72), then zero to two twiddled radix-4 stages on plain
    complex twiddles (24; untwiddled, 16, when they come first)."""
    lg = n.bit_length() - 1
    q = n // 4
    if not radix8:
        if lg % 2:
            return (n // 8) * 52 + q * 22 * ((lg - 3) // 2)
        return q * 16 + q * 22 * (lg // 2 - 1)
    s8 = lg // 3 - 1 if (lg % 3 == 1 and lg >= 4) else lg // 3
    s4 = 2 if lg % 3 == 1 else 1 if lg % 3 == 2 else 0
    b8 = n // 8
    inst = (b8 * 52 + b8 * 72 * (s8 - 1)) if s8 else 0
    return inst + sum(q * (16 if (s8 == 0 and i == 0) else 24) for i in range(s4))


def fp64_pipe(n: int, per_kernel_ms: dict, sm_mhz, probe_tinst, variants=(0, 0, 0)) -> dict:
    """FP64-pipe roofline of the three kernels at n x n: the transforms' FP64
    instructions per launch (element work excluded, so the fractions are lower
    bounds) over the measured launch time, against the nominal rate (2 FP64
    thread-instructions per SM per cycle at the sampled SM clock) and the DFMA
    rate measured by tara_measure_dfma_rate."""
    import math

    import torch
    nh = n // 2 + 1
    live = math.ceil((n + n) / 2.0 / 3.0)  # columns below the 2/3 cut (integer wavenumbers)
    f = [fft_fp64_inst(n, bool(v & 4)) for v in variants]  # per kernel: its radix path
    inst = {"k_col_inverse": 4 * nh * f[0], "k_row_nl": (n // 2) * 5 * f[1], "k_col_forward": live * f[2]}
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    nominal = 2.0 * sms * (sm_mhz or 2070.0) * 1e6
    ach = {k: inst[k] / (per_kernel_ms[k] * 1e-3) for k in inst if k in per_kernel_ms}
    return {"inst_per_launch": inst, "achieved_inst_per_s": ach, "nominal_inst_per_s": nominal,
            "measured_dfma_inst_per_s": probe_tinst,
            "frac_of_nominal": {k: v / nominal for k, v in ach.items()},
            "frac_of_measured_dfma": {k: v / probe_tinst for k, v in ach.items()} if probe_tinst else None,
            "count": "transform butterflies only; element work excluded (fractions are lower bounds)"}


def run_ours(args) -> None:
    import numpy as np
    import torch

    import tara_gb300 as tg
    from tara_gb300 import shard

    rank, ws, dist = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    n = args.n
    prec = {"fp32": tg.PREC_FP32, "df64": tg.PREC_DF64}.get(args.precision, tg.PREC_FP64)
    s = tg.Solver2D(n, scheme=tg.SCHEME_RK4, nu=NU, dt=DT, precision=prec)
    s.init_random(K0, ENERGY, SEED.get(n, 1))
    if args.variants:
        tuned = {"variants": [int(v) for v in args.variants.split(",")], "ms": None}
        s.set_variants(tuned["variants"])
    else:
        tuned = s.autotune(2)  # configuration per kernel (the state is restored)
    dfma_rate = tg.measure_dfma_rate(5) if prec == tg.PREC_FP64 and rank == 0 else None
    s.step(args.warmup)
    s.synchronize()

    # ---- device-resident timed region (CUDA events on the solver's stream)
    sampler = ClockSampler(local).start() if rank == 0 else None
    if sampler:
        time.sleep(0.5)  # let nvidia-smi start before the timed region
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.mark("start")
    prof = s.step_timed(args.steps)
    torch.cuda.synchronize()
    if sampler:
        sampler.mark("end")
    if dist:
        dist.barrier()
    clocks = sampler.stop() if sampler else None
    el_ms = shard.max_over_ranks(prof["total_ms"], dist)
    e, z = s.diag()  # also raises on non-finite values

    # ---- end to end through the public API with pinned host buffers
    nh = n // 2 + 1
    host_in = torch.empty((n, nh), dtype=torch.complex128, pin_memory=True).numpy()
    host_out = torch.empty((n, nh), dtype=torch.complex128, pin_memory=True).numpy()
    host_in[:] = s.get_state()
    e2e_steps = max(1, min(args.steps, 10))
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.set_state(host_in)
        s.step(1)
        s.get_state_into(host_out)
        host_in, host_out = host_out, host_in
    torch.cuda.synchronize()
    e2e_el = shard.max_over_ranks(time.perf_counter() - t0, dist)

    if rank != 0:
        s.close()
        return

    # ---- roofline of the dominant kernel (algorithmic bytes / event time)
    F = 16.0 * nh * n  # one FP64 half spectrum
    alg_bytes = {  # per launch: what each kernel must read and write at minimum
        "k_col_inverse": 5 * F,   # read omega_hat, write 4 spectra
        "k_row_nl": 5 * F,        # read 4 spectra, write the products' spectrum
        "k_col_forward": 5 * F,   # RK4 stages average (4F, 6F, 6F, 4F + 1F) ~ 5F
    }
    ks = prof["kernels"]
    dom = max(ks, key=lambda k: ks[k]["ms"])
    avg_ms = ks[dom]["ms"] / max(1, ks[dom]["launches"])
    peak, peak_kind = peaks()
    achieved = alg_bytes[dom] / (avg_ms * 1e-3) / 1e9
    traffic = from_profiles("traffic_bytes_per_launch", dom, n) if prec == tg.PREC_FP64 else None
    value = n * n * args.steps * ws / (el_ms * 1e-3)
    cpu = cpu_baseline(n, budget_s=args.cpu_budget) if not args.no_cpu_baseline else None
    if cpu:
        # the reference's own 2D path runs on one thread (no OpenMP, no FFTW threads)
        one = cpu_baseline(n, budget_s=min(args.cpu_budget, 8.0), threads=1)
        cpu["single_thread"] = {"value": one["value"], "cores": one["cores"], "sample": one["sample"]}
    fp64 = (fp64_pipe(n, {k: v["ms"] / max(1, v["launches"]) for k, v in ks.items()},
                      (clocks or {}).get("sm_mhz"), dfma_rate, tuned["variants"])
            if prec == tg.PREC_FP64 else None)
    roof64 = None
    if fp64:
        # the FP64-pipe roofline beside the HBM one: the transforms' algorithmic
        # FP64 instructions (element work excluded) over the measured DFMA rate,
        # for the dominant kernel and for the whole RK4 step (4 RHS evaluations)
        pk = fp64["measured_dfma_inst_per_s"] or fp64["nominal_inst_per_s"]
        step_inst = 4 * sum(fp64["inst_per_launch"].values())
        step_rate = step_inst / (el_ms / args.steps * 1e-3)
        roof64 = {"bound": "fp64", "kernel": dom, "achieved": fp64["achieved_inst_per_s"][dom], "peak": pk,
                  "peak_kind": "measured DFMA rate" if fp64["measured_dfma_inst_per_s"] else "nominal",
                  "unit": "FP64 inst/s", "frac": fp64["achieved_inst_per_s"][dom] / pk,
                  "count": "transform butterflies only (a lower bound)",
                  "step": {"inst_per_step": step_inst, "achieved": step_rate, "frac": step_rate / pk}}
        # the same with every FP64 instruction the kernels execute, as ncu
        # counted them (sm__inst_executed_pipe_fp64 x 32) in the capture summarised
        # in profiles/rhs2d_fp64_2048_traffic.txt
        cnt = {k: from_profiles("fp64_thread_inst_per_launch", k, n) for k in fp64["inst_per_launch"]}
        if all(cnt.values()):
            per_ms = {k: v["ms"] / max(1, v["launches"]) for k, v in ks.items()}
            step_all = 4 * sum(cnt.values())
            roof64["all_fp64_inst"] = {
                "inst_per_launch": cnt[dom], "achieved": cnt[dom] / (per_ms[dom] * 1e-3),
                "frac": cnt[dom] / (per_ms[dom] * 1e-3) / pk,
                "step": {"inst_per_step": step_all, "achieved": step_all / (el_ms / args.steps * 1e-3),
                         "frac": step_all / (el_ms / args.steps * 1e-3) / pk}}
    line = {
        "metric": {tg.PREC_FP64: METRIC, tg.PREC_FP32: METRIC.replace("FP64", "FP32 form"),
                   tg.PREC_DF64: METRIC.replace("FP64", "double-float form")}[prec],
        "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {tg.PREC_FP64: "f64", tg.PREC_FP32: "f32 transforms / f64 state",
                                                  tg.PREC_DF64: "df64 (f32 pair) transforms / f64 state"}[prec],
        "data": "synthetic (seeded random-phase spectrum, Philox4x32-10)",
        "config": {"workload": workload(n),
                   "l2": "working set > L2 (no flush)", "parallelism": f"replicas x{ws}"},
        "e2e": {"value": n * n * e2e_steps * ws / e2e_el, "unit": UNIT,
                "h2d_bytes_per_step": int(F), "d2h_bytes_per_step": int(F),
                "path": "tara2d_set_state(pinned host) + tara2d_step(1) + tara2d_get_state"},
        "gpu_launches": s.launches_per_step * args.steps,
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "avg_launch_ms": avg_ms,
                     "limiter": ("FP64 pipe (GB300: 2 FP64 thread-instructions per SM per cycle)"
                                 if prec == tg.PREC_FP64 else
                                 "FP32 pipes and global-load latency (double-float: profiles/rhs2d_df64_2048_ncu_full.md)"
                                 if prec == tg.PREC_DF64 else "FP32 pipes and shared-memory bank conflicts"),
                     "fp64_pipe_busy_pct_ncu": (from_profiles("fp64_pipe_busy_pct", dom, n)
                                                if prec == tg.PREC_FP64 else None),
                     "per_kernel_ms": {k: v["ms"] / max(1, v["launches"]) for k, v in ks.items()}},
        "clocks": clocks,
        "fp64_pipe": fp64,
        "roofline_fp64": roof64,
        "tile_variants": tuned["variants"],
        "autotune_ms": tuned["ms"],  # per-launch ms in context: configurations 0-7 (rows) x the three kernels
        "diag": {"energy": e, "enstrophy": z},
        "cpu_baseline": cpu,
    }
    if ws == 1 and not args.no_side:
        line["other_configs"] = side_workloads(args)
    print(json.dumps(line), flush=True)
    s.close()


def side_workloads(args) -> dict:
    """Short measurements of the other benchmark configurations in the same run
    (one GPU): the 384-run ensemble (FP32 form, RK4; autotuned form and tiles),
    the 128^3 3D MHD AB2 step, the closure network's training step and the
    closure step against the 1024^2 step it replaces.  Each reports its own
    metric; a failure is recorded, not raised."""
    import copy

    out = {}
    for name, fn in (("ensemble_384_runs", run_ensemble), ("mhd3d_128", run_mhd3d),
                     ("fno_train_batch32", run_fno_train), ("closure_step_128", run_closure_step)):
        a = copy.copy(args)
        a.steps, a.warmup, a.ens_error_steps, a.ens_form = 10, 3, 0, "auto"
        try:
            ln = fn(a, emit=False)
            out[name] = {k: ln[k] for k in ("metric", "value", "unit", "ms_per_step", "dtype") if k in ln}
            for k in ("form", "persistent", "form_ms_per_step", "radix", "gemm_forms_ms_per_step",
                      "fine_1024_fp64_ms_per_step", "simtime_speedup_vs_fine_1024"):
                if k in ln:
                    out[name][k] = ln[k]
        except Exception as exc:  # reported beside the headline, never hides it
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
    return out


PROFILE_RANGE = False  # --profile-range: the timed regions run inside cudaProfilerStart/Stop


def timed_on_stream(stream_ptr: int, fn):
    """CUDA-event time (ms) of fn() on the library stream stream_ptr (with
    --profile-range, inside a profiler range, so that `ncu --profile-from-start
    off` captures the timed launches only)."""
    import torch

    st = torch.cuda.ExternalStream(stream_ptr)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    if PROFILE_RANGE:
        torch.cuda.profiler.start()
    a.record(st)
    fn()
    b.record(st)
    b.synchronize()
    if PROFILE_RANGE:
        torch.cuda.profiler.stop()
    return a.elapsed_time(b)


def ensemble_runs(per_rank: int, world_size: int = 1) -> list[tuple[int, float, int]]:
    """The global run list (n, k0, seed) of the ensemble workload: per_rank x
    world_size runs at each of 128^2, 256^2 and 512^2 in that order, k0 drawn
    from numpy default_rng(4000) on U[4,10], seed 4000 + r."""
    import numpy as np

    per = per_rank * world_size
    k0 = np.random.default_rng(4000).uniform(4.0, 10.0, 3 * per)
    return [(n, float(k0[r]), 4000 + r) for r, n in enumerate([128] * per + [256] * per + [512] * per)]


def run_ensemble(args, emit: bool = True) -> dict | None:
    """Ensemble of independent 2D runs, RK4, nu = 1e-3, dt = 1e-4, FP32
    transforms and products with FP64 state: per rank 3 x ens_runs_per_size runs
    (default 128 each at 128^2, 256^2, 512^2; 384 in all on one GPU).  The global
    list holds N times as many (same size mix), k0 ~ U[4,10] (numpy
    default_rng(4000)), seed 4000 + r; each rank steps its cost-balanced shard
    (tara_gb300.shard) with no exchange between ranks, so the scaling is weak.
    One CUDA-graph launch per ensemble step on each rank; tile variants picked
    by the autotuner first."""
    import numpy as np
    import torch

    import tara_gb300 as tg
    from tara_gb300 import shard

    rank, ws, dist = dist_init()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    runs = ensemble_runs(args.ens_runs_per_size, ws)
    per = args.ens_runs_per_size * ws
    idx, mine = shard.shard_of(runs, rank, ws)
    e = tg.Ensemble(mine, precision=tg.PREC_FP32, nu=1e-3, dt=1e-4)
    e.autotune(3)  # tiles and radix per kernel and size, then graph vs persistent
    form = getattr(args, "ens_form", "auto")
    if form != "auto":
        e.set_form({"graph": tg.ENS_GRAPH, "persistent4": tg.ENS_PERSISTENT4,
                    "persistent8": tg.ENS_PERSISTENT8}[form])
    e.step(args.warmup)
    e.synchronize()
    if dist:
        dist.barrier()
    ms = shard.max_over_ranks(timed_on_stream(e.stream, lambda: e.step(args.steps)), dist)
    e.synchronize()
    pts = sum(n * n for n, _, _ in runs)
    form = e.form()
    persistent = form["form"] != "graph"
    groups = e.groups()
    line = {"metric": f"ensemble grid-pt*steps/s ({len(runs)} runs: {per} each at 128^2, 256^2, 512^2; RK4)",
            "value": pts * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "dtype": "f32 transforms / f64 state",
            "data": "synthetic (seeded random-phase spectra)",
            "config": {"workload": "ensemble of uneven runs",
                       "launch": ("one cooperative launch for all timed steps" if persistent
                                  else "one cudaGraphLaunch per step"),
                       "l2": "working set > L2 (no flush)",
                       "parallelism": f"runs sharded x{ws} (cost-balanced, no exchange)"},
            # the persistent form is one kernel launch per step() call; the graph
            # replays every pass kernel of every size per step
            "gpu_launches": int(shard.sum_over_ranks(1 if persistent else e.launches_per_step * args.steps,
                                                     dist)),
            "persistent": persistent, "form": form["form"], "form_ms_per_step": form["ms_per_step"],
            "radix": {str(g["n"]): ["radix-8" if v & 4 else "radix-4" for v in g["variants"]]
                      for g in groups},
            "autotune": groups}
    if args.ens_error_steps:
        e64 = tg.Ensemble(mine, precision=tg.PREC_FP64, nu=1e-3, dt=1e-4)
        e.step(args.ens_error_steps - args.steps - args.warmup)
        e64.step(args.ens_error_steps)
        e.synchronize()
        e64.synchronize()
        local = []
        for r in range(len(mine)):
            a, b = e.get_state(r), e64.get_state(r)
            local.append(float(np.linalg.norm(a - b) / np.linalg.norm(b)))
        e64.close()
        errs = shard.gather_by_index(idx, local, len(runs), dist)
        if rank == 0:
            line["error_vs_fp64"] = {"steps": args.ens_error_steps, "max": max(errs),
                                     "median": float(np.median(errs)),
                                     "per_size_max": {str(n): max(x for (m, _, _), x in zip(runs, errs) if m == n)
                                                      for n in (128, 256, 512)}}
    if rank == 0:
        if emit:
            print(json.dumps(line), flush=True)
    e.close()
    return line if rank == 0 else None


def run_coh2d(args) -> None:
    """The 2D compressible solvers, AB2 steps at n^2 from the reference drivers'
    initial states, FP64:
      coh2d  isothermal hydro (derive2coh + ab2coh; src/main2coh.f95: disk + five
             point vortices, n = 1, mux = muy = 2e-4, CS = 3.77, 2 pi box);
             11 inverse and 3 forward real 2D transforms per step
      com2d  MHD (derive2com + ab2com; src/main2com.f95: rho = 1, ux = -sin y,
             uy = sin x, B = (1, 1), CS = 100, mu = 1e-3, eta = 1e-4, forcing
             kf = A = 1); 8 inverse and 11 forward real 2D transforms per step
    CUDA events on the solver's stream; e2e through set_state (pinned host) +
    step(1) + get_state; the FP64-pipe roofline of the whole step from the
    transforms' FP64 instructions."""
    import numpy as np
    import torch

    import tara_gb300 as tg

    torch.cuda.set_device(0)
    n = args.n
    mhd = args.workload == "com2d"
    if mhd:
        dt = 1e-5 * (2048.0 / n)  # sound-speed CFL at CS = 100
        s = tg.Com2D(n, dt=dt)
        s.init_reference(2.0, 2.0, 1.0)
        nfield, ninv, nfwd = 6, 8, 11
    else:
        dt = 2.5e-4 * (1024.0 / n)  # CFL-scaled from the reference's 1e-3 at 64^2-256^2
        s = tg.Coh2D(n, dt=dt)
        s.init_vortices(2.0, 2.0)
        nfield, ninv, nfwd = 3, 11, 3
    s.step(args.warmup)
    s.synchronize()
    st = torch.cuda.ExternalStream(s.stream)
    sampler = ClockSampler(0).start()
    time.sleep(0.5)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    sampler.mark("start")
    a.record(st)
    s.step(args.steps)
    b.record(st)
    torch.cuda.synchronize()
    sampler.mark("end")
    clocks = sampler.stop()
    el_ms = a.elapsed_time(b)
    s.synchronize()  # raises on non-finite values
    nh = n // 2 + 1
    F = 16.0 * nh * n
    host_in = torch.empty((nfield, n, nh), dtype=torch.complex128, pin_memory=True).numpy()
    host_out = torch.empty((nfield, n, nh), dtype=torch.complex128, pin_memory=True).numpy()
    host_in[:] = s.get_state()
    e2e_steps = max(1, min(args.steps, 10))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.set_state(host_in)  # history reset: the e2e loop times the transfer path only
        s.step(1)
        s.get_state_into(host_out)
        host_in, host_out = host_out, host_in
    torch.cuda.synchronize()
    e2e_el = time.perf_counter() - t0
    f = fft_fp64_inst(n)
    inst = (ninv + nfwd) * nh * f + (ninv + nfwd) * (n // 2) * f
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    nominal = 2.0 * sms * ((clocks or {}).get("sm_mhz") or 2070.0) * 1e6
    ms_step = el_ms / args.steps
    peak, peak_kind = peaks()
    # spectra F, real fields F/2: coh 3+11 | 22 | 11+5.5 | 5.5+1.5 | 1.5+3 | 6 | 15 ;
    # com 12 | 16 | 8+4 | 4+2 | 2+4 | 8 | 4 | 2+1 | 4+3.5+1+3.5 | 3.5+7 | 14 | 7+4+6+18+18
    traffic_f = 130 if mhd else 85
    # dominant launch: the 11-field inverse column transform, reads and writes 11 spectra
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import oracle as orc

        O = orc.load()
        O.set_threads(os.cpu_count() or 1)
        m = 512
        st0 = O.ic_com(m, m) if mhd else O.ic_coh(m, m)
        steps_c, t_c = 0, 0.0
        while t_c < args.cpu_budget and steps_c < 200:
            t1 = time.perf_counter()
            if mhd:
                st0, _ = O.run_com(st0, orc.com_params(), 1e-5 * 2048.0 / m, 1)
            else:
                st0, _ = O.run_coh(st0, orc.coh_params(), 2.5e-4 * 1024.0 / m, 1)
            t_c += time.perf_counter() - t1
            steps_c += 1
        name = "derive2com/ab2com" if mhd else "derive2coh/ab2coh"
        cpu = {"value": m * m * steps_c / t_c, "unit": UNIT, "cores": O.threads(), "kind": "port",
               "sample": f"{steps_c} AB2 step(s) at {m}^2 in {t_c:.2f} s (oracle C restatement of "
                         f"{name}, own radix-2 FFT, {O.threads()} OpenMP threads)"}
    what = ("2D compressible MHD (derive2com + ab2com)" if mhd
            else "2D compressible isothermal hydro (derive2coh + ab2coh)")
    workload = (f"derive2com + ab2com, {n}x{n}, 2pi box, mu=1e-3, eta=1e-4, CS=100, kf=A=1, dt={dt:g}" if mhd
                else f"derive2coh + ab2coh, {n}x{n}, 2pi box, mux=muy=2e-4, CS=3.77, dt={dt:g}")
    line = {"metric": f"grid-pt*steps/s at {n}^2, {what}, FP64",
            "value": n * n * args.steps / (el_ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (the reference driver's vortex initial state)",
            "config": {"workload": workload, "l2": "working set > L2 (no flush)"},
            "e2e": {"value": n * n * e2e_steps / e2e_el, "unit": UNIT, "h2d_bytes_per_step": int(nfield * F),
                    "d2h_bytes_per_step": int(nfield * F),
                    "path": ("tara_com2d" if mhd else "tara_coh2d") + "_set_state(pinned host) + _step(1) + _get_state"},
            "gpu_launches": s.launches_per_step * args.steps,
            "roofline": {"bound": "hbm", "kernel": f"whole AB2 step ({s.launches_per_step} launches)",
                         "achieved": traffic_f * F / (ms_step * 1e-3) / 1e9, "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": traffic_f * F / (ms_step * 1e-3) / 1e9 / peak, "traffic": None,
                         "bytes_per_step": f"{traffic_f} F (F = one FP64 half spectrum): the unfused passes' reads "
                                           "and writes of spectra (F each) and real fields (F/2 each)",
                         "limiter": "FP64 pipe"},
            "fp64_pipe": {"inst_per_step": inst, "achieved_inst_per_s": inst / (ms_step * 1e-3),
                          "nominal_inst_per_s": nominal, "frac_of_nominal": inst / (ms_step * 1e-3) / nominal,
                          "count": f"transform butterflies only ({ninv} c2r + {nfwd} r2c); element work excluded"},
            "clocks": clocks, "cpu_baseline": cpu}
    s.close()
    print(json.dumps(line), flush=True)


def run_mhd3d(args, emit: bool = True) -> dict:
    """128^3 compressible MHD, FP64, AB2, nu = eta = 0.01, dt = 1e-3."""
    import torch

    import tara_gb300 as tg

    torch.cuda.set_device(0)
    n = 128
    s = tg.Solver3D(n, defined=1, nu_u=0.01, eta_b=0.01, dt=1e-3)
    s.init_orszag_tang(0.01, 4, 3)  # tara3d_init_orszag_tang: 1 % perturbation at |k| <= 4, seed 3
    s.step(args.warmup)
    s.synchronize()
    ms = timed_on_stream(s.stream, lambda: s.step(args.steps))
    s.synchronize()
    d = s.diag()
    line = {"metric": "grid-pt*steps/s at 128^3 FP64 (3D compressible MHD, AB2)",
            "value": n**3 * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (Orszag-Tang-type profile + 1% solenoidal noise)",
            "config": {"workload": "3D MHD 128^3, nu=eta=0.01, dt=1e-3, AB2, 20 transforms/step"},
            "gpu_launches": None, "diag": {"pressure": d[0], "kinetic": d[1], "total_E": d[2],
                                           "magnetic": d[3]}}
    if emit:
        print(json.dumps(line), flush=True)
    s.close()
    return line


def run_closure(args) -> None:
    """Learned closure: training data from 1024^2 FP64 decaying-turbulence runs
    (nu = 5e-5, k0 = 8), box-filtered (8 x 8 block means) to 128^2 with the exact
    subgrid vorticity flux as target; 4-layer FNO, 32 channels, 16 modes per
    axis, GELU, BF16 tensor-core GEMMs with FP32 accumulation, Adam lr 1e-3,
    batch 32; flux amplitude and an extra coarse eddy viscosity calibrated on 16
    validation seeds; evaluated on 32 held-out seeds over 5 eddy-turnover times
    against the filtered 1024^2 plain run.  The value is the closure's simulated time per wall-second over that of
    the plain 1024^2 FP64 solver on the same GPU (one run each, CUDA events)."""
    import torch

    from tara_gb300 import closure as cl

    torch.cuda.set_device(0)
    s = cl.ClosureSetup(epochs=args.closure_epochs)
    out = cl.run_all(s, log=lambda m: print(m, file=sys.stderr, flush=True))
    ev, tp = out["eval"], out["throughput"]
    line = {"metric": "closure speedup: simulated time per wall-second, 128^2 + FNO closure vs plain 1024^2 FP64",
            "value": tp["closure_speedup"], "unit": "x", "n_gpus": 1, "steps": None, "warmup": None,
            "ms_per_step": tp["closure_ms_per_step"], "higher_is_better": True, "vs_baseline": None,
            "dtype": "bf16 GEMMs / f32 network / f64 state", "data": "synthetic (seeded decaying turbulence)",
            "config": {"workload": "learned closure 1024^2 -> 128^2, 5 eddy times", "fine_dt": s.dt_fine,
                       "coarse_dt": s.dt_coarse, "coarse_precision": "fp32 transforms" if s.coarse_precision else "fp64",
                       "eval_runs": s.eval_runs, "cal_runs": s.cal_runs, "samples": s.samples},
            "spectrum_error": {"avg_spectrum_closure": ev["err_avg_closure"], "avg_spectrum_plain_coarse": ev["err_avg_plain"],
                               "mean_per_sample_closure": ev["mean_err_closure"],
                               "mean_per_sample_plain_coarse": ev["mean_err_plain"], "shells": ev["kmax"],
                               "fallback": ev["fallback"]},
            "a_priori": out["train"]["val"], "alpha": out["alpha"], "nu_e": out["nu_e"],
            "calibration": ({k: out["calibration"][k] for k in ("err_avg", "fallback", "best", "best_nu", "seed", "runs")}
                            if "calibration" in out else None),
            "energy_first_last": {k: [v[0], v[-1]] for k, v in ev["energy"].items()},
            "throughput": tp, "train": {k: out["train"][k] for k in ("train_steps", "wall_s", "best_epoch")},
            "data_gen_s": out["data"]["train"]["wall_s"]}
    print(json.dumps(line, default=str), flush=True)


def run_cufft(args) -> None:
    """Comparison only: cuFFT (through torch.fft) doing just the transforms of
    one right-hand side -- 4 inverse 2D c2r of (N, N/2+1) spectra and 1 forward
    2D r2c -- against one complete fused right-hand side of ours (Poisson
    inversion, derivatives, the same transforms, the dealiased product and the
    stage update), at N^2 in FP64 and in the FP32 form.  CUDA events; ours from
    tara2d_step_timed (an RK4 step is four right-hand sides)."""
    import torch

    import tara_gb300 as tg

    torch.cuda.set_device(0)
    n = args.n
    reps = max(3, args.steps)
    out = {}
    for name, cdt, rdt, prec in (("fp64", torch.complex128, torch.float64, tg.PREC_FP64),
                                 ("fp32", torch.complex64, torch.float32, tg.PREC_FP32)):
        g = torch.Generator(device="cuda").manual_seed(11)
        spec = torch.randn(4, n, n // 2 + 1, dtype=cdt, device="cuda", generator=g)
        real = torch.randn(n, n, dtype=rdt, device="cuda", generator=g)
        for _ in range(args.warmup):
            torch.fft.irfft2(spec, s=(n, n))
            torch.fft.rfft2(real)
        st = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        for _ in range(reps):
            torch.fft.irfft2(spec, s=(n, n))
            torch.fft.rfft2(real)
        b.record(st)
        torch.cuda.synchronize()
        cufft_ms = a.elapsed_time(b) / reps
        s = tg.Solver2D(n, scheme=tg.SCHEME_RK4, precision=prec, nu=NU, dt=DT)
        s.init_random(K0, ENERGY, SEED.get(n, 1))
        s.autotune(2)
        s.step(args.warmup)
        ours_ms = s.step_timed(reps)["total_ms"] / (4 * reps)
        s.close()
        out[name] = {"cufft_transforms_ms": cufft_ms, "ours_full_rhs_ms": ours_ms,
                     "ratio_cufft_over_ours": cufft_ms / ours_ms}
        del spec, real
    line = {"metric": f"one RHS at {n}^2: cuFFT transforms only vs our fused RHS (comparison)",
            "value": out["fp64"]["ratio_cufft_over_ours"], "unit": "x (cuFFT time / ours)", "n_gpus": 1,
            "steps": reps, "warmup": args.warmup, "higher_is_better": True, "vs_baseline": None,
            "dtype": "f64 and f32", "data": "synthetic (random spectra / seeded state)",
            "config": {"workload": "cuFFT comparison", "cufft": "torch.fft.irfft2 of 4 fields + rfft2 of 1",
                       "ours": "tara2d RK4 step / 4 (3 fused kernels per RHS)"},
            "results": out}
    print(json.dumps(line), flush=True)


def run_fno_train(args, emit: bool = True) -> dict:
    """Training step of the closure network: 128^2, 6 input channels, 4 Fourier
    layers, 32 channels, 16 modes per axis, projection 128, batch 32, BF16
    tensor-core GEMMs with FP32 accumulation, Adam (lr 1e-4) on seeded random
    data; CUDA events on the network's stream."""
    import torch

    import tara_gb300 as tg

    torch.cuda.set_device(0)
    B = 32
    net = tg.FNO(tg.fno_default_config(ci=6, max_batch=B))
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(B, 128, 128, 6, device="cuda", generator=g)
    t = torch.randn(B, 128, 128, 2, device="cuda", generator=g)
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        net.train_step(x.data_ptr(), t.data_ptr(), B, lr=1e-4, want_loss=False)

    def steps():
        for _ in range(args.steps):
            net.train_step(x.data_ptr(), t.data_ptr(), B, lr=1e-4, want_loss=False)

    ms = timed_on_stream(net.stream, steps)
    # the same step with the channel GEMMs on tcgen05 (accumulators in tensor memory)
    net.set_mode(tg.FNO_BF16_TMEM)
    for _ in range(args.warmup):
        net.train_step(x.data_ptr(), t.data_ptr(), B, lr=1e-4, want_loss=False)
    ms_tc = timed_on_stream(net.stream, steps)
    net.train_step(x.data_ptr(), t.data_ptr(), B, lr=0.0)  # reports a tensor-memory wait that gave up
    net.set_mode(tg.FNO_BF16)
    line = {"metric": "closure-network training samples/s (128^2, 6->32 ch, 4 layers, 16 modes, batch 32)",
            "value": B * args.steps / (ms * 1e-3), "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "vs_baseline": None, "dtype": "bf16 GEMM operands / f32 accumulation and activations",
            "data": "synthetic (seeded normal inputs and targets)",
            "config": {"workload": "FNO train step", "batch": B, "params": net.num_params},
            "gemm_forms_ms_per_step": {"mma.sync (value)": ms / args.steps, "tcgen05 + TMEM": ms_tc / args.steps}}
    if emit:
        print(json.dumps(line), flush=True)
    net.close()
    return line


def run_closure_step(args, emit: bool = True) -> dict:
    """One coarse closure step at 128^2: the 6 feature channels of the state,
    the FNO forward (batch 1, the fused inference kernels), the flux divergence
    and an RK4 step of the FP32-form solver (dt 4e-3, nu 5e-5), replayed as one
    CUDA graph; CUDA events on the solver's stream.  Random-initialised network
    (the cost does not depend on the weights).  Beside it, the plain 1024^2
    FP64 RK4 step (dt 5e-4, autotuned) that the closure replaces, and the ratio
    of simulated time per second (the closure workload's throughput figure;
    its accuracy needs the trained network of that workload)."""
    import numpy as np
    import torch

    import tara_gb300 as tg

    torch.cuda.set_device(0)
    s = tg.Solver2D(128, scheme=tg.SCHEME_RK4, precision=tg.PREC_FP32, nu=5e-5, dt=4e-3,
                    kpi=np.pi, lx=2 * np.pi, ly=2 * np.pi)
    s.init_random(8.0, 0.5, 9000)
    tuned = s.autotune(2)
    net = tg.FNO(tg.fno_default_config(ci=6, max_batch=1))
    c = tg.Closure(s, net, np.full(6, 0.05), 0.01)
    c.step(args.warmup)
    s.synchronize()
    ms = timed_on_stream(s.stream, lambda: c.step(args.steps))
    s.synchronize()
    c.close()
    net.close()
    s.close()
    fine = tg.Solver2D(1024, scheme=tg.SCHEME_RK4, precision=tg.PREC_FP64, nu=5e-5, dt=5e-4,
                       kpi=np.pi, lx=2 * np.pi, ly=2 * np.pi)
    fine.init_random(8.0, 0.5, 9000)
    fine.autotune(2)
    fine.step(args.warmup)
    fine.synchronize()
    fsteps = max(3, args.steps // 10)
    fms = timed_on_stream(fine.stream, lambda: fine.step(fsteps)) / fsteps
    fine.close()
    cms = ms / args.steps
    line = {"metric": "closure steps/s (128^2 FP32-form RK4 + FNO subgrid flux, one run)",
            "value": args.steps / (ms * 1e-3), "unit": "steps/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": cms, "higher_is_better": True,
            "vs_baseline": None, "dtype": "bf16 GEMMs / f32 network / f64 state",
            "data": "synthetic (seeded random-phase state, random network)",
            "config": {"workload": "closure step", "graph": "one cudaGraphLaunch per step"},
            "coarse_tile_variants": tuned["variants"],
            "fine_1024_fp64_ms_per_step": fms,
            "simtime_speedup_vs_fine_1024": (4e-3 / cms) / (5e-4 / fms)}
    if emit:
        print(json.dumps(line), flush=True)
    return line


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the timed regions with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--no-side", action="store_true",
                    help="skip the short runs of the other benchmark configurations")
    ap.add_argument("--workload", default="rk4-2048",
                    choices=["rk4-2048", "ensemble", "mhd3d", "closure", "fno-train", "closure-step", "cufft",
                             "coh2d", "com2d"],
                    help="rk4-2048 is the headline; the others measure the ensemble, 3D MHD and the learned closure")
    ap.add_argument("--ens-runs-per-size", type=int, default=128,
                    help="ensemble: runs of each size per rank (the 384-run ensemble on one GPU uses 128)")
    ap.add_argument("--ens-error-steps", type=int, default=0,
                    help="ensemble: also report the per-run error vs FP64 after this many steps")
    ap.add_argument("--closure-epochs", type=int, default=20, help="closure: training epochs")
    ap.add_argument("--variants", default=None,
                    help="fixed configurations 'a,b,c' of the three step kernels (tile variant, "
                         "+4 for the radix-8 path) instead of the autotuner, for profiling")
    ap.add_argument("--ens-form", default="auto", choices=["auto", "graph", "persistent4", "persistent8"],
                    help="ensemble: the autotuner's fastest form, or a fixed one")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32", "df64"],
                    help="rk4-2048: fp32 runs the FP32 form (FP32 transforms, FP64 state), df64 the "
                         "double-float form (transforms in FP32 pairs, FP64 state); the headline is fp64")
    args = ap.parse_args()
    global PROFILE_RANGE
    PROFILE_RANGE = args.profile_range
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble":
        run_ensemble(args)
    elif args.workload == "mhd3d":
        run_mhd3d(args)
    elif args.workload in ("coh2d", "com2d"):
        run_coh2d(args)
    elif args.workload == "closure":
        run_closure(args)
    elif args.workload == "fno-train":
        run_fno_train(args)
    elif args.workload == "cufft":
        run_cufft(args)
    elif args.workload == "closure-step":
        run_closure_step(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
