"""bench.py's JSON contract on the CPU: the reference arm (the oracle on the host
cores) prints one line with every key the contract names, ranks other than 0
print nothing, and the FP64 instruction count behind the FP64-pipe roofline
matches the transform's butterflies."""
from __future__ import annotations

import json
import os
import subprocess
import sys

from conftest import ROOT

import bench

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"}


def _run(args, **env):
    e = dict(os.environ, CUDA_VISIBLE_DEVICES="", **env)
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                          timeout=300, cwd=str(ROOT), env=e)


def test_reference_arm_line():
    r = _run(["--impl", "reference", "--n", "64", "--steps", "2", "--warmup", "3"])
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3
    assert d["unit"] == bench.UNIT and d["metric"] == bench.METRIC and d["higher_is_better"] is True
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= set(cb) and cb["value"] == d["value"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_are_silent():
    r = _run(["--impl", "reference", "--n", "64", "--steps", "2", "--warmup", "3"], RANK="1", WORLD_SIZE="2")
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def test_warmup_is_at_least_three():
    r = _run(["--impl", "reference", "--n", "32", "--steps", "1", "--warmup", "0"])
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1])["warmup"] == 3


def test_fft_fp64_instruction_count():
    # 2048 = 8 * 4^4: an untwiddled radix-8 stage, then 4 ratio-form radix-4 stages
    assert bench.fft_fp64_inst(2048) == 256 * 52 + 512 * 22 * 4 == 58368
    # 1024 = 4^5: an untwiddled radix-4 stage, then 4 ratio-form ones
    assert bench.fft_fp64_inst(1024) == 256 * 16 + 256 * 22 * 4
    for n in (16, 32, 64, 128, 256, 512, 1024, 2048):
        lg = n.bit_length() - 1
        # about 3 FP64 instructions per point per radix-2 stage, fewer for the untwiddled first stage
        assert 2.0 * n * lg <= bench.fft_fp64_inst(n) <= 3.0 * n * lg


def test_cpu_baseline_thread_counts():
    """The all-core port baseline and the single-thread one (the reference's own
    2D path is single-threaded) report the threads they used."""
    one = bench.cpu_baseline(64, budget_s=0.2, threads=1)
    assert one["cores"] == 1 and one["value"] > 0 and one["kind"] == "port"
    many = bench.cpu_baseline(64, budget_s=0.2)
    assert many["cores"] >= 1 and many["unit"] == bench.UNIT
