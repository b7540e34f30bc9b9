"""Sharding of the ensemble across ranks (tara_gb300/shard.py, bench.py's
ensemble workload): the cost-balanced partition on one process, and the
multi-rank host logic -- max-over-ranks time, summed launch counts, the gather
of per-run error scalars to rank 0 -- as world_size-2 gloo ranks on the CPU."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

import bench
from tara_gb300 import shard


# ------------------------------------------------------------------ one process
def test_partition_covers_each_run_once():
    sizes = [128, 512, 256, 512, 128, 128, 256, 64, 1024, 128, 256]
    for ws in (1, 2, 3, 4, 8, 16):
        parts = shard.partition_runs(sizes, ws)
        assert len(parts) == ws
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(sizes)))
        assert all(p == sorted(p) for p in parts)


def test_partition_one_rank_keeps_the_global_order():
    runs = bench.ensemble_runs(128, 1)
    idx, mine = shard.shard_of(runs, 0, 1)
    assert idx == list(range(len(runs))) and mine == runs


@pytest.mark.parametrize("ws", [2, 4, 8])
def test_bench_ensemble_shards_have_the_same_mix(ws):
    """Weak scaling: every rank of the bench's ensemble holds per runs of each
    size, so each shard is the one-GPU workload's shape."""
    per = 128
    runs = bench.ensemble_runs(per, ws)
    assert len(runs) == 3 * per * ws
    assert runs[: per] == bench.ensemble_runs(per, 1)[: per]  # same k0 stream, same seeds
    for r in range(ws):
        _, mine = shard.shard_of(runs, r, ws)
        counts = {n: sum(1 for m, _, _ in mine if m == n) for n in (128, 256, 512)}
        assert counts == {128: per, 256: per, 512: per}


def test_partition_balances_uneven_costs():
    sizes = [512] * 5 + [256] * 7 + [128] * 13
    parts = shard.partition_runs(sizes, 3)
    loads = [sum(shard.run_cost(sizes[i]) for i in p) for p in parts]
    # longest-processing-time bound: max load <= mean + the largest single cost
    assert max(loads) <= sum(loads) / 3 + shard.run_cost(512)


def test_partition_is_deterministic_and_rejects_bad_world_size():
    sizes = [128, 256, 512] * 9
    assert shard.partition_runs(sizes, 4) == shard.partition_runs(list(sizes), 4)
    with pytest.raises(ValueError):
        shard.partition_runs(sizes, 0)


def test_gather_single_process():
    assert shard.gather_by_index([2, 0, 1], [0.2, 0.0, 0.1], 3) == [0.0, 0.1, 0.2]
    with pytest.raises(ValueError):
        shard.gather_by_index([0, 0], [1.0, 2.0], 2)
    with pytest.raises(ValueError):
        shard.gather_by_index([0], [1.0], 2)
    with pytest.raises(ValueError):
        shard.gather_by_index([0, 1], [1.0], 2)
    assert shard.max_over_ranks(3.5) == 3.5 and shard.sum_over_ranks(2) == 2.0


# ------------------------------------------------------------------ gloo ranks
def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _spawn(tmp_path, mode: str, ws: int = 2, per: int = 4):
    """Start ws ranks of shard_worker.py; returns (rank 0's output file, logs)."""
    out = tmp_path / f"rank0_{mode}.json"
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()),
               WORLD_SIZE=str(ws), CUDA_VISIBLE_DEVICES="")
    procs = [subprocess.Popen([sys.executable, str(ROOT / "tests" / "shard_worker.py"), str(out), mode, str(per)],
                              env=dict(env, RANK=str(r), LOCAL_RANK=str(r)), cwd=str(ROOT),
                              stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
             for r in range(ws)]
    logs = []
    try:
        for p in procs:
            logs.append(p.communicate(timeout=240)[0].decode(errors="replace"))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    assert all(p.returncode == 0 for p in procs), "\n".join(logs)
    return out, logs


def _run_ranks(tmp_path, mode: str, ws: int = 2, per: int = 4) -> dict:
    out, _ = _spawn(tmp_path, mode, ws, per)
    return json.loads(out.read_text())


def test_gloo_two_ranks_gather_and_reduce(tmp_path):
    res = _run_ranks(tmp_path, "ok")
    assert res["max_t"] == 2.5                      # max over ranks of 1.5 + rank
    assert res["sum_launches"] == 30.0              # 10 + 20
    assert res["gathered"] == res["expected"]       # global order restored on rank 0
    a, b = res["all_indices"]
    assert sorted(a + b) == list(range(24)) and not set(a) & set(b)


@pytest.mark.parametrize("mode", ["duplicate", "missing"])
def test_gloo_gather_detects_bad_shards(tmp_path, mode):
    res = _run_ranks(tmp_path, mode)
    assert "gathered" not in res
    assert ("twice" in res["error"]) if mode == "duplicate" else ("no rank" in res["error"])


def test_gloo_two_ranks_bench_ensemble_line(tmp_path):
    """bench.py --workload ensemble on two gloo ranks (stand-ins for the GPU
    objects): one JSON line from rank 0 only, the time the slower rank's, the
    points of both shards, launches summed, and the per-run errors gathered in
    global order."""
    per = 4
    _, logs = _spawn(tmp_path, "bench", per=per)
    lines0 = [l for l in logs[0].splitlines() if l.startswith("{")]
    assert len(lines0) == 1 and not any(l.startswith("{") for l in logs[1].splitlines())
    line = json.loads(lines0[0])
    runs = bench.ensemble_runs(per, 2)
    pts = sum(n * n for n, _, _ in runs)
    assert line["n_gpus"] == 2 and line["scaling"] == "weak" and line["steps"] == 2
    assert line["ms_per_step"] == pytest.approx(11.0 / 2)      # max over ranks of 10 + rank ms
    assert line["value"] == pytest.approx(pts * 2 / 11e-3)
    assert line["gpu_launches"] == 2 * 36 * 2
    errs = [1e-7 * seed / 4000.0 for _, _, seed in runs]
    ev = line["error_vs_fp64"]
    assert ev["max"] == pytest.approx(max(errs), rel=1e-6)
    for n in (128, 256, 512):
        assert ev["per_size_max"][str(n)] == pytest.approx(
            max(e for (m, _, _), e in zip(runs, errs) if m == n), rel=1e-6)
