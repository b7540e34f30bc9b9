"""One rank of the sharded-ensemble host logic over gloo (run by test_shard.py).

Usage: RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT in the environment;
argv = output JSON path, mode ("ok", "duplicate", "missing", or "bench" for
bench.py's ensemble workload with stand-ins for the GPU objects), runs per size
per rank.
Each rank takes its shard of the bench's global run list, makes one scalar per
run from the run itself (so rank 0 can check the gathered order), a
rank-dependent "time", and rank 0 writes what the collectives returned.
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def main() -> None:
    import torch.distributed as dist

    import bench
    from tara_gb300 import shard

    out, mode, per = sys.argv[1], sys.argv[2], int(sys.argv[3])
    dist.init_process_group("gloo", init_method="env://")
    rank, ws = dist.get_rank(), dist.get_world_size()
    runs = bench.ensemble_runs(per, ws)
    idx, mine = shard.shard_of(runs, rank, ws)
    vals = [n + 1e-6 * seed for n, _, seed in mine]
    if mode == "duplicate" and rank == ws - 1:  # report rank 0's first run a second time
        other = shard.partition_runs([r[0] for r in runs], ws)[0][0]
        idx, vals = idx + [other], vals + [0.0]
    if mode == "missing" and rank == ws - 1:
        idx, vals = idx[1:], vals[1:]
    res = {"rank": rank, "indices": idx,
           "max_t": shard.max_over_ranks(1.5 + rank, dist),
           "sum_launches": shard.sum_over_ranks(10 * (rank + 1), dist)}
    try:
        g = shard.gather_by_index(idx, vals, len(runs), dist)
        res["gathered"] = g
    except ValueError as e:
        res["error"] = str(e)
    all_idx = [None] * ws
    dist.all_gather_object(all_idx, idx)
    res["all_indices"] = all_idx
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        res["expected"] = [n + 1e-6 * seed for n, _, seed in runs]
        Path(out).write_text(json.dumps(res))


def bench_ensemble() -> None:
    """bench.py's ensemble workload on this rank with the GPU objects replaced by
    stand-ins: each run's "FP32" state differs from its "FP64" one by a factor
    1 + 1e-7 * seed / 4000, and rank r's timed region takes 10 + r ms, so rank 0's
    line can be checked against the shard logic."""
    import types

    import numpy as np
    import torch

    import bench
    import tara_gb300 as tg

    class Ensemble:
        def __init__(self, runs, precision, nu, dt):
            self.runs, self.fp32 = list(runs), precision == tg.PREC_FP32

        def autotune(self, trial_steps):
            pass

        def step(self, n):
            pass

        def synchronize(self):
            pass

        stream = 0
        launches_per_step = 36

        def groups(self):
            return []

        def form(self):
            return {"form": "graph", "ms_per_step": {"graph": 1.0}}

        def get_state(self, r):
            n, _, seed = self.runs[r]
            w = np.full((n, n // 2 + 1), 1.0 + 0.5j)
            return w * (1.0 + 1e-7 * seed / 4000.0) if self.fp32 else w

        def close(self):
            pass

    tg.Ensemble = Ensemble
    torch.cuda.set_device = lambda d: None
    rank = int(os.environ["RANK"])
    bench.timed_on_stream = lambda stream, fn: (fn(), 10.0 + rank)[1]
    per = int(sys.argv[3])
    bench.run_ensemble(types.SimpleNamespace(ens_runs_per_size=per, warmup=3, steps=2, ens_error_steps=10))
    import torch.distributed as dist

    dist.destroy_process_group()


if __name__ == "__main__":
    if sys.argv[2] == "bench":
        bench_ensemble()
    else:
        main()
