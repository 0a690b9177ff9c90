"""CPU, two processes over gloo: the N > 1 host logic of bench.py -- every
rank times its own replica, the job time is the slowest rank's (max over
ranks), the rate counts all ranks' work, replicas get distinct seeds, and
only rank 0 runs and prints the reference arm."""
import os
import socket
import sys
import types

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from tests.conftest import REPO


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, ws: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(REPO))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, _ = bench.dist_setup()
        local_ms = 1.0 + 0.5 * rank                      # rank 1 is the slow replica
        job_ms = bench.max_over_ranks(local_ms, ws)
        dist.barrier()
        args = types.SimpleNamespace(N=2, log2I=6, R=4, J=64, warmup=1, steps=1)
        ref_line = bench.run_reference(args, ws, rank)
        out[rank] = {"ws": got_ws, "rank": got_rank, "job_ms": job_ms,
                     "rate": bench.whole_job_rate(ws, 50000, job_ms / 1e3),
                     "seeds": bench.replica_seeds(rank), "ref_is_none": ref_line is None,
                     "ref_impl": None if ref_line is None else ref_line["impl"]}
    finally:
        dist.destroy_process_group()


def test_bench_multirank_host_logic_gloo():
    pytest.importorskip("numpy")
    ws = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(ws, _free_port(), out), nprocs=ws, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for r in (0, 1):
        assert res[r]["ws"] == 2 and res[r]["rank"] == r
        assert res[r]["job_ms"] == 1.5                     # the slowest replica
        assert res[r]["rate"] == pytest.approx(2 * 50000 / 1.5e-3)
    assert res[0]["seeds"]["factors"] != res[1]["seeds"]["factors"]
    assert res[0]["seeds"]["sampler"] != res[1]["seeds"]["sampler"]
    assert not res[0]["ref_is_none"] and res[0]["ref_impl"] == "reference"
    assert res[1]["ref_is_none"]                           # rank 1 runs no reference work


def test_bench_spawns_its_own_ranks():
    """`bench.py --gpus 2` without an external launcher relaunches itself as
    two ranks (torch.distributed.run on 127.0.0.1); the ranks rendezvous,
    take the max over ranks and only rank 0 prints its line."""
    import json
    import subprocess
    env = dict(os.environ)
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    res = subprocess.run([sys.executable, str(REPO / "bench.py"), "--gpus", "2", "--workload", "launcher-check"],
                         capture_output=True, text=True, timeout=240, env=env, cwd=str(REPO))
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(ln) for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    line = lines[0]
    assert line["n_gpus"] == 2 and line["rank"] == 0 and line["local_rank"] == 0
    assert line["max_over_ranks"] == 2.0                   # rank 1's value
    assert line["whole_job_rate"] == 2 * 100.0 / 2.0
