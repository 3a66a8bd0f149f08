"""The N>1 path of bench.py on CPU with world_size-2 gloo process groups: the path does not
shard ("replicas only"), so the only cross-rank operations are the timing reductions (max over
ranks, sum over ranks, barriers), and under torchrun the reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out_path):
    os.environ.update({"WORLD_SIZE": "2", "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local = bench.dist_setup()
    res = {"ws": ws, "rank": r,
           "max": bench.dist_max(float(r + 1) * 1.5, ws),
           "sum": bench.dist_sum(float(r + 1), ws)}
    bench.dist_barrier(ws)
    with open("%s.%d" % (out_path, rank), "w") as f:
        json.dump(res, f)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_timing_reductions_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    out = str(tmp_path / "res")
    mp.start_processes(_worker, args=(port, out), nprocs=2, join=True, start_method="spawn")
    for rank in range(2):
        with open("%s.%d" % (out, rank)) as f:
            r = json.load(f)
        assert r["ws"] == 2 and r["rank"] == rank
        assert r["max"] == 3.0 and r["sum"] == 3.0


def test_reference_arm_runs_on_rank0_only_under_torchrun():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--side", "16", "--steps", "1", "--warmup", "0", "--gpus", "2", "--ref-sweeps", "20"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["cpu_baseline"]["value"] == d["value"]
    # the timed steps are exactly --steps after --warmup, and the reference's own divergence
    # after its fixed iterations is reported
    assert d["steps"] == 1 and d["warmup"] == 0
    assert d["config"]["max_div_post_projection"] >= 0.0
