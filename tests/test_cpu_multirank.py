"""The multi-rank (N>1) path on CPU with the gloo backend, world size 2.

bench.py --gpus N runs one replica per GPU ("replicas only": every rank owns its lattice and
the data path has no collective); the ranks meet only in a barrier around the timed region
and in the max over ranks of the elapsed time, and rank 0 prints the one JSON line.  The
reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    bench.barrier(dist)
    ms = bench.max_over_ranks(dist, 10.0 + 5.0 * rank)  # rank 1 is the slower replica
    bench.barrier(dist)
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as fh:
        json.dump({"rank": rank, "max_ms": ms}, fh)
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    pytest.importorskip("torch.distributed")
    import torch.multiprocessing as mp
    port = free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for rank in (0, 1):
        got = json.load(open(os.path.join(str(tmp_path), "rank%d.json" % rank)))
        assert got["max_ms"] == 15.0, got


def test_reference_arm_under_torchrun():
    pytest.importorskip("torch.distributed")
    port = free_port()
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--size", "16", "--steps", "2", "--warmup", "3"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
