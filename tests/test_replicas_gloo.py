"""The several-GPU form of bench.py is replicas only (every rank runs the
whole workload on its own GPU, no data-path collective); its host logic --
rendezvous, barrier, max over ranks of the step time, rank 0 alone printing
-- runs here as world_size-2 gloo ranks on the CPU."""
import json
import os
import socket
import subprocess
import sys

import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    ws_, rank_, local = bench.dist_setup()
    assert (ws_, rank_, local) == (ws, rank, rank)
    assert dist.get_backend() == "gloo"
    # each rank's step time; the job's time is the slowest rank's
    t = bench.max_over_ranks(1.5 + rank, ws_, torch.device("cpu"))
    bench.barrier(ws_)
    out[rank] = t
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_on_gloo():
    ws = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_rank_main, args=(ws, _free_port(), out), nprocs=ws, join=True)
    assert dict(out) == {0: 1.5 + ws - 1, 1: 1.5 + ws - 1}


def test_reference_arm_under_torchrun_prints_once():
    """bench.py --impl reference launched as two ranks: rank 0 times the CPU
    reference and prints one JSON line, rank 1 exits without work."""
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "sdf_queries_per_s" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
