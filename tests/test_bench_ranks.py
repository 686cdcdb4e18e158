"""The replica path of bench.py on two gloo ranks (CPU): every rank reports the job's clock,
the largest per-rank step time, and a single rank is left untouched."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    assert bench.dist_info() == (rank, world, rank)
    out[rank] = bench.max_over_ranks(10.0 + 7.5 * rank, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        assert dict(out) == {0: 17.5, 1: 17.5}


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, "cpu") == 3.25


def _run_reference(tmp_path, rank="0"):
    import json
    import subprocess
    env = dict(os.environ, RANK=rank, WORLD_SIZE="2" if rank != "0" else "1", LOCAL_RANK=rank)
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "1", "--steps", "1", "--warmup", "1",
                          "--data", str(tmp_path)], capture_output=True, text=True, env=env,
                         timeout=600, check=True)
    return [json.loads(l) for l in out.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line(tmp_path):
    """bench.py --impl reference (the CPU restatement of the reference's step, on the n = 16
    workload here) prints one line with the bench contract's keys on rank 0, and nothing on
    the other ranks."""
    lines = _run_reference(tmp_path)
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["unit"] == "s" and d["value"] > 0
    assert d["higher_is_better"] is False and d["n_gpus"] == 1 and d["steps"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"] and d["config"]["n_dets"] > 0
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0
    assert _run_reference(tmp_path, rank="1") == []
