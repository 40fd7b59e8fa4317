"""The multi-process paths of bench.py on the CPU: the max-over-ranks timing reduction with two gloo
ranks, and the reference arm under torchrun with two ranks (rank 0 alone works and prints one JSON
line; the other rank exits 0 without work).  A DMRG update does not shard: N GPUs run N replicas."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(1.5 + rank, dist, "cpu")
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank_main, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_max_over_ranks_single_process_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25


def _reference_json(cmd):
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    return lines


def _check_reference_line(d):
    assert d["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config"):
        assert k in d
    assert d["value"] > 0 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


ARGS = ["--impl", "reference", "--chi", "16", "--L", "12", "--steps", "1", "--warmup", "1"]


def test_reference_arm_json_line():
    lines = _reference_json([sys.executable, "bench.py"] + ARGS)
    assert len(lines) == 1
    _check_reference_line(json.loads(lines[0]))


def test_reference_arm_under_torchrun_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--gpus", "2"] + ARGS
    lines = _reference_json(cmd)
    assert len(lines) == 1  # rank 0 only
    d = json.loads(lines[0])
    _check_reference_line(d)
    assert d["n_gpus"] == 2


def test_reference_arm_tv_model():
    lines = _reference_json([sys.executable, "bench.py", "--model", "tv"] + ARGS)
    assert len(lines) == 1
    d = json.loads(lines[0])
    _check_reference_line(d)
    assert d["config"]["workload"].startswith("tv_L12_chi16") and d["config"]["N_particles"] == 6
