"""bench.py's multi-process plumbing on the host: the max-over-ranks reduction
with two gloo ranks, and the reference arm (the oracle on the host cores)
launched under torchrun with two ranks, where rank 0 alone prints its line."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as tdist

    import bench

    tdist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        out[rank] = bench.max_over_ranks(1.5 + rank, True)
    finally:
        tdist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp

    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_reference_arm_two_ranks():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "3", "--warmup", "1",
           "--workload", "tg100_f64"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port"
    # the line contract: the same metric, unit and direction as the GPU arm
    for k in ("metric", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "dtype", "data", "config"):
        assert k in d, k
    assert d["unit"] == "MLUPS" and d["higher_is_better"] is True and d["n_gpus"] == 2
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["unit"] == d["unit"]
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert "workload" in d["config"]


def test_reference_arm_maps_no_cuda_library():
    """the reference arm (the oracle on the host cores) builds its workload
    without loading the product's CUDA library, and prints the same config
    as the GPU arm"""
    code = (
        "import json, sys, types\n"
        "sys.argv = ['bench.py']\n"
        "import bench\n"
        "args = types.SimpleNamespace(steps=1, warmup=1, gpus=1, workload='tg100_f64')\n"
        "bench.run_reference(args, 0, 1)\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('MAPPED' if 'librrlbm' in maps else 'CLEAN')\n"
        "p, st = bench.make('tg100_f64')\n"
        "print(json.dumps(bench.config_of('tg100_f64', p, 1)))\n")
    env = dict(os.environ, OMP_NUM_THREADS="2")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    out = r.stdout.splitlines()
    assert "CLEAN" in out, r.stdout
    line = json.loads([l for l in out if l.startswith('{"metric"')][0])
    assert line["config"] == json.loads(out[-1])
    assert "f64" not in line["config"]["workload"] and line["dtype"] == "f64"
