"""The replica path of bench.py on CPU (world size 2, gloo): the
max-over-ranks reduction of the timings, and the reference arm under
torchrun, where rank 0 alone samples and prints one JSON line and the other
rank exits 0 without work."""

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_max_over_ranks_with_two_gloo_ranks():
    code = ("import sys, torch, torch.distributed as dist; sys.path.insert(0, %r); import bench; "
            "dist.init_process_group('gloo'); r = dist.get_rank(); "
            "print(bench.max_over_ranks(r + 0.25, torch.device('cpu')), flush=True); "
            "dist.destroy_process_group()" % str(ROOT))
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()), WORLD_SIZE="2")
    procs = [subprocess.Popen([sys.executable, "-c", code], env=dict(env, RANK=str(r)), stdout=subprocess.PIPE,
                              stderr=subprocess.PIPE, text=True) for r in range(2)]
    outs = []
    for p in procs:
        try:
            out, err = p.communicate(timeout=180)
        except subprocess.TimeoutExpired:
            for q in procs:
                q.kill()
            raise
        assert p.returncode == 0, err
        outs.append(float(out.strip().splitlines()[-1]))
    assert outs == [1.25, 1.25]


def test_max_over_ranks_without_a_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    import torch

    assert bench.max_over_ranks(3.5, torch.device("cpu")) == 3.5


def test_reference_arm_under_torchrun_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--L", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
    assert d["same_config"] and d["config"]["L"] == 2 and d["cpu_baseline"]["thread_speedup"] > 0
