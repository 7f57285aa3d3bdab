"""The N > 1 path of bench.py on CPU with the gloo backend (world size 2):
replicas time independently, the step time is the maximum over ranks, the
whole-job value is world_size x per-rank units over that time, and under
torchrun only rank 0 prints the reference arm's line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, times, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    t = bench.max_over_ranks(times[rank])
    out[rank] = (t, bench.whole_job_rate(world, 1000.0, t / 1e3))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    times = [12.5, 17.25]
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(2, free_port(), times, out), nprocs=2, join=True)
        res = dict(out)
    for r in (0, 1):
        t, rate = res[r]
        assert t == max(times)
        assert rate == pytest.approx(2 * 1000.0 / (max(times) / 1e3))


def test_reference_arm_under_torchrun_prints_once(oracle):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--workload", "chain", "--qubits", "12", "--cpu-rows", "1024", "--steps", "2",
           "--warmup", "3"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
