"""The benchmark's multi-GPU path is replicas only (independent scene pools,
one per rank, no data-path collective): its host logic under two `gloo`
ranks on the CPU.  Each rank's timed region ends at a barrier, the whole-job
value uses the maximum time over ranks, and the reference arm is run and
printed by rank 0 alone while the other ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    w, r, _ = bench.dist_setup()
    ms = 10.0 + 5.0 * r           # rank-dependent step time
    bench.dist_barrier(w)
    t_max = bench.dist_max(ms, w)
    n, steps = 1000, 4
    value = w * n * steps / (t_max / 1000.0)
    q.put((r, w, t_max, value))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_max_time_and_value():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2, 2]
    assert out[0][2] == out[1][2] == 15.0            # max over ranks
    assert out[0][3] == out[1][3] == 2 * 1000 * 4 / 0.015


def test_reference_arm_under_torchrun_prints_once():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--ref-budget", "2"]
    p = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=900, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0


def test_reference_arm_never_loads_the_cuda_library():
    """The reference arm times the CPU algorithm on scenes sampled by the
    oracle's own samplers: the process maps no library of the CUDA path."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3', "
            "'--ref-budget', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); print('CUDA_LIB_MAPPED', 'libsph_gb300' in maps)")
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=900, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    assert "CUDA_LIB_MAPPED False" in p.stdout
    line = json.loads([ln for ln in p.stdout.splitlines() if ln.startswith("{")][0])
    assert line["impl"] == "reference" and line["value"] > 0
