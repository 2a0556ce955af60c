"""Host-side logic of the batched/served workloads: seeded scene generators
and the benchmark's reference arm contract.  (The request loop's host logic
is tested in test_server_host.py.)"""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

import sph_gb300
from sph_gb300 import workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_batched_mix_is_seeded_and_sized():
    a = workloads.batched_mix(n_scenes=256, seed=42, steps=500)
    b = workloads.batched_mix(n_scenes=256, seed=42, steps=500)
    assert len(a) == 256
    n = np.array([s[0].shape[0] for s in a])
    assert int(n.sum()) == 4151352
    assert n.min() >= 1000 and n.max() <= 70000
    for (xa, ba, pa, sa), (xb, bb, pb, sb) in zip(a[:8], b[:8]):
        assert np.array_equal(xa, xb) and np.array_equal(ba, bb) and pa == pb and sa == sb == 500
    # fluid inside the 1 m box, 2r off the walls; boundary points on or inside it
    for x, bnd, p, _ in a[:32]:
        r = p["radius"]
        assert x.min() >= 2 * r - 1e-9 and x.max() <= 1.0 - 2 * r
        assert bnd.min() >= -1e-9 and bnd.max() <= 1.0 + 1e-9
        assert p["method"] == 2 and p["boundary"] == 2 and p["eta"] == 0.001


def test_sphere_obstacles_keep_clear_of_the_fluid():
    rng = np.random.default_rng(3)
    for _ in range(20):
        x, b, p, _ = workloads.make_scene(rng, 8000)
        h = 4 * p["radius"]
        box = sph_gb300.sample_box(h, (0, 0, 0), (1, 1, 1))
        extra = b[box.shape[0]:]
        if extra.shape[0] == 0:
            continue
        # every obstacle point is at least h from every fluid particle
        d2 = ((x[:, None, :] - extra[None, ::7, :]) ** 2).sum(-1)
        assert d2.min() >= h * h


def test_request_stream_is_poisson_with_periodic_big_scene():
    reqs = workloads.request_stream(rate=200, duration=10.0, seed=7, big_every=10.0)
    t = np.array([q[0] for q in reqs])
    assert np.all(np.diff(t) >= 0)
    assert 1800 < len(reqs) < 2200
    assert sum(1 for q in reqs if q[0] == 10.0) >= 1
    x, b, p, steps = reqs[0][1]()
    assert 200 <= steps <= 2000 and 1000 * 0.5 <= x.shape[0] <= 200000 * 1.5


def test_dam_break_sizes():
    x, b, p, steps = workloads.dam_break()
    assert x.shape[0] == 125000 and b.shape[0] == 60802 and steps == 2000 and p["radius"] == 0.005


def test_reference_arm_prints_contract_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--ref-budget", "2"], capture_output=True, text=True, env=env, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "particle-steps/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["config"]["workload"] == "batched_mix_256"
