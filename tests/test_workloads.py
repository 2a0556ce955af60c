"""Host-side logic of the batched/served workloads: seeded scene generators,
the request loop's admission / continuous batching / retirement (against a
fake pool with the same interface and the same capacity error), and the
benchmark's reference arm contract."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import numpy as np

import sph_gb300
from sph_gb300 import serve, workloads

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


class FakePool:
    """Pool stand-in: capacity in particles, per-scene step counters."""

    def __init__(self, capacity):
        self.capacity, self.used, self.next = capacity, 0, 0
        self.scenes = {}
        self.steps_run = 0

    def add_scene(self, x, boundary_points=None, steps=1, **params):
        n = x.shape[0]
        if self.used + n > self.capacity:
            raise sph_gb300.PoolFull("full")
        sid = self.next
        self.next += 1
        self.scenes[sid] = [n, steps, 0]
        self.used += n
        return sid

    def step(self, k):
        self.steps_run += k
        for s in self.scenes.values():
            s[2] = min(s[1], s[2] + k)

    def synchronize(self):
        pass

    def poll(self):
        return [sid for sid, s in self.scenes.items() if s[2] >= s[1]]

    def remove(self, sid):
        self.used -= self.scenes.pop(sid)[0]

    def query(self, sid):
        return {"steps": self.scenes[sid][2]}, False

    def get(self, sid, field):
        return np.zeros((self.scenes[sid][0], 3))


def _tiny_requests(k, n=100, steps=30, spacing=0.0):
    x = np.zeros((n, 3))
    return [(i * spacing, lambda: (x, None, {}, steps)) for i in range(k)]


def test_serve_completes_every_request_and_counts_work():
    pool = FakePool(capacity=1000)
    out = serve.serve(pool, _tiny_requests(25), duration=60.0, epoch_steps=10)
    assert out["completed"] == 25 and out["waiting"] == 0 and out["resident"] == 0
    assert out["particle_steps"] == 25 * 100 * 30
    assert out["p50_latency_s"] is not None and out["p99_latency_s"] >= out["p50_latency_s"]
    assert pool.used == 0


def test_serve_admits_by_capacity_and_batches_continuously():
    pool = FakePool(capacity=350)   # three 100-particle scenes fit at a time
    seen = []
    real_step = pool.step

    def step(k):
        seen.append(len(pool.scenes))
        assert pool.used <= pool.capacity
        real_step(k)

    pool.step = step
    out = serve.serve(pool, _tiny_requests(10), duration=60.0, epoch_steps=10)
    assert out["completed"] == 10
    assert max(seen) == 3
    # scenes join while others are mid-run: with 30-step scenes and 10-step
    # epochs, a full batch retires together, so residency drops to 0 only at
    # the end; with staggered step counts new scenes join mid-run
    reqs = [(0.0, (lambda s=s: (np.zeros((100, 3)), None, {}, s))) for s in (10, 20, 30, 40, 50, 60)]
    pool2 = FakePool(capacity=350)
    joined = []
    orig_add = pool2.add_scene

    def add(x, **kw):
        joined.append({sid: s[2] for sid, s in pool2.scenes.items()})
        return orig_add(x, **kw)

    pool2.add_scene = add
    serve.serve(pool2, reqs, duration=60.0, epoch_steps=10)
    # some scene was admitted while another had already made progress
    assert any(any(v > 0 for v in snap.values()) for snap in joined)


def test_serve_lookahead_skips_a_scene_that_does_not_fit():
    big = np.zeros((900, 3))
    small = np.zeros((50, 3))
    reqs = [(0.0, lambda: (small, None, {}, 100)), (0.0, lambda: (big, None, {}, 10)),
            (0.0, lambda: (small, None, {}, 10))]
    pool = FakePool(capacity=920)
    order = []
    orig = pool.add_scene

    def add(x, **kw):
        sid = orig(x, **kw)
        order.append(x.shape[0])
        return sid

    pool.add_scene = add
    out = serve.serve(pool, reqs, duration=60.0, epoch_steps=10)
    assert out["completed"] == 3
    # the second small scene was admitted before the big one (look-ahead)
    assert order[:2] == [50, 50] and order[2] == 900


def test_reference_arm_prints_contract_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--ref-budget", "2"], capture_output=True, text=True, env=env, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "particle-steps/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["config"]["workload"] == "batched_mix_256"
