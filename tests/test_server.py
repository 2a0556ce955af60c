"""The library's request loop (sph_server_*) on the real pool.

A seeded stream of small DFSPH scenes is submitted from this thread while the
server's driver steps the pool, on a pool too small to hold them all at once
(so scenes wait, join between epochs while others are mid-run, and leave as
they complete).  Every scene completes its steps, and its final positions and
velocities equal, bit for bit, the same scene run alone in a pool of its own:
the pool's per-scene reductions are fixed-point integer sums, so nothing
depends on what else is resident or on when the scene was admitted."""
import math
import time

import numpy as np
import pytest

import sph_gb300
from scenes import jitter

pytestmark = pytest.mark.gpu


def stream(n_scenes=10, seed=11):
    from sph_gb300 import workloads

    rng = np.random.default_rng(seed)
    out = []
    for k in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(300), math.log(2500)))))
        x, b, p, _ = workloads.make_scene(rng, n, r=0.02, box_side=0.6)
        out.append((jitter(x, 0.02, 200 + k), b, p, int(rng.integers(8, 40))))
    return out


def test_served_scenes_equal_scenes_run_alone(gpu_lib):
    scenes = stream()
    total = sum(s[0].shape[0] for s in scenes)
    P = sph_gb300.Pool(max_particles=total // 3, max_boundary=400_000, max_keys=4_000_000, max_scenes=16)
    P.set_graph(True)
    srv = sph_gb300.Server(P, epoch_steps=4, lookahead=4, keep_results=True)
    ids = []
    for x, b, p, steps in scenes:
        ids.append(srv.submit(x, boundary_points=b, steps=steps, **p))
        time.sleep(0.01)
    assert srv.drain(120.0)
    st = srv.stats()
    assert st["completed"] == len(scenes) and st["failed"] == 0 and st["queued"] == 0
    assert st["particle_steps"] == sum(s[0].shape[0] * s[3] for s in scenes)
    assert 0 < st["p50_latency_s"] <= st["p99_latency_s"]
    for rid, (x, b, p, steps) in zip(ids, scenes):
        info = srv.query(rid)
        assert info["state"] == sph_gb300.REQUEST_DONE and info["steps_done"] == steps and info["status"] == 0
        A = sph_gb300.Pool(max_particles=x.shape[0], max_boundary=b.shape[0], max_keys=1_000_000, max_scenes=1)
        A.set_graph(True)
        a = A.add_scene(x, boundary_points=b, steps=steps, **p)
        A.step(steps)
        assert np.array_equal(srv.fetch(rid, "x"), A.get(a, "x"))
        assert np.array_equal(srv.fetch(rid, "v"), A.get(a, "v"))
        A.close()
    srv.close()


def test_server_reports_a_failing_scene_and_keeps_serving(gpu_lib):
    """A scene the pool rejects (not DFSPH) fails at admission; a NaN scene
    is retired with its status; the others complete."""
    scenes = stream(4, seed=3)
    P = sph_gb300.Pool(max_particles=100_000, max_boundary=400_000, max_keys=4_000_000, max_scenes=16)
    srv = sph_gb300.Server(P, epoch_steps=4)
    x, b, p, _ = scenes[0]
    bad = srv.submit(x, boundary_points=b, steps=5, **dict(p, method=0))
    xn = x.copy()
    xn[0, 0] = np.nan
    nan = srv.submit(xn, boundary_points=b, steps=50, **p)
    good = [srv.submit(x, boundary_points=b, steps=s, **p) for x, b, p, s in scenes[1:]]
    assert srv.drain(120.0)
    assert srv.query(bad)["state"] == sph_gb300.REQUEST_FAILED
    q = srv.query(nan)
    assert q["state"] == sph_gb300.REQUEST_DONE and q["status"] & sph_gb300.STATUS_NONFINITE and q["steps_done"] < 50
    for g in good:
        assert srv.query(g)["state"] == sph_gb300.REQUEST_DONE and srv.query(g)["status"] == 0
    srv.close()
