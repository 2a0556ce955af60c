"""Failure detection through the status word, with faults injected on the
host: NaN or absurd values written into one scene's host-staged state before
it is handed to the library, and solver limits that cannot be met.  Nothing
here faults, traps or hangs the GPU.

The reference has no failure detection (no NaN checks; its solver loops stop
at maxIterations, DFSPHSolver.cpp:327,512).  Here:
  * SPH_STATUS_NONFINITE: a position or velocity is NaN / Inf (checked at
    every grid build: such a particle meets no neighbour, so no solver sum
    notices it, in the reference either) or a solver reduction saw NaN /
    Inf.  A pooled scene is retired after that step (polls report it done,
    short of its steps); the other scenes of the pool are bit-identical to a
    pool without it.
  * SPH_STATUS_DIVERGED (pool): a particle's error is too large for the
    scene's fixed-point error sum; its average then reads +Inf.
  * SPH_STATUS_ITER_CAP / _V: a solve stopped at the cap above tolerance.
"""
import numpy as np
import pytest

import oracle
import sph_gb300
from scenes import jitter, lattice
from util import relerr

pytestmark = pytest.mark.gpu

NONFINITE, ITER_CAP, ITER_CAP_V, DIVERGED = (sph_gb300.STATUS_NONFINITE, sph_gb300.STATUS_ITER_CAP,
                                             sph_gb300.STATUS_ITER_CAP_V, sph_gb300.STATUS_DIVERGED)


def mk(seed, n_side=7, r=0.02, box=0.5):
    lo = 2 * r + 0.01 * (seed % 3)
    x = jitter(lattice(r, (lo, lo, lo), (lo + 2 * r * n_side, lo + 2 * r * n_side * 0.8, lo + 2 * r * n_side)), r, seed)
    b = sph_gb300.sample_box(4 * r, (0, 0, 0), (box, box, box))
    return x, b, dict(method=2, boundary=2, radius=r, eta=0.001, eta_v=0.001, precision="f32")


CLEAN = [mk(1), mk(2, 6), mk(3, 8, box=0.6)]


def run_pool(scenes, steps, graph=True):
    P = sph_gb300.Pool(max_particles=100_000, max_boundary=200_000, max_keys=2_000_000, max_scenes=16)
    P.set_graph(graph)
    ids = [P.add_scene(x, v, boundary_points=b, steps=20, **p) for x, v, b, p in scenes]
    P.step(steps)
    P.synchronize()
    return P, ids


def with_v(scenes):
    return [(x, None, b, p) for x, b, p in scenes]


@pytest.mark.parametrize("graph", [True, False], ids=["graph", "host"])
def test_nan_scene_is_flagged_retired_and_isolated(gpu_lib, graph):
    x, b, p = mk(4)
    x = x.copy()
    x[17, 1] = np.nan                     # one position NaN in the host-staged state
    scenes = with_v(CLEAN[:2]) + [(x, None, b, p)] + with_v(CLEAN[2:])
    P, ids = run_pool(scenes, 6, graph)
    bad = ids[2]
    st, done = P.query(bad)
    assert st["status"] & NONFINITE
    assert done and st["steps"] < 20      # retired after the step that saw it
    assert bad in P.poll()
    R, rids = run_pool(with_v(CLEAN), 6, graph)
    for i, j in zip(ids[:2] + ids[3:], rids):
        s1, d1 = P.query(i)
        assert s1["status"] & NONFINITE == 0 and not d1 and s1["steps"] == 6
        for f in ("x", "v", "rho"):
            assert np.array_equal(P.get(i, f), R.get(j, f)), f


def test_absurd_velocity_is_flagged_and_isolated(gpu_lib):
    """A particle at 1e15 m/s: its neighbours' predicted densities reach
    ~1e10 rest densities in the first density solve, beyond what the scene's
    fixed-point error sum holds (DIVERGED; a later NaN retires the scene);
    the other scenes are unaffected, bit for bit.  (At 1e12 m/s the density
    solve absorbs the particle's compression and nothing is flagged, as in
    the reference.)"""
    x, b, p = mk(5)
    v = np.zeros_like(x)
    v[40] = (1e15, 0.0, 0.0)
    scenes = [(x, v, b, p)] + with_v(CLEAN)
    P, ids = run_pool(scenes, 5)
    st, _ = P.query(ids[0])
    assert st["status"] & (DIVERGED | NONFINITE)
    R, rids = run_pool(with_v(CLEAN), 5)
    for i, j in zip(ids[1:], rids):
        assert P.query(i)[0]["status"] & (DIVERGED | NONFINITE) == 0
        for f in ("x", "v"):
            assert np.array_equal(P.get(i, f), R.get(j, f)), f


def test_one_scene_context_flags_nan(gpu_lib):
    x, b, p = mk(6)
    x = x.copy()
    x[3, 0] = np.nan
    for precision in ("f32", "f64"):
        s = sph_gb300.Scene(**dict(p, precision=precision))
        s.set_fluid(x)
        s.add_boundary_points(b)
        s.init()
        s.step(2)
        assert s.stats()["status"] & NONFINITE, precision


def test_iteration_cap_is_flagged_and_matches_reference(gpu_lib):
    """max_it = 1 with tolerances no single iteration meets: every step's
    density and divergence solves stop at one iteration, above tolerance
    (the reference's loops, DFSPHSolver.cpp:327,512, both bounded by
    maxIterations), in the pool and the one-scene solver alike; fields still
    match the oracle run with the same limits within the FP32 bounds."""
    x, b, p = CLEAN[0]
    p = dict(p, eta=1e-9, eta_v=1e-9, max_it=1, min_it=1, min_it_v=1)
    q = {k: v for k, v in p.items() if k != "precision"}
    o = oracle.OracleScene(q, x, points=b)
    P = sph_gb300.Pool(max_particles=50_000, max_boundary=100_000, max_keys=1_000_000, max_scenes=4)
    sid = P.add_scene(x, boundary_points=b, steps=10, **p)
    s = sph_gb300.Scene(neighbor_list_max=64, **p)
    s.set_fluid(x)
    s.add_boundary_points(b)
    s.init()
    for step in range(3):
        o.step(1)
        P.step(1)
        s.step(1)
        assert o.scalar("iterations") == 1 and o.scalar("iterationsV") == 1
        for st in (P.query(sid)[0], s.stats()):
            assert st["iterations"] == 1 and st["iterations_v"] == 1
            assert st["status"] & ITER_CAP and st["status"] & ITER_CAP_V
        assert relerr(P.get(sid, "x"), o.get("x")) <= 1e-6
        assert relerr(P.get(sid, "rho"), o.get("rho")) <= 1e-5
        assert relerr(s.get("x"), o.get("x")) <= 1e-6


def test_status_clean_on_a_normal_mix(gpu_lib):
    P, ids = run_pool(with_v(CLEAN), 6)
    for i in ids:
        assert P.query(i)[0]["status"] & (NONFINITE | DIVERGED | ITER_CAP | ITER_CAP_V) == 0
