"""Batched pool: scenes resident together on one GPU.

* a scene's results are the same alone and in a mix of other scenes, and when
  other scenes are admitted or removed while it runs (bit-exact: per-scene
  reductions use fixed-point integer sums, so nothing depends on the mix);
* a pooled scene matches the one-scene solver (same FP32 pair-list
  arithmetic) within the FP32 tolerance of the parity tests;
* graph-captured pool steps equal host-driven ones; step counts complete;
  admission respects capacity.
"""
import numpy as np
import pytest

import sph_gb300
from scenes import jitter, lattice
from util import relerr

pytestmark = pytest.mark.gpu


def mk(seed, n_side=8, r=0.02, box=0.5, spheres=()):
    lo = 2 * r + 0.01 * (seed % 3)
    x = jitter(lattice(r, (lo, lo, lo), (lo + 2 * r * n_side, lo + 2 * r * n_side * 0.8, lo + 2 * r * n_side)), r, seed)
    b = [sph_gb300.sample_box(4 * r, (0, 0, 0), (box, box, box))]
    for c, rad in spheres:
        b.append(sph_gb300.sample_sphere(r, c, rad))
    params = dict(method=2, boundary=2, radius=r, eta=0.001, eta_v=0.001, precision="f32")
    return x, np.concatenate(b), params


A = mk(1, 9, spheres=[((0.3, 0.4, 0.3), 0.06)])
OTHERS = [mk(2, 6), mk(3, 11, box=0.6), mk(4, 5, r=0.025, box=0.4)]


def pool_run(scenes, steps, graph=False, admit_later=(), later_at=0):
    P = sph_gb300.Pool(max_particles=200_000, max_boundary=400_000, max_keys=4_000_000, max_scenes=64)
    if graph:
        P.set_graph(True)
    ids = [P.add_scene(x, boundary_points=b, steps=1000, **p) for x, b, p in scenes]
    if admit_later:
        P.step(later_at)
        ids += [P.add_scene(x, boundary_points=b, steps=1000, **p) for x, b, p in admit_later]
        P.step(steps - later_at)
    else:
        P.step(steps)
    P.synchronize()
    return P, ids


def test_scene_alone_equals_scene_in_mix(gpu_lib):
    P1, (a1,) = pool_run([A], 8)
    P2, ids = pool_run([OTHERS[0], A, OTHERS[1], OTHERS[2]], 8)
    a2 = ids[1]
    for f in ("x", "v", "rho", "alpha"):
        assert np.array_equal(P1.get(a1, f), P2.get(a2, f)), f
    s1, _ = P1.query(a1)
    s2, _ = P2.query(a2)
    assert s1["sum_iterations"] == s2["sum_iterations"] and s1["dt"] == s2["dt"] and s1["time"] == s2["time"]


def test_admission_and_removal_mid_run_do_not_change_a_scene(gpu_lib):
    P1, (a1,) = pool_run([A], 8)
    P2, ids = pool_run([A, OTHERS[0]], 8, admit_later=[OTHERS[1], OTHERS[2]], later_at=3)
    a2 = ids[0]
    assert np.array_equal(P1.get(a1, "x"), P2.get(a2, "x"))
    # remove a neighbour and keep going
    P2.remove(ids[1])
    P1.step(4)
    P2.step(4)
    assert np.array_equal(P1.get(a1, "x"), P2.get(a2, "x"))
    assert np.array_equal(P1.get(a1, "v"), P2.get(a2, "v"))


def test_pooled_scene_matches_one_scene_solver(gpu_lib):
    x, b, p = A
    P, (a,) = pool_run([A], 6)
    s = sph_gb300.Scene(neighbor_list_max=64, **p)
    s.set_fluid(x)
    s.add_boundary_points(b)
    s.init()
    s.step(6)
    assert relerr(P.get(a, "x"), s.get("x")) <= 1e-6
    assert relerr(P.get(a, "rho"), s.get("rho")) <= 1e-5
    assert np.abs(P.get(a, "v") - s.get("v")).max() <= 2.5e-3
    assert P.query(a)[0]["sum_iterations"] == s.stats()["sum_iterations"]


FORCES = dict(visc_method=2, visc=0.01, bvisc=0.01, st_method=3, st=0.5, adh_method=4, adh=0.1)


def test_pooled_scene_with_surface_tension_and_adhesion(gpu_lib):
    """XSPH, Akinci surface tension and adhesion in a pooled scene, beside
    scenes without forces: within FP32 rounding of the one-scene solver (whose
    walks split a small scene's candidates over lanes; the pool's take one
    lane), equal iteration counts; the other scenes equal their runs without
    it, bit for bit."""
    x, b, p = A
    p = dict(p, **FORCES)
    P, ids = pool_run([(x, b, p)] + OTHERS, 6)
    s = sph_gb300.Scene(neighbor_list_max=64, **p)
    s.set_fluid(x)
    s.add_boundary_points(b)
    s.init()
    s.step(6)
    assert relerr(P.get(ids[0], "x"), s.get("x")) <= 1e-6
    assert relerr(P.get(ids[0], "rho"), s.get("rho")) <= 1e-5
    assert np.abs(P.get(ids[0], "v") - s.get("v")).max() <= 2.5e-3
    assert P.query(ids[0])[0]["sum_iterations"] == s.stats()["sum_iterations"]
    P0, ids0 = pool_run(OTHERS, 6)
    for i, j in zip(ids[1:], ids0):
        assert np.array_equal(P.get(i, "x"), P0.get(j, "x"))
        assert np.array_equal(P.get(i, "v"), P0.get(j, "v"))


def test_build_work_counts(gpu_lib):
    """sph_pool_count_work: every pair within h is a candidate, and the listed
    pairs (non-zero gradient, self excluded) are among the pairs within h."""
    P, ids = pool_run([A] + OTHERS, 3)
    w = P.count_work()
    pairs, overflow = P.list_pairs()
    n = sum(P.query(i)[0]["num_fluid"] for i in ids)
    assert overflow == 0
    assert w["fluid_candidates"] >= w["fluid_pairs"] >= pairs + n   # + each particle itself
    assert w["boundary_candidates"] >= w["boundary_pairs"] > 0
    assert 60 <= w["fluid_candidates"] / n <= 216


def test_pool_list_overflow_falls_back_to_cell_walks(gpu_lib):
    """With 8 list slots every pooled particle overflows its list: the build's
    first divergence error and every solver pass take the cell walks; results
    agree with full lists within FP32 rounding, iteration counts equal."""
    def run(kmax):
        P = sph_gb300.Pool(max_particles=200_000, max_boundary=400_000, max_keys=4_000_000, max_scenes=64,
                           neighbor_list_max=kmax)
        ids = [P.add_scene(x, boundary_points=b, steps=1000, **p) for x, b, p in [A] + OTHERS]
        P.step(4)
        P.synchronize()
        return P, ids

    P64, i64 = run(64)
    P8, i8 = run(8)
    assert P8.list_pairs()[1] > 0
    for a, b in zip(i64, i8):
        assert relerr(P8.get(b, "x"), P64.get(a, "x")) <= 1e-6
        assert relerr(P8.get(b, "rho"), P64.get(a, "rho")) <= 1e-5
        assert np.abs(P8.get(b, "v") - P64.get(a, "v")).max() <= 2.5e-3
        assert P8.query(b)[0]["sum_iterations"] == P64.query(a)[0]["sum_iterations"]


def test_graph_pool_equals_host_pool(gpu_lib):
    P1, ids1 = pool_run([A] + OTHERS, 6, graph=False)
    P2, ids2 = pool_run([A] + OTHERS, 6, graph=True)
    for i1, i2 in zip(ids1, ids2):
        assert np.array_equal(P1.get(i1, "x"), P2.get(i2, "x"))
    assert P2.launch_count() > 0


def test_step_counts_complete_and_poll(gpu_lib):
    P = sph_gb300.Pool(max_particles=100_000, max_boundary=200_000, max_keys=2_000_000, max_scenes=8)
    x, b, p = A
    short = P.add_scene(x, boundary_points=b, steps=3, **p)
    long = P.add_scene(OTHERS[0][0], boundary_points=OTHERS[0][1], steps=6, **OTHERS[0][2])
    P.step(4)
    assert P.poll() == [short]
    st, done = P.query(short)
    assert done and st["steps"] == 3
    P.remove(short)
    P.step(3)
    st, done = P.query(long)
    assert done and st["steps"] == 6
    assert P.poll() == [long]


def test_admission_respects_capacity(gpu_lib):
    x, b, p = A
    P = sph_gb300.Pool(max_particles=x.shape[0] + 10, max_boundary=400_000, max_keys=4_000_000, max_scenes=8)
    P.add_scene(x, boundary_points=b, steps=5, **p)
    with pytest.raises(sph_gb300.PoolFull):
        P.add_scene(x, boundary_points=b, steps=5, **p)
    assert P.usage()["particles"] == x.shape[0]


def test_timed_profiled_steps_and_list_stats(gpu_lib):
    """step_timed advances like step; the per-kernel profile covers the
    pool's kernels; list occupancy is reported; results are unchanged by
    profiling."""
    scenes = [A] + OTHERS
    P1, ids1 = pool_run(scenes, 3, graph=True)
    ms = P1.step_timed(4)
    assert ms > 0
    P2, ids2 = pool_run(scenes, 3)
    P2.set_profiling(True)
    P2.step(4)
    prof = P2.profile()
    assert {"k_pool_build_lists", "k_pool_correct", "k_pool_errors_density", "k_pool_errors_div"} <= set(prof)
    assert all(c > 0 and t >= 0 for c, t in prof.values())
    for s1, s2 in zip(ids1, ids2):
        assert np.array_equal(P1.get(s1, "x"), P2.get(s2, "x"))
        assert P1.query(s1)[0]["steps"] == 7
    pairs, overflow = P1.list_pairs()
    n = sum(x.shape[0] for x, _, _ in scenes)
    assert 10 * n < pairs < 64 * n and overflow == 0
    out = np.empty((A[0].shape[0], 3))
    assert P1.get(ids1[0], "v", out=out) is out


def test_autotuned_shapes_do_not_change_results(gpu_lib, tmp_path, monkeypatch):
    """The tuner's measurement steps are ordinary steps; any launch shape it
    may pick gives bit-identical results."""
    monkeypatch.setenv("SPH_GB300_TUNE_FILE", str(tmp_path / "tune.txt"))
    scenes = [A] + OTHERS

    def run(tuning=None, mode=0, steps=28):
        P = sph_gb300.Pool(max_particles=200_000, max_boundary=400_000, max_keys=4_000_000, max_scenes=64)
        P.set_autotune(mode)
        if tuning:
            P.set_tuning(**tuning)
        ids = [P.add_scene(x, boundary_points=b, steps=1000, **p) for x, b, p in scenes]
        P.set_graph(True)
        P.step(steps)
        P.synchronize()
        return P, ids

    ref, rids = run()
    variants = [dict(build_block=128, build_occupancy=896, queue_depth=16, solver_block=128, solver_occupancy=2048,
                     scan_width=4),
                dict(build_block=256, build_occupancy=1024, queue_depth=64, solver_block=256, solver_occupancy=1536,
                     scan_width=8)]
    for t in variants:
        P, ids = run(tuning=t)
        assert P.tuning()["build_block"] == t["build_block"]
        for a, b in zip(rids, ids):
            for f in ("x", "v", "rho"):
                assert np.array_equal(ref.get(a, f), P.get(b, f)), (t, f)
    P, ids = run(mode=2)
    tu = P.tuning()
    assert tu["source"] == 2 and tu["steps_left"] == 0
    assert "build block" in P.tuning_log() and "solver block" in P.tuning_log()
    for a, b in zip(rids, ids):
        assert np.array_equal(ref.get(a, "x"), P.get(b, "x"))
    # a second pool of the same size takes the cached shapes without measuring
    Q, _ = run(mode=1, steps=1)
    q = Q.tuning()
    assert q["source"] == 1 and q["steps_left"] == 0
    keys = ("build_block", "build_occupancy", "queue_depth", "solver_block", "solver_occupancy", "scan_width")
    assert all(q[k] == tu[k] for k in keys)
    with pytest.raises(sph_gb300.SPHError):
        Q.set_tuning(build_block=96)
    with pytest.raises(sph_gb300.SPHError):
        Q.set_tuning(solver_occupancy=1000)


def test_submitter_thread_and_stepping_thread_share_a_pool(gpu_lib):
    """One host thread admits scenes while another steps and polls the same
    pool (calls are serialised by the pool).  Every admitted scene runs its
    steps, and scene A's results equal A run alone."""
    import threading
    import time

    P = sph_gb300.Pool(max_particles=200_000, max_boundary=400_000, max_keys=4_000_000, max_scenes=64)
    P.set_graph(True)
    a = P.add_scene(A[0], boundary_points=A[1], steps=30, **A[2])
    ids, errors = [], []

    def submit():
        try:
            for k in range(6):
                x, b, p = OTHERS[k % len(OTHERS)]
                ids.append(P.add_scene(x, boundary_points=b, steps=12, **p))
                time.sleep(0.005)
        except Exception as e:  # reported below
            errors.append(e)

    t = threading.Thread(target=submit)
    t.start()
    done = set()
    # step until the submitter has finished and every scene it admitted has
    # run its steps (a scene admitted late still needs its 12 steps)
    for _ in range(5000):
        P.step(1)
        done.update(P.poll())
        if not t.is_alive() and set(ids) | {a} <= done:
            break
    t.join()
    assert not errors, errors
    P.synchronize()
    done.update(P.poll())
    assert set(ids) | {a} <= done
    R, rid = pool_run([A], 30)
    assert np.array_equal(P.get(a, "x"), R.get(rid[0], "x"))
    assert np.array_equal(P.get(a, "v"), R.get(rid[0], "v"))
