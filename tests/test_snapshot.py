"""Checkpoint / resume of pooled scenes (sph_pool_snapshot / sph_pool_restore).

The reference cannot resume a run: its frame files hold positions and
velocities only (SceneLoader::writeFluid, SceneLoader.cpp:200-264), without
the time step, the DFSPH warm-start k / kv and the iteration history that the
next steps depend on (DFSPHSolver.cpp:592-690, 827-870).  A snapshot holds the
scene's whole device state, its grid box and its solver scalars: a scene
restored into another pool, beside other scenes, continues bit for bit as the
uninterrupted run."""
import numpy as np
import pytest

import sph_gb300
from scenes import jitter, lattice

pytestmark = pytest.mark.gpu


def mk(seed, n_side=8, r=0.02, box=0.5, v=None):
    lo = 2 * r + 0.01 * (seed % 3)
    x = jitter(lattice(r, (lo, lo, lo), (lo + 2 * r * n_side, lo + 2 * r * n_side * 0.8, lo + 2 * r * n_side)), r, seed)
    b = sph_gb300.sample_box(4 * r, (0, 0, 0), (box, box, box))
    vel = np.zeros_like(x)
    if v is not None:
        vel[:, 1] = v
    return x, vel, b, dict(method=2, boundary=2, radius=r, eta=0.001, eta_v=0.001, dt=2e-3, precision="f32",
                          visc_method=2, visc=0.01)


A = mk(1, 9, v=-1.0)
OTHERS = [mk(2, 6), mk(3, 7, box=0.6)]


def new_pool(graph=True):
    P = sph_gb300.Pool(max_particles=100_000, max_boundary=200_000, max_keys=2_000_000, max_scenes=16)
    P.set_graph(graph)
    return P


def stats(P, sid):
    st, done = P.query(sid)
    return st, done


@pytest.mark.parametrize("graph", [True, False], ids=["graph", "host"])
def test_restored_scene_continues_bit_for_bit(gpu_lib, graph):
    x, v, b, p = A
    P1 = new_pool(graph)
    a1 = P1.add_scene(x, v, boundary_points=b, steps=20, **p)
    for s in OTHERS:
        P1.add_scene(s[0], s[1], boundary_points=s[2], steps=20, **s[3])
    P1.step(7)
    snap = P1.snapshot(a1)
    P1.step(9)
    # another pool, other neighbours, the scene restored with the steps it had left
    P2 = new_pool(graph)
    P2.add_scene(OTHERS[1][0], boundary_points=OTHERS[1][2], steps=50, **OTHERS[1][3])
    P2.step(3)
    a2 = P2.restore(snap)
    P2.step(9)
    for f in ("x", "v", "rho", "alpha", "k", "kv"):
        assert np.array_equal(P1.get(a1, f), P2.get(a2, f)), f
    s1, d1 = stats(P1, a1)
    s2, d2 = stats(P2, a2)
    for key in ("time", "dt", "steps", "sum_iterations", "sum_iterations_v", "iterations", "status"):
        assert s1[key] == s2[key], key
    assert s1["steps"] == 16
    # the steps it had left: 20 - 7; P2 ran 9 of its 13
    P1.step(4)
    P2.step(4)
    assert stats(P1, a1)[1] and stats(P2, a2)[1] and stats(P2, a2)[0]["steps"] == 20


def test_two_restores_of_one_snapshot_are_identical_and_steps_can_be_set(gpu_lib):
    x, v, b, p = A
    P = new_pool()
    a = P.add_scene(x, v, boundary_points=b, steps=5, **p)
    P.step(5)
    assert P.query(a)[1]
    snap = P.snapshot(a)
    Q = new_pool()
    r1 = Q.restore(snap, steps=6)
    r2 = Q.restore(snap, steps=6)
    Q.step(6)
    assert np.array_equal(Q.get(r1, "x"), Q.get(r2, "x"))
    assert Q.query(r1)[0]["steps"] == 11 and Q.query(r1)[1]
    # the restored scene's own continuation equals the original pool's
    P.remove(a)
    a3 = P.restore(snap, steps=6)
    P.step(6)
    assert np.array_equal(P.get(a3, "v"), Q.get(r1, "v"))


def test_restore_rejects_what_is_not_a_snapshot(gpu_lib):
    x, v, b, p = A
    P = new_pool()
    a = P.add_scene(x, v, boundary_points=b, steps=5, **p)
    P.step(1)
    snap = P.snapshot(a)
    with pytest.raises(sph_gb300.SPHError):
        P.restore(b"not a snapshot" + bytes(200))
    with pytest.raises(sph_gb300.SPHError):
        P.restore(snap[:-8])
    bad = bytearray(snap)
    bad[8] ^= 0xFF  # version
    with pytest.raises(sph_gb300.SPHError):
        P.restore(bytes(bad))
