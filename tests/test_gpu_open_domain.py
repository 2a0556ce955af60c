"""Particles outside the grid box.

The reference hashes cells without bounds (HashTable.h:79-102), so a particle
anywhere has its neighbours found.  The dense grid here covers the scene's box
plus a two-cell margin and keeps a particle that leaves it in the nearest
border cell, with its true offset from that cell's corner, and sets the sticky
status bit SPH_STATUS_OUT_OF_GRID.  Neighbours are still found: clamping moves
two particles within h of each other into the same or adjacent cells, every
candidate is tested on its true distance, and the walks trim a neighbour
column only by its true distance from the particle.  The FP32 build culls
such a particle in FP32 (the half-precision cull needs in-cell offsets).

Each case starts a jittered block that sticks out of a deliberately small
grid box on every side and moves down through its floor, with no boundary,
and compares with the oracle (whose hash grid has no bounds), first with the
box held fixed (sph_ctx_set_grid_growth(0)), then with the box growing.  FP64: within
1e-5 relative with equal iteration counts.  FP32: leaving the grid box costs
no accuracy, so the errors against the oracle stay within 1.5x those of the
same FP32 run in a grid box that holds every particle (measured on GB300,
max over the steps, small / full box: DFSPH positions 1.34e-5 / 1.33e-5,
densities 2.75e-4 / 2.74e-4, velocities 1.8e-4 / 2.4e-4 of the largest
speed; WCSPH 1.2e-7 / 1.1e-7, 2.1e-6 / 2.2e-6, 6e-6 / 9e-6).  The DFSPH
errors are larger than in the parity scenes because the steps are 40x
longer (dt 4 ms): the FP32 rounding of the velocity corrections, sums of
nearly cancelling terms, grows into positions and densities with dt.
"""
import numpy as np
import pytest

import oracle
import sph_gb300
from scenes import jitter, lattice
from util import relerr

pytestmark = pytest.mark.gpu

# The grid box is the domain plus two cells of h = 0.08 m on each side:
# x, z in [0.16, 0.64] m and y in [0.08, 0.48] m, while the block spans
# [0.02, 0.78] x [0.02, 0.38] x [0.02, 0.78] m and moves down at 2 m/s.
DOMAIN = dict(domain_min=(0.35, 0.25, 0.35), domain_max=(0.45, 0.3, 0.45))
CASES = {
    "dfsph_open": (dict(method=2, boundary=0, radius=0.02, eta=0.001, eta_v=0.001, dt=4e-3, max_dt=5e-3), 8),
    "wcsph_open": (dict(method=0, boundary=0, radius=0.02, stiffness=1000.0, gamma=7.0, visc_method=2, visc=0.01,
                        dt=1e-3), 20),
}
OUT_OF_GRID = 1


def _state():
    x = jitter(lattice(0.02, (0.0, 0.0, 0.0), (0.8, 0.4, 0.8)), 0.02, 3)
    v = np.zeros_like(x)
    v[:, 1] = -2.0
    return x, v


def _scene(params, precision, x, v, domain, grow=False):
    s = sph_gb300.Scene(precision=precision, **params, **domain)
    s.set_fluid(x, v)
    s.set_grid_growth(grow)
    s.init()
    return s


def _errors(s, o):
    vo = o.get("v")
    return np.array([relerr(s.get("x"), o.get("x")), relerr(s.get("rho"), o.get("rho")),
                     np.abs(s.get("v") - vo).max() / np.abs(vo).max()])


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("name", list(CASES))
def test_particles_outside_the_grid_box_match_oracle(gpu_lib, name, precision):
    params, steps = CASES[name]
    x, v = _state()
    o = oracle.OracleScene(params, x, v=v)
    s = _scene(params, precision, x, v, DOMAIN)
    full = _scene(params, precision, x, v, {}) if precision == "f32" else None
    assert s.stats()["status"] & OUT_OF_GRID
    err = np.zeros(3)
    err_full = np.zeros(3)
    for step in range(steps):
        o.step(1)
        s.step(1)
        if precision == "f64":
            for f in ("x", "v", "rho", "p"):
                e = relerr(s.get(f), o.get(f))
                assert e <= 1e-5, (name, step, f, e)
        else:
            full.step(1)
            err = np.maximum(err, _errors(s, o))
            err_full = np.maximum(err_full, _errors(full, o))
        if params["method"] != 0:
            assert s.stats()["iterations"] == int(o.scalar("iterations")), (name, step)
    if precision == "f32":
        assert full.stats()["status"] == 0
        assert np.all(err <= 1.5 * err_full + np.array([1e-7, 1e-6, 1e-5])), (name, err, err_full)
    # its lowest layer is now more than h below the grid box's floor (0.08 m)
    assert s.get("x")[:, 1].min() < -0.01
    assert s.stats()["status"] & ~OUT_OF_GRID == 0
    assert s.stats()["grid_growths"] == 0


# A box that holds every particle of the growth test for all its steps, and
# the steps each case needs to fall through the floor of its own starting box
# (the domain widened to hold the block, plus two cells: y >= -0.16 m).
BIG = dict(domain_min=(-0.5, -1.0, -0.5), domain_max=(1.3, 0.6, 1.3))
GROW_STEPS = {"dfsph_open": 48, "wcsph_open": 120}


@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("name", list(CASES))
def test_grid_box_grows_without_changing_results(gpu_lib, name, precision):
    """The same open blocks with grid growth on (the default).  The box
    starts around every point and grows after a periodic check (every 16
    steps) sees a particle kept in a border cell.  FP64: every step equals
    the run in a fixed box that holds all particles throughout (same cell
    lattice, same walk order, absolute positions; only the particles' sorted
    order differs) to 1e-9, and the oracle to 1e-5, with equal iteration
    counts.  FP32: a particle kept in a border cell until the check computes
    its pairs in another cell frame, so the two runs part at rounding level;
    its errors against the oracle stay within 1.5x those of the fixed big box."""
    params, _ = CASES[name]
    x, v = _state()
    o = oracle.OracleScene(params, x, v=v)
    s = _scene(params, precision, x, v, DOMAIN, grow=True)
    ref = _scene(params, precision, x, v, BIG)
    assert s.stats()["status"] == 0 and ref.stats()["status"] == 0
    err = np.zeros(3)
    err_ref = np.zeros(3)
    for step in range(GROW_STEPS[name]):
        s.step(1)
        ref.step(1)
        o.step(1)
        if precision == "f64":
            for f in ("x", "v", "rho"):
                e = relerr(s.get(f), ref.get(f))
                assert e <= 1e-9, (name, step, f, e)
                e = relerr(s.get(f), o.get(f))
                assert e <= 1e-5, (name, step, f, e)
            if params["method"] != 0:
                assert s.stats()["iterations"] == int(o.scalar("iterations")), (name, step)
        else:
            err = np.maximum(err, _errors(s, o))
            err_ref = np.maximum(err_ref, _errors(ref, o))
    st = s.stats()
    assert st["grid_growths"] >= 1 and st["status"] == OUT_OF_GRID, st
    assert ref.stats()["status"] == 0 and ref.stats()["grid_growths"] == 0
    if precision == "f32":
        assert np.all(err <= 1.5 * err_ref + np.array([1e-7, 1e-6, 1e-5])), (name, err, err_ref)
