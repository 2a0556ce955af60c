"""Parity scenes shared by the oracle, the golden fixtures and the GPU tests.

Each scene is a dict of parameters (the oracle's names, which sph_gb300.Scene
also accepts), an initial fluid state built on the reference's lattice
(Simulation::buildFluidBlock: spacing 2r from min + r) with optional seeded
jitter, and the Akinci boundary shapes.  Sizes are small so the FP64 CPU
oracle finishes in seconds.
"""
from __future__ import annotations

import numpy as np


def lattice(r, mn, mx):
    """Simulation::buildFluidBlock (Simulation.cpp:512-539), vectorised."""
    dist = 2.0 * r
    n = [int(np.floor((mx[k] - mn[k]) / dist + 1e-5)) for k in range(3)]
    i, j, k = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]), indexing="ij")
    out = np.stack([i.ravel() * dist + (mn[0] + r), j.ravel() * dist + (mn[1] + r), k.ravel() * dist + (mn[2] + r)],
                   axis=1)
    return out.astype(np.float64)


def jitter(x, r, seed):
    rng = np.random.default_rng(seed)
    return x + rng.uniform(-0.01 * r, 0.01 * r, x.shape)


SCENES = {
    # DFSPH dam break with Akinci walls (the headline solver).  The block
    # starts 2r off the walls: with its first layer at r from an Akinci wall
    # the reference's DFSPH ejects wall particles at ~500 m/s in step 1.
    "dfsph_akinci": dict(
        params=dict(method=2, boundary=2, radius=0.02, eta=0.001, eta_v=0.001, cfl=1.0, dt=1e-4, min_dt=1e-5,
                    max_dt=5e-3, fps=60.0),
        fluid=lambda: lattice(0.02, (0.04, 0.04, 0.04), (0.44, 0.44, 0.44)),
        boxes=[((0.0, 0.0, 0.0), (0.8, 0.6, 0.6))],
        spheres=[],
    ),
    # DFSPH with a sphere obstacle and XSPH + surface tension + adhesion.
    # Jittered: the reference's cohesion kernel jumps by 2x at r = h/2
    # (Cohesion.h:36-37 leaves valueCoef2 unscaled), exactly the lattice
    # spacing, so an unjittered lattice makes last-bit rounding pick branches.
    "dfsph_forces": dict(
        params=dict(method=2, boundary=2, radius=0.02, visc_method=2, visc=0.01, bvisc=0.01, st_method=3, st=0.5,
                    adh_method=4, adh=0.1),
        fluid=lambda: jitter(lattice(0.02, (0.05, 0.05, 0.05), (0.35, 0.35, 0.35)), 0.02, 11),
        boxes=[((0.0, 0.0, 0.0), (0.6, 0.6, 0.6))],
        spheres=[((0.3, 0.5, 0.3), 0.08)],
    ),
    # DFSPH with artificial viscosity
    "dfsph_artvisc": dict(
        params=dict(method=2, boundary=2, radius=0.02, visc_method=1, visc=0.01, bvisc=0.01),
        fluid=lambda: lattice(0.02, (0.05, 0.05, 0.05), (0.35, 0.3, 0.35)),
        boxes=[((0.0, 0.0, 0.0), (0.5, 0.5, 0.5))],
        spheres=[],
    ),
    # WCSPH settling block in a cube boundary with XSPH (the CPU-runnable
    # configuration, scaled down): jitter +-0.01 r, seed 1234
    "wcsph_cube": dict(
        params=dict(method=0, boundary=0, radius=0.025, stiffness=1000.0, gamma=7.0, visc_method=2, visc=0.01,
                    has_cube=1, cube_min=(0.0, 0.0, 0.0), cube_max=(1.0, 1.0, 1.0)),
        fluid=lambda: jitter(lattice(0.025, (0.0, 0.0, 0.0), (0.5, 0.5, 0.5)), 0.025, 1234),
        boxes=[],
        spheres=[],
    ),
    # WCSPH with Akinci walls and boundary XSPH
    "wcsph_akinci": dict(
        params=dict(method=0, boundary=2, radius=0.02, visc_method=2, visc=0.01, bvisc=0.01),
        fluid=lambda: lattice(0.02, (0.1, 0.1, 0.1), (0.4, 0.35, 0.4)),
        boxes=[((0.0, 0.0, 0.0), (0.5, 0.5, 0.5))],
        spheres=[((0.25, 0.05, 0.25), 0.05)],
    ),
    # PCISPH drop with standard viscosity, surface tension, cohesion, adhesion.
    # The pool starts one lattice spacing off the walls: with its first layer
    # at r from an Akinci wall the reference's own PCISPH blows up in the
    # first step (Poly6-derived scaling factor, Spiky pressure gradient).
    "pcisph_drop": dict(
        params=dict(method=1, boundary=2, radius=0.02, eta=0.001, min_it=3, max_it=100, visc_method=0, visc=0.01,
                    bvisc=0.01, st_method=3, st=0.5, adh_method=4, adh=0.1),
        fluid=lambda: jitter(np.concatenate([
            lattice(0.02, (0.04, 0.04, 0.04), (0.56, 0.12, 0.56)),
            lattice(0.02, (0.2, 0.2, 0.2), (0.36, 0.36, 0.36)),
        ]), 0.02, 5),
        boxes=[((0.0, 0.0, 0.0), (0.6, 0.6, 0.6))],
        spheres=[],
    ),
    # DFSPH inside a cube boundary (clamp after the divergence solve)
    "dfsph_cube": dict(
        params=dict(method=2, boundary=0, radius=0.02, has_cube=1, cube_min=(0.0, 0.0, 0.0),
                    cube_max=(0.4, 0.4, 0.4)),
        fluid=lambda: lattice(0.02, (0.0, 0.0, 0.0), (0.3, 0.3, 0.3)),
        boxes=[],
        spheres=[],
    ),
}


def _bh_fluid():
    """A pool 1.5 r off the floor and walls of the box (inside the PCISPH
    model's collision radius h/2) plus a falling block, all moving towards
    the walls, so that every step has colliding particles."""
    return jitter(np.concatenate([lattice(0.02, (0.01, 0.01, 0.01), (0.3, 0.12, 0.3)),
                                  lattice(0.02, (0.2, 0.3, 0.2), (0.4, 0.4, 0.4))]), 0.02, 5)


def _bh_velocity(x):
    v = np.zeros_like(x)
    v[:, 0] = -0.2
    v[:, 1] = -0.5
    return v


# PCISPH boundary model (boundary 1): a container box (normals inwards) and a
# solid sphere obstacle (normals outwards), for each solver.
_BH = dict(bh_boxes=[((0.0, 0.0, 0.0), (0.6, 0.6, 0.6), 1)], bh_spheres=[((0.3, 0.2, 0.3), 0.05, 0)],
           velocity=_bh_velocity, fluid=_bh_fluid, boxes=[], spheres=[])
SCENES.update({
    "wcsph_bh": dict(params=dict(method=0, boundary=1, radius=0.02, bh_normal_fct=0.5, bh_tang_fct=0.9,
                                 visc_method=2, visc=0.01), **_BH),
    # three fixed pressure iterations: with the default cap the reference's own
    # solve diverges on this model (its boundary points, 0.45 h apart, have a
    # self-density of ~1.5 rho0, so their pressure grows every iteration; the
    # fluid reaches 7,750 m/s in one step) and amplifies last-bit differences
    # to 1e-6 in a step, which no other implementation could reproduce
    "pcisph_bh": dict(params=dict(method=1, boundary=1, radius=0.02, bh_normal_fct=0.5, bh_tang_fct=0.9, eta=0.001,
                                  min_it=3, max_it=3), **_BH),
    "dfsph_bh": dict(params=dict(method=2, boundary=1, radius=0.02, bh_normal_fct=0.5, bh_tang_fct=0.9, eta=0.001,
                                 eta_v=0.001), **_BH),
})


def scene(name):
    s = SCENES[name]
    return s["params"], s["fluid"](), s["boxes"], s["spheres"]


def scene_extra(name, x):
    """Initial velocities and PCISPH-model shapes of a scene: (v or None,
    [(min, max, inverted)], [(centre, radius, inverted)])."""
    s = SCENES[name]
    v = s["velocity"](x) if "velocity" in s else None
    return v, s.get("bh_boxes", []), s.get("bh_spheres", [])


# Emitters (Emitter.cpp, FluidModel::addEmitter): a tilted circular emitter
# firing from t = 0 and a square one firing downwards from t = 3 ms, each
# budgeted for a few groups (the circle's budget is not a whole number of
# groups, so its last partial group is never emitted), over a jittered pool.
# 30 steps, state kept every third step.  DFSPH and PCISPH with Akinci walls,
# WCSPH with the cube boundary, and a DFSPH scene whose fluid comes only from
# an emitter.
def _unit(q):
    q = np.asarray(q, dtype=np.float64)
    return tuple(float(t) for t in q / np.linalg.norm(q))


_EMIT_CIRCLE = dict(type=1, num=19 * 3 + 5, position=(0.4, 0.55, 0.4), velocity=2.0, rotation=_unit((0.9, 0.3, 0.2, 0.1)),
                    start=0.0, width=0.1, height=0.0, spacing=1.0)
_EMIT_SQUARE = dict(type=0, num=24 * 2, position=(0.25, 0.5, 0.3), velocity=1.5,
                    rotation=(0.7071067811865476, 0.7071067811865476, 0.0, 0.0), start=0.003, width=0.24, height=0.16,
                    spacing=1.2)
_BOX08 = [((0.0, 0.0, 0.0), (0.8, 0.8, 0.8))]


def _emit_pool():
    return jitter(lattice(0.02, (0.04, 0.04, 0.04), (0.3, 0.2, 0.3)), 0.02, 5)


EMIT_SCENES = {
    "dfsph_emit": dict(params=dict(method=2, boundary=2, radius=0.02, dt=2e-3, eta=0.001, eta_v=0.001),
                       fluid=_emit_pool, boxes=_BOX08, spheres=[], emitters=[_EMIT_CIRCLE, _EMIT_SQUARE]),
    "wcsph_emit": dict(params=dict(method=0, boundary=0, radius=0.02, dt=5e-4, stiffness=1000.0, gamma=7.0, has_cube=1,
                                   cube_min=(0.0, 0.0, 0.0), cube_max=(0.8, 0.8, 0.8)),
                       fluid=_emit_pool, boxes=[], spheres=[], emitters=[_EMIT_CIRCLE, _EMIT_SQUARE]),
    "pcisph_emit": dict(params=dict(method=1, boundary=2, radius=0.02, dt=1e-3, eta=0.01, min_it=3, max_it=20),
                        fluid=_emit_pool, boxes=_BOX08, spheres=[], emitters=[_EMIT_CIRCLE, _EMIT_SQUARE]),
    "dfsph_emit_only": dict(params=dict(method=2, boundary=2, radius=0.02, dt=2e-3),
                            fluid=lambda: np.zeros((0, 3)), boxes=_BOX08, spheres=[], emitters=[_EMIT_CIRCLE]),
}
EMIT_STEPS, EMIT_DUMP_EVERY = 30, 3


def emit_scene(name):
    """(params, x, boxes, spheres, emitters) of an emitter scene."""
    s = EMIT_SCENES[name]
    return s["params"], s["fluid"](), s["boxes"], s["spheres"], s["emitters"]
