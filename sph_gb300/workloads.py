"""Seeded synthetic scenes for the DFSPH workloads (no dataset is involved).

* ``dam_break``     one 125,000-particle dam break with Akinci walls;
* ``pcisph_drop``   PCISPH with standard viscosity, Akinci surface tension and
                    adhesion: a 5-layer pool on the floor of a 1 m Akinci box
                    and a sphere of fluid (R = 0.2 m) 0.6 m above it, r = 5 mm;
* ``batched_mix``   independent scenes: per-scene particle counts log-uniform
                    in [2k, 64k], fluid blocks with aspect ratios uniform in
                    [0.5, 2] at the box corner, 0-3 Akinci sphere obstacles of
                    radius 0.05-0.2 m placed at random in a 1 m Akinci box,
                    r = 0.01 m, 0.1 % density error;
* ``request_stream`` Poisson arrivals of scenes drawn like the mix but with
                    1k-200k particles (log-uniform, boxes grown beyond 1 m so
                    the fluid fills at most 40 % of the volume) and 200-2000
                    steps, plus a 4M-particle dam break at a fixed interval.

Fluid blocks start 2r off the walls: with its first layer at r from an Akinci
wall the reference's DFSPH ejects wall-adjacent particles in the first step.

The point sets come from the library's samplers (``sph_gb300.fluid_block``,
``sample_box``, ``sample_sphere``: the reference's lattice and Akinci
samplings).  A caller that must not load the library -- a CPU baseline that
times another implementation of the same scenes -- passes any object with the
same three functions as ``geometry``.
"""
from __future__ import annotations

import math
import types

import numpy as np

from . import fluid_block, sample_box, sample_sphere

LIBRARY_GEOMETRY = types.SimpleNamespace(fluid_block=fluid_block, sample_box=sample_box, sample_sphere=sample_sphere)

DFSPH = dict(method=2, boundary=2, eta=0.001, eta_v=0.001, cfl=1.0, max_it=100, dt=1e-4, min_dt=1e-5, max_dt=5e-3,
             fps=60.0, precision="f32")


def _block(r, corner, dims, geometry=None):
    g = geometry or LIBRARY_GEOMETRY
    d = 2.0 * r
    mn = np.asarray(corner, dtype=np.float64)
    mx = mn + np.asarray(dims, dtype=np.float64) * d + 1e-9
    return g.fluid_block(r, mn, mx), (mn, mx)


def make_scene(rng, n_target, r=0.01, box_side=1.0, steps=500, spheres=True, geometry=None):
    """One scene of the mix: (x, boundary points, params, steps)."""
    g = geometry or LIBRARY_GEOMETRY
    d = 2.0 * r
    a_xz = rng.uniform(0.5, 2.0)
    a_y = rng.uniform(0.5, 2.0)
    nmax = int((box_side - 4 * r) / d) - 1
    nx = max(2, int(round((n_target / (a_y * a_xz)) ** (1.0 / 3.0))))
    dims = [min(nx, nmax), min(max(2, int(round(nx * a_y))), nmax), min(max(2, int(round(nx * a_xz))), nmax)]
    x, (bmn, bmx) = _block(r, (2 * r, 2 * r, 2 * r), dims, g)
    pts = [g.sample_box(4 * r, (0.0, 0.0, 0.0), (box_side, box_side, box_side))]
    if spheres:
        for _ in range(int(rng.integers(0, 4))):
            for _try in range(50):
                rad = rng.uniform(0.05, 0.2) * box_side
                c = rng.uniform(rad + 2 * d, box_side - rad - 2 * d, 3)
                # keep clear of the block
                q = np.clip(c, bmn - 2 * d, bmx + 2 * d)
                if np.linalg.norm(c - q) > rad + 2 * d:
                    pts.append(g.sample_sphere(r, c, rad))
                    break
    params = dict(DFSPH, radius=r)
    return x, np.concatenate(pts), params, int(steps)


def batched_mix(n_scenes=256, seed=42, steps=500, r=0.01, geometry=None):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(2000), math.log(64000)))))
        out.append(make_scene(rng, n, r=r, steps=steps, geometry=geometry))
    return out


def dam_break(r=0.005, n_side=50, box=(1.5, 0.8, 0.8), steps=2000):
    x, _ = _block(r, (2 * r, 2 * r, 2 * r), (n_side, n_side, n_side))
    b = sample_box(4 * r, (0.0, 0.0, 0.0), box)
    return x, b, dict(DFSPH, radius=r), int(steps)


def pcisph_drop(r=0.005, steps=1000):
    """A 0.05 m-deep pool (round(0.05 / 2r) layers, 2r off the walls) and a
    lattice sphere of R = 0.2 m centred 0.6 m above the pool top in a 1 m
    Akinci box; PCISPH, standard viscosity 0.01, Akinci surface tension 0.5
    and adhesion 0.1, eta 0.001, 3-100 iterations, dt = 1e-4 s.  At r = 5 mm:
    5 layers, 48,020 + 33,401 = 81,421 particles; at r = 2.75 mm: 9 layers,
    291,600 + 198,171 = 489,771 particles (the 500k drop)."""
    d = 2 * r
    n = int((1.0 - 4 * r) / d)
    layers = max(1, int(round(0.05 / d)))
    pool, (pmn, pmx) = _block(r, (2 * r, 2 * r, 2 * r), (n, layers, n))
    c = np.array([0.5, pmx[1] + 0.6, 0.5])
    R = 0.2
    cube = fluid_block(r, c - R - r, c + R + r)
    ball = cube[np.sum((cube - c) ** 2, axis=1) <= R * R]
    x = np.concatenate([pool, ball])
    b = sample_box(4 * r, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    params = dict(method=1, boundary=2, radius=r, eta=0.001, min_it=3, max_it=100, dt=1e-4, visc_method=0,
                  visc=0.01, st_method=3, st=0.5, adh_method=4, adh=0.1)
    return x, b, params, int(steps)


def big_dam_break(r=0.004, steps=200):
    """4M-particle dam break: a 1.6 x 0.8 x 1.6 m block in a 3 x 1.5 x 1.5 m box
    (the 4M particles at r = 0.004 m need ~2 m^3 of fluid)."""
    d = 2 * r
    dims = (int(1.6 / d), int(0.8 / d), int(1.6 / d))
    x, _ = _block(r, (2 * r, 2 * r, 2 * r), dims)
    b = sample_box(4 * r, (0.0, 0.0, 0.0), (3.0, 1.5, 1.5))
    return x, b, dict(DFSPH, radius=r), int(steps)


def request_stream(rate=200.0, duration=10.0, seed=7, big_every=10.0, r=0.01, big_steps=200):
    """[(arrival_s, builder)] sorted by arrival; builder() -> scene tuple."""
    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        n = int(round(math.exp(rng.uniform(math.log(1000), math.log(200000)))))
        steps = int(rng.integers(200, 2001))
        side = 1.0 if n <= 50000 else (n * (2 * r) ** 3 / 0.4) ** (1.0 / 3.0)
        s = int(rng.integers(0, 2**31))
        reqs.append((t, lambda n=n, steps=steps, side=side, s=s: make_scene(np.random.default_rng(s), n, r=r,
                                                                          box_side=side, steps=steps)))
    if big_every and big_every > 0:
        tb = big_every
        while tb <= duration:
            reqs.append((tb, lambda: big_dam_break(steps=big_steps)))
            tb += big_every
    reqs.sort(key=lambda q: q[0])
    return reqs
