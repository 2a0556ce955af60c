"""Live pin of the C restatement against the reference's own sources, built
headless (oracle/_ref).  Runs only where the reference tree is available;
elsewhere the golden fixtures carry the pin."""
import numpy as np
import pytest

import oracle
from scenes import jitter, lattice

pytestmark = pytest.mark.skipif(not oracle.reference_available(), reason="reference build not present")

CASES = [
    ("dfsph_cube_jitter", dict(method=2, boundary=0, radius=0.02, has_cube=1, cube_min=(0, 0, 0), cube_max=(0.4, 0.5, 0.4)),
     lambda: jitter(lattice(0.02, (0, 0, 0), (0.3, 0.3, 0.3)), 0.02, 7), [], []),
    ("pcisph_akinci_xsph", dict(method=1, boundary=2, radius=0.02, visc_method=2, visc=0.02, bvisc=0.01, eta=0.002,
                                min_it=2, max_it=20),
     lambda: lattice(0.02, (0.05, 0.05, 0.05), (0.3, 0.4, 0.3)), [((0, 0, 0), (0.5, 0.6, 0.5))], [((0.25, 0.5, 0.25), 0.06)]),
    ("wcsph_art", dict(method=0, boundary=2, radius=0.02, visc_method=1, visc=0.05, bvisc=0.02, stiffness=500, gamma=7),
     lambda: jitter(lattice(0.02, (0.02, 0.02, 0.02), (0.3, 0.3, 0.3)), 0.02, 3), [((0, 0, 0), (0.4, 0.4, 0.4))], []),
]


@pytest.mark.parametrize("name,params,fluid,boxes,spheres", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_live_reference(name, params, fluid, boxes, spheres):
    x = fluid()
    ref = oracle.run_reference(params, x, boxes=boxes, spheres=spheres, steps=4)
    o = oracle.OracleScene(params, x, boxes=boxes, spheres=spheres)
    for s in range(1, 5):
        o.step(1)
        for f in ("x", "v", "rho", "p"):
            assert np.array_equal(o.get(f).ravel(), ref[f"s{s}.{f}"]), (name, s, f)


# Open domains: no boundary, a jittered block moving down at 2 m/s; the
# reference's hash grid has no bounds, so every particle keeps its neighbours
# wherever it goes (the GPU tests of particles leaving the grid box compare
# with the restatement on these scenes).
OPEN = [
    ("dfsph_open", dict(method=2, boundary=0, radius=0.02, eta=0.001, eta_v=0.001, dt=4e-3, max_dt=5e-3)),
    ("wcsph_open", dict(method=0, boundary=0, radius=0.02, stiffness=1000.0, gamma=7.0, visc_method=2, visc=0.01,
                        dt=1e-3)),
]


@pytest.mark.parametrize("name,params", OPEN, ids=[c[0] for c in OPEN])
def test_oracle_matches_live_reference_in_an_open_domain(name, params):
    x = jitter(lattice(0.02, (0.0, 0.0, 0.0), (0.4, 0.2, 0.4)), 0.02, 3)
    v = np.zeros_like(x)
    v[:, 1] = -2.0
    ref = oracle.run_reference(params, x, v=v, steps=4)
    o = oracle.OracleScene(params, x, v=v)
    for s in range(1, 5):
        o.step(1)
        for f in ("x", "v", "rho", "p"):
            assert np.array_equal(o.get(f).ravel(), ref[f"s{s}.{f}"]), (name, s, f)


# The full-size configurations of the GPU tests: the restatement equals the
# reference bit for bit there too, and the workloads' boundary points equal
# the reference's own sampling of the box.
FULL = [
    ("pcisph_drop_81k", "pcisph_drop", ((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))),
    ("dam_break_125k", "dam_break", ((0.0, 0.0, 0.0), (1.5, 0.8, 0.8))),
]


@pytest.mark.parametrize("name,make,box", FULL, ids=[c[0] for c in FULL])
def test_oracle_matches_live_reference_at_full_size(name, make, box):
    from sph_gb300 import workloads

    x, b, params, _ = getattr(workloads, make)()
    p = {k: v for k, v in params.items() if k != "precision"}
    ref = oracle.run_reference(p, x, boxes=[box], steps=2)
    o = oracle.OracleScene(p, x, boxes=[box])
    o.step(2)
    for f in ("x", "v", "rho", "p"):
        assert np.array_equal(o.get(f).ravel(), ref[f"s2.{f}"]), (name, f)
    o2 = oracle.OracleScene(p, x, points=b)
    o2.step(2)
    assert np.array_equal(o2.get("x"), o.get("x"))
