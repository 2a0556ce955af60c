"""A fixed GPU workload for the bounds-checked build comparison
(tests/test_bounds_check.py): a pool of six scenes of the benchmark mix (pair
lists, graph steps), a one-scene DFSPH dam break at r = 0.02 (pair lists) and
a one-scene PCISPH drop at r = 0.01 (candidate lists).  Prints one JSON line:
a SHA-256 of every result field and each run's status word.  The library is
the one SPH_GB300_LIBRARY names (the ordinary one when unset)."""
import hashlib
import json
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import sph_gb300  # noqa: E402
from scenes import jitter  # noqa: E402
from sph_gb300 import workloads  # noqa: E402


def main():
    h = hashlib.sha256()
    status = {}
    P = sph_gb300.Pool(max_particles=400_000, max_boundary=600_000, max_keys=8_000_000, max_scenes=8)
    P.set_graph(True)
    ids = [P.add_scene(x, boundary_points=b, steps=100, **p) for x, b, p, _ in workloads.batched_mix(n_scenes=6, seed=3)]
    P.step(10)
    for i in ids:
        for f in ("x", "v", "rho", "alpha"):
            h.update(np.ascontiguousarray(P.get(i, f)).tobytes())
        status[f"pool{i}"] = P.query(i)[0]["status"]
    x, b, p, _ = workloads.dam_break(r=0.02, n_side=15, box=(1.2, 0.8, 0.8))
    s = sph_gb300.Scene(**p)
    s.set_fluid(jitter(x, 0.02, 1))
    s.add_boundary_points(b)
    s.init()
    s.step(10)
    for f in ("x", "v", "rho"):
        h.update(np.ascontiguousarray(s.get(f)).tobytes())
    status["dam"] = s.stats()["status"]
    x, b, p, _ = workloads.pcisph_drop(0.01)
    s = sph_gb300.Scene(threads_per_particle=1, **dict(p, precision="f32"))
    s.set_fluid(jitter(x, 0.01, 2))
    s.add_boundary_points(b)
    s.init()
    s.step(10)
    for f in ("x", "v", "rho"):
        h.update(np.ascontiguousarray(s.get(f)).tobytes())
    status["drop"] = s.stats()["status"]
    print(json.dumps({"hash": h.hexdigest(), "status": status}))


if __name__ == "__main__":
    main()
