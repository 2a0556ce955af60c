"""PCISPH / WCSPH candidate lists against the cell walks they replace.

With one lane per particle the PCISPH step records, in its density pass, the
fluid candidates of the 27 cells within h + 0.1 h at the current positions
(walk order, with each candidate's cell offset), and the normals, non-pressure
force, predicted-density and pressure-acceleration passes visit that list
instead of the cells (CandLists, sph_kernels.cuh); WCSPH's pressure-force
and non-pressure-force passes likewise.  The terms a list leaves
out are exactly the ones the walks skip, so a scene run with lists must equal
the same scene run with walks (neighbor_list_max = 0) bit for bit: here the
PCISPH drop (viscosity, surface tension, adhesion, Akinci walls) through its
impact, in FP32 and FP64; a fast scene whose predicted displacements exceed
the lists' margin (the predicted-density pass then walks the cells); and
lists too short for most particles (those walk); and the same drop as a
WCSPH scene (stiffness 1000, gamma 7, with the same forces)."""
import numpy as np
import pytest

import sph_gb300
from scenes import jitter
from sph_gb300 import workloads

pytestmark = pytest.mark.gpu

R = 0.01


def drop(case):
    x, b, p, _ = workloads.pcisph_drop(R)
    x = jitter(x, R, 5)
    v = np.zeros_like(x)
    if case == "impact":
        # the sphere already falling at 3.4 m/s, 2 cm above the pool
        top = x[:, 1] > 0.07
        x[top, 1] -= 0.38
        v[top, 1] = -3.4
    if case == "fast":
        v[:, 1] = -3.0
        p = dict(p, dt=1e-3)
    if case == "wcsph":
        top = x[:, 1] > 0.07
        x[top, 1] -= 0.38
        v[top, 1] = -3.4
        p = dict(p, method=0, stiffness=1000.0, gamma=7.0, dt=5e-5)
    return x, v, b, p


def run(x, v, b, p, precision, lists, steps, graph):
    s = sph_gb300.Scene(precision=precision, threads_per_particle=1, neighbor_list_max=lists, **p)
    s.set_fluid(x, v)
    s.add_boundary_points(b)
    s.init()
    s.set_graph(graph)
    s.set_profiling(not graph)
    s.step(steps)
    s.synchronize()
    return s


@pytest.mark.parametrize("case,precision,lists", [("impact", "f32", 64), ("impact", "f64", 64), ("fast", "f32", 64),
                                                  ("impact", "f32", 16), ("wcsph", "f32", 64), ("wcsph", "f64", 64)])
@pytest.mark.parametrize("graph", [False, True], ids=["host", "graph"])
def test_candidate_lists_equal_cell_walks(gpu_lib, case, precision, lists, graph):
    x, v, b, p = drop(case)
    steps = 40
    a = run(x, v, b, p, precision, lists, steps, graph)
    w = run(x, v, b, p, precision, 0, steps, graph)
    if not graph:
        assert "k_density_cand" in a.profile()
    for f in ("x", "v", "rho"):
        assert np.array_equal(a.get(f), w.get(f)), f
    sa, sw = a.stats(), w.stats()
    assert sa["sum_iterations"] == sw["sum_iterations"] and sa["status"] == sw["status"]
    if case != "fast":
        assert sa["status"] == 0
    assert np.isfinite(a.get("x")).all()
    print(case, precision, lists, "graph" if graph else "host", "iterations", sa["sum_iterations"])
