"""Step phases under the reference's phase-timer names (NVTX ranges, and CUDA
event times while profiling is on): which phases a step reports, that each
runs once per host-driven step, that the phases of a step lie inside its
"Step computation" time, and that a graph step is one "Step computation".
The names follow Simulation::startCounting / stopCounting
(DFSPHSolver.cpp:43-101, PCISPHSolver.cpp:26-67, WCSPHSolver.cpp:20-64,
Simulation.cpp:158); fused phases join the reference's names with '+'."""
import pytest

import sph_gb300
from scenes import jitter, lattice

pytestmark = pytest.mark.gpu

R = 0.02


def fluid():
    return jitter(lattice(R, (2 * R, 2 * R, 2 * R), (0.3, 0.25, 0.3)), R, 5)


def walls():
    return sph_gb300.sample_box(4 * R, (0, 0, 0), (0.6, 0.6, 0.6))


SOLVERS = {
    "dfsph_lists": (dict(method=2, boundary=2, precision="f32", visc_method=2, visc=0.01), 64,
                    ["npForces", "Density solver", "Fill grid", "Neigh search+Densities+Alpha factor",
                     "Divergence solver"]),
    "dfsph_f64": (dict(method=2, boundary=2, precision="f64", visc_method=2, visc=0.01), 0,
                  ["npForces", "Density solver", "Fill grid", "Densities+Alpha factor", "Divergence solver"]),
    "pcisph": (dict(method=1, boundary=2, precision="f32", visc_method=0, visc=0.01, st_method=3, st=0.5), 0,
               ["Fill grid", "Densities", "npForces", "Pressure solver", "Integration"]),
    "wcsph": (dict(method=0, boundary=2, precision="f32", visc_method=2, visc=0.01, dt=1e-4), 0,
              ["Fill grid", "Densities+Pressures", "Pressure force", "NPForces", "Integratio"]),
}


def check_steps(ph, steps, inner):
    assert ph["Step computation"][0] == steps
    for name in inner:
        assert name in ph, (name, sorted(ph))
        assert ph[name][0] == steps, (name, ph[name])
    total = ph["Step computation"][1]
    inside = sum(ms for name, (_, ms) in ph.items() if name != "Step computation")
    assert 0.0 < inside <= total * 1.001 + 1e-3, (inside, total)


@pytest.mark.parametrize("solver", list(SOLVERS))
def test_one_scene_phases(gpu_lib, solver):
    params, lists, inner = SOLVERS[solver]
    s = sph_gb300.Scene(radius=R, neighbor_list_max=lists, **params)
    s.set_fluid(fluid())
    s.add_boundary_points(walls())
    s.init()
    s.set_profiling(True)
    s.step(3)
    ph = s.phase_profile()
    print(solver, ph)
    check_steps(ph, 3, inner)
    assert s.phase_profile() == {}      # consumed
    s.set_graph(True)
    s.step(2)
    assert set(s.phase_profile()) == {"Step computation"}


def test_pool_phases(gpu_lib):
    P = sph_gb300.Pool(max_particles=50_000, max_boundary=100_000, max_keys=1_000_000, max_scenes=4)
    P.set_autotune(0)
    P.set_graph(False)
    for k in range(2):
        P.add_scene(jitter(lattice(R, (2 * R, 2 * R, 2 * R), (0.3, 0.25 + 0.04 * k, 0.3)), R, 7 + k),
                    boundary_points=walls(), steps=50, radius=R, method=2, boundary=2, precision="f32")
    P.step(1)   # admission
    P.set_profiling(True)
    P.phase_profile()
    P.step(3)
    ph = P.phase_profile()
    print(ph)
    check_steps(ph, 3, ["Density solver", "Fill grid", "Neigh search+Densities+Alpha factor", "Divergence solver"])
