"""The GPU drop-in solvers (sph_gb300/adapter/) compiled with the reference.

GpuWCSPHSolver / GpuPCISPHSolver / GpuDFSPHSolver derive from the reference's
solver classes and override SPHSolver::init/step/resizeData
(src/SPHSolver.h:37-39).  Here, where the reference tree is present:

* `make -C oracle adapter` compiles them against the reference's unmodified
  headers and links them, with the reference's sources, to the library;
* the reference's src/Simulation.cpp compiled under
  `-include sph_gpu_select.h` constructs the GPU solvers in its factory
  (Simulation::setSimulationMethod, src/Simulation.cpp:207-231), and the
  plain build does not;
* the scene the GPU solvers' init() reads from the reference's live objects
  after Simulation::importScene (settings, solver parameters, forces,
  fluid, boundary points and normals, emitters) equals, for every committed
  scene file, the reference's own state (fixtures of the reference build)
  and the library's own reading of the same file.

Running the reference with the GPU solvers (oracle/adapter_run.cpp) needs
the reference's sources and a GPU on one machine, which no machine of this
build has: the CPU machine has no GPU and the GPU machine no reference tree.
"""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
import sph_gb300
from util import GOLDEN

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")
SCENE_DIR = os.path.join(GOLDEN, "scenes")
FILES = sorted(f[:-5] for f in os.listdir(SCENE_DIR) if f.endswith(".json"))

pytestmark = pytest.mark.skipif(not oracle.reference_available(), reason="reference build not present")


@pytest.fixture(scope="module")
def adapter():
    sph_gb300.build()
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "adapter", "-j8"], check=True, capture_output=True)
    exe = os.path.join(REF_DIR, "adapter_capture")
    assert os.path.exists(exe) and os.path.exists(os.path.join(REF_DIR, "adapter_run"))
    return exe


def undefined_symbols(obj):
    out = subprocess.run(["nm", "-C", "-u", obj], check=True, capture_output=True, text=True).stdout
    return out


def test_factory_constructs_the_gpu_solvers(adapter):
    gpu = undefined_symbols(os.path.join(REF_DIR, "gpu", "Simulation.o"))
    cpu = undefined_symbols(os.path.join(REF_DIR, "parity", "Simulation.o"))
    for cls in ("GpuWCSPHSolver", "GpuPCISPHSolver", "GpuDFSPHSolver"):
        assert f"vtable for {cls}" in gpu, cls
        assert cls not in cpu


def capture(exe, name, tmp_path):
    """The adapter's capture of the scene file after importScene, run in a
    directory holding the file and its meshes (paths are relative to the
    working directory, as the reference reads them)."""
    run = tmp_path / "run"
    run.mkdir()
    src = os.path.join(SCENE_DIR, name + ".json")
    shutil.copy(src, run / (name + ".json"))
    cfg = json.load(open(src))
    for b in cfg.get("Boundary", []):
        for g in b.get("geometry", []):
            dst = run / g["path"]
            dst.parent.mkdir(parents=True, exist_ok=True)
            shutil.copy(os.path.join(SCENE_DIR, g["path"]), dst)
    out = tmp_path / "capture.bin"
    with open(os.devnull, "rb") as dn_in, open(os.devnull, "wb") as dn_out:
        subprocess.run([exe, name + ".json", str(out)], stdin=dn_in, stdout=dn_out, check=True, cwd=run,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    return oracle.read_dump(str(out)), cfg, run


DESC_FIELDS = ("simulation_method", "boundary_method", "particle_radius", "time_step", "max_time_step", "fps",
               "density0", "viscosity_method", "surface_tension_method", "surface_tension", "adhesion_method",
               "adhesion", "has_cube")


@pytest.mark.parametrize("name", FILES)
def test_captured_scene_equals_reference_state_and_library_reading(adapter, name, tmp_path, monkeypatch):
    cap, cfg, run = capture(adapter, name, tmp_path)
    monkeypatch.chdir(run)
    path = str(run / (name + ".json"))
    g = dict(np.load(os.path.join(GOLDEN, f"file_{name}.npz")))
    # the reference's own state after importScene + init
    na = cap["x"].size // 3
    assert na == g["init.rho"].size
    assert np.array_equal(cap["x"], g["init.x"][: 3 * na])
    assert np.array_equal(cap["v"], g["init.v"][: 3 * na])
    c = cfg["Configuration"]
    if c["boundaryMethod"] == 2:
        assert np.array_equal(cap["boundary"], g["b.x"]) and cap["bh_points"].size == 0
    elif c["boundaryMethod"] == 1:
        assert np.array_equal(cap["bh_points"], g["b.x"]) and cap["boundary"].size == 0
        # the model's normals as the oracle builds the same shapes (pinned to
        # the reference build, normals included)
        b = cfg["Boundary"][0]
        o = oracle.OracleScene(dict(method=c["simulationMethod"], boundary=1, radius=c["particleRadius"]),
                               cap["x"].reshape(-1, 3),
                               bh_boxes=[(q["min"], q["max"], q["inverted"]) for q in b.get("box", [])],
                               bh_spheres=[(q["pos"], q["radius"], q["inverted"]) for q in b.get("sphere", [])])
        assert np.array_equal(cap["bh_points"], o.get("bx").ravel())
        assert np.array_equal(cap["bh_normals"], o.get("bn").ravel(), equal_nan=True)
    else:
        assert cap["boundary"].size == 0 and cap["bh_points"].size == 0
    # emitters: FluidModel::addEmitter's arguments (SceneLoader.cpp:115-138)
    emits = cfg["Fluid"]["FluidModel"][0].get("emitters", [])
    em = cap["emitters"].reshape(-1, 15)
    assert em.shape[0] == len(emits)
    for row, e in zip(em, emits):
        assert row[0] == e["type"] and row[1] == e["numParticles"] and list(row[2:5]) == e["position"]
        assert row[5] == e["velocity"] and list(row[6:10]) == e["rotation"]
        assert (row[10], row[11], row[12], row[13], row[14]) == (e["startTime"], e["width"], e["height"],
                                                                 e["spacing"], 0.0)
    assert cap["num_fluid_total"][0] == na + sum(e["numParticles"] for e in emits)
    # the library's reading of the same file (sph_ctx_load_scene): the same
    # descriptor, up to what the reference itself normalises -- the minimum
    # time step is min(minTimeStep, 1/fps) (TimeManager.h:55) and a force
    # with a zero coefficient does not exist (FluidModel.cpp:73-122)
    s = sph_gb300.Scene.load(path, init=False)
    d = s.desc()
    nf, nb = s.counts()
    s.close()
    for f in DESC_FIELDS:
        assert cap["desc." + f][0] == d[f], f
    assert list(cap["desc.gravity"]) == d["gravity"]
    assert cap["desc.min_time_step"][0] == min(d["min_time_step"], 1.0 / d["fps"])
    assert cap["desc.viscosity"][0] == d["viscosity"]
    if d["viscosity"] != 0.0:
        assert cap["desc.boundary_viscosity"][0] == d["boundary_viscosity"]
    if d["simulation_method"] == 0:
        assert cap["desc.stiffness"][0] == d["stiffness"] and cap["desc.gamma"][0] == d["gamma"]
    else:
        for f in ("max_error", "min_iterations", "max_iterations"):
            assert cap["desc." + f][0] == d[f], f
    if d["simulation_method"] == 2:
        for f in ("max_error_v", "cfl_factor", "min_iterations_v", "max_iterations_v"):
            assert cap["desc." + f][0] == d[f], f
    if d["boundary_method"] == 1:
        assert cap["desc.bh_normal_fct"][0] == d["bh_normal_fct"]
        assert cap["desc.bh_tangential_fct"][0] == d["bh_tangential_fct"]
    assert nf == na and nb == cap["boundary"].size // 3 + cap["bh_points"].size // 3
