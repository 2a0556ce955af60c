"""Scene files and frame files.

Scene files (SceneLoader::readConfiguration + Simulation::importScene) are
checked against the reference's own loader run on the same JSON files
(tests/golden/scenes/*.json, fixtures file_*.npz made by
tests/golden/make_golden.py): the settings and particle counts on the CPU,
and on the GPU the initial state bit for bit and 12 steps within the FP64
parity tolerance (1e-5 relative).  Frame files (SceneLoader::writeFluid):
the same frame numbers and file names as the reference's, the same
structure and counts, values within the FP64 tolerance, and numbers laid out
as the reference writes them.  The layout rules below are first checked
against every number in the reference's own frame files: the reference's
JSON writer (Grisu2 digit generation) gives the shortest round-trip digits
except for about one number in 10^4, where it writes a longer digit string
of the same value; this writer always writes the shortest.
"""
import json
import math
import os
import re
import tempfile
from decimal import Decimal

import numpy as np
import pytest

import sph_gb300
from util import GOLDEN, relerr

SCENE_DIR = os.path.join(GOLDEN, "scenes")
FILES = sorted(f[:-5] for f in os.listdir(SCENE_DIR) if f.endswith(".json"))
STEP_FIELDS = ("x", "v", "rho", "p", "alpha", "div", "pred", "k", "kv", "pacc")


_RESOLVED = {}


def scene_path(name):
    """The scene file; a scene with meshes is copied with its mesh paths
    (relative to the file) made absolute, since they are read relative to
    the working directory."""
    path = os.path.join(SCENE_DIR, name + ".json")
    cfg = json.load(open(path))
    if not any(b.get("geometry") for b in cfg.get("Boundary", [])):
        return path
    if name not in _RESOLVED:
        for b in cfg["Boundary"]:
            for g in b.get("geometry", []):
                g["path"] = os.path.abspath(os.path.join(SCENE_DIR, g["path"]))
        d = tempfile.mkdtemp(prefix="sph_scene_")
        _RESOLVED[name] = os.path.join(d, name + ".json")
        with open(_RESOLVED[name], "w") as f:
            json.dump(cfg, f)
    return _RESOLVED[name]


def fixture(name):
    return dict(np.load(os.path.join(GOLDEN, f"file_{name}.npz")))


def fmt(v):
    """A double as the frame files write it: the shortest digits that read
    back to it, in nlohmann::json's layout (decimal point position n:
    'ddd00.0' for k <= n <= 15, 'dd.dd' for 0 < n <= 15, '0.00dd' for
    -4 < n <= 0, else 'd.ddde+XX')."""
    if not math.isfinite(v):
        return "null"
    sign = "-" if math.copysign(1.0, v) < 0 else ""
    v = abs(v)
    if v == 0.0:
        return sign + "0.0"
    t = Decimal(repr(v)).normalize().as_tuple()
    digits = "".join(map(str, t.digits))
    k = len(digits)
    n = k + t.exponent
    if k <= n <= 15:
        body = digits + "0" * (n - k) + ".0"
    elif 0 < n <= 15:
        body = digits[:n] + "." + digits[n:]
    elif -4 < n <= 0:
        body = "0." + "0" * (-n) + digits
    else:
        x = n - 1
        body = digits[0] + ("." + digits[1:] if k > 1 else "") + "e" + ("-" if x < 0 else "+") + f"{abs(x):02d}"
    return sign + body


def frame_text(st):
    """The frame file SceneLoader::writeFluid writes for a parsed state."""
    out = f'{{"numActiveParticles":{st["numActiveParticles"]},"numParticles":{st["numParticles"]}'
    tri = lambda a: "[" + ",".join("[" + ",".join(fmt(float(c)) for c in p) + "]" for p in a) + "]"
    if st["numParticles"]:
        out += ',"positions":' + tri(st["positions"])
    out += ',"time":' + fmt(st["time"]) + ',"timeStep":' + fmt(st["timeStep"])
    if st["numParticles"]:
        out += ',"velocities":' + tri(st["velocities"])
    return out + "}"


# ---------------------------------------------------------------------------
# CPU: loader settings and counts, errors, the frame layout rules
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("name", FILES)
def test_scene_file_settings_and_counts(name):
    sph_gb300.build()
    cfg = json.load(open(scene_path(name)))
    g = fixture(name)
    s = sph_gb300.Scene.load(scene_path(name), init=False)
    d = s.desc()
    c, fl = cfg["Configuration"], cfg["Fluid"]
    fm = fl["FluidModel"][0]
    assert d["simulation_method"] == c["simulationMethod"] and d["boundary_method"] == c["boundaryMethod"]
    assert d["particle_radius"] == c["particleRadius"] and d["time_step"] == c["timeStep"] and d["fps"] == c["fps"]
    assert d["gravity"] == c["gravity"] and d["density0"] == fm["density0"]
    assert d["viscosity_method"] == fl["viscosityMethod"] and d["surface_tension_method"] == fl["surfaceTensionMethod"]
    if fl["viscosityMethod"] > -1:
        assert d["viscosity"] == fm["viscosity"] and d["boundary_viscosity"] == fm["boundaryViscosity"]
    if c["simulationMethod"] != 0:
        assert d["max_error"] == c["eta"] and d["max_iterations"] == c["maxIterations"]
    if c["boundaryMethod"] == 1:
        b = cfg["Boundary"][0]
        assert d["bh_normal_fct"] == b["normalFct"] and d["bh_tangential_fct"] == b["tangFct"]
    assert d["has_cube"] == 0
    nf, nb = s.counts()
    assert nf == g["init.rho"].size
    assert nb == (g["b.x"].size // 3 if "b.x" in g else 0)
    s.close()


def _write(tmp_path, cfg):
    p = tmp_path / "scene.json"
    p.write_text(json.dumps(cfg) if not isinstance(cfg, str) else cfg)
    return str(p)


def test_scene_file_errors(tmp_path):
    sph_gb300.build()
    base = json.load(open(scene_path("dfsph_dam_emitter")))
    cases = []
    c = json.loads(json.dumps(base)); del c["Configuration"]["fps"]; cases.append((c, "Configuration.fps"))
    c = json.loads(json.dumps(base)); c["Fluid"]["FluidModel"].append(c["Fluid"]["FluidModel"][0]); cases.append((c, "one fluid model"))
    c = json.loads(json.dumps(base)); c["Boundary"][0]["geometry"] = [{"path": "/nonexistent/a.obj", "spacing": 1.0}]
    cases.append((c, "a.obj"))
    c = json.loads(json.dumps(base)); c["Boundary"][0]["geometry"] = [{"spacing": 1.0}]
    cases.append((c, "geometry[0].path"))
    c = json.loads(json.dumps(base)); c["Boundary"].append(c["Boundary"][0]); cases.append((c, "more than one Boundary"))
    c = json.loads(json.dumps(base)); c["Configuration"]["simulationMethod"] = 5; cases.append((c, "simulationMethod"))
    c = json.loads(json.dumps(base)); c["Configuration"]["gravity"] = [0, -9.81]; cases.append((c, "gravity"))
    cases.append(('{"Configuration": {', "JSON"))
    for cfg, word in cases:
        with pytest.raises(sph_gb300.SPHError, match=re.escape(word)):
            sph_gb300.Scene.load(_write(tmp_path, cfg), init=False)
    with pytest.raises(sph_gb300.SPHError, match="cannot read"):
        sph_gb300.Scene.load(str(tmp_path / "missing.json"), init=False)


def test_scene_file_without_lists_and_boundary(tmp_path):
    """Missing fluidBlocks / emitters / Boundary lists count as empty."""
    sph_gb300.build()
    c = json.load(open(scene_path("wcsph_open_emitter")))
    del c["Fluid"]["FluidModel"][0]["emitters"]
    s = sph_gb300.Scene.load(_write(tmp_path, c), init=False)
    assert s.counts() == (125, 0)


NUMBER = re.compile(r"-?\d+(?:\.\d+)?(?:e[+-]\d+)?")


@pytest.mark.parametrize("name", FILES)
def test_frame_layout_rules_reproduce_reference_frames(name):
    """The layout rules reproduce the reference's frame files: the same
    text outside the numbers, and every number either identical or (the
    reference's Grisu2 digits not the shortest) of the same value, layout
    and length within one digit, for at most 1 number in 1000."""
    g = fixture(name)
    frames = sorted(int(k[5:-4]) for k in g if k.endswith(".raw"))
    assert frames
    total = longer = 0
    for f in frames:
        raw = bytes(g[f"frame{f}.raw"]).decode()
        mine = frame_text(json.loads(raw))
        assert NUMBER.sub("#", raw) == NUMBER.sub("#", mine), (name, f)
        for a, b in zip(NUMBER.findall(raw), NUMBER.findall(mine)):
            total += 1
            if a != b:
                longer += 1
                assert float(a) == float(b) and len(a) == len(b) + 1 and ("e" in a) == ("e" in b), (a, b)
    assert longer <= max(1, total // 1000), (longer, total)


def test_number_layout_cases():
    assert fmt(0.0) == "0.0" and fmt(-0.0) == "-0.0"
    assert fmt(1000.0) == "1000.0" and fmt(1e14) == "100000000000000.0" and fmt(1e15) == "1e+15"
    assert fmt(1.5) == "1.5" and fmt(0.07) == "0.07" and fmt(0.0001) == "0.0001" and fmt(1e-05) == "1e-05"
    assert fmt(-9.81) == "-9.81" and fmt(1.2345e-7) == "1.2345e-07" and fmt(float("nan")) == "null"


# ---------------------------------------------------------------------------
# GPU: imported scenes and frame files against the reference
# ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("name", FILES)
def test_imported_scene_matches_reference(gpu_lib, name):
    g = fixture(name)
    s = sph_gb300.Scene.load(scene_path(name), precision="f64")
    assert np.array_equal(s.get("x").ravel(), g["init.x"])
    if "b.x" in g:
        assert np.array_equal(s.get("bx").ravel(), g["b.x"])
    for step in range(1, 13):
        s.step(1)
        if f"s{step}.x" not in g:
            continue
        assert s.n == g[f"s{step}.rho"].size, (name, step)
        for f in STEP_FIELDS:
            key = f"s{step}.{f}"
            if key in g:
                e = relerr(s.get(f), g[key])
                assert e <= 1e-5, (name, key, e)
        st = s.stats()
        assert abs(st["time"] - g[f"s{step}.time"][0]) <= 1e-12 * max(g[f"s{step}.time"][0], 1e-300)
        assert st["iterations"] == int(g[f"s{step}.iterations"][0]), (name, step)


@pytest.mark.gpu
@pytest.mark.parametrize("name", FILES)
def test_frame_files_match_reference(gpu_lib, name, tmp_path):
    g = fixture(name)
    s = sph_gb300.Scene.load(scene_path(name), precision="f64")
    stem = str(tmp_path / "scene.json")
    s.set_frame_output(stem, True)
    s.step(12)
    s.synchronize()  # frame files are written by a host thread; complete after synchronize
    ref = sorted(int(k[5:-4]) for k in g if k.endswith(".raw"))
    mine = sorted(int(f[6:-5]) for f in os.listdir(tmp_path) if re.fullmatch(r"scene_\d{4}\.json", f))
    assert mine == ref
    assert s.frame == ref[-1] + 1
    for f in ref:
        raw = open(tmp_path / f"scene_{f:04d}.json").read()
        st = json.loads(raw)
        assert raw == frame_text(st)  # the writer's layout
        assert st["numParticles"] == g[f"frame{f}.numParticles"][0]
        assert st["numActiveParticles"] == g[f"frame{f}.numActiveParticles"][0]
        assert abs(st["time"] - g[f"frame{f}.time"][0]) <= 1e-12 * g[f"frame{f}.time"][0]
        assert abs(st["timeStep"] - g[f"frame{f}.timeStep"][0]) <= 1e-12 * g[f"frame{f}.timeStep"][0]
        for key in ("positions", "velocities"):
            a = np.asarray(st[key], dtype=np.float64).ravel()
            assert relerr(a, g[f"frame{f}.{key}"]) <= 1e-5, (name, f, key)
        na = st["numActiveParticles"]
        assert not np.any(np.asarray(st["positions"])[na:])


@pytest.mark.gpu
@pytest.mark.parametrize("save", [False, True])
def test_run_stops_at_the_end_time(gpu_lib, tmp_path, save):
    """Simulation::run: 1 ms steps while time <= 0.0101 s: 11 steps, with or
    without frame output (frames at 4 and 8 ms)."""
    s = sph_gb300.Scene.load(scene_path("wcsph_open_emitter"), precision="f64")
    if save:
        s.set_frame_output(str(tmp_path / "scene.json"), True)
    assert s.run() == 11
    assert abs(s.stats()["time"] - 0.011) < 1e-12
    assert s.run() == 0
    if save:
        assert sorted(os.listdir(tmp_path)) == ["scene_0001.json", "scene_0002.json"]


@pytest.mark.gpu
def test_frame_files_written_while_stepping_match_synchronous_frames(gpu_lib, tmp_path):
    """Frames queued to the writer thread during 12 graph steps equal the
    frames written synchronously (sph_ctx_write_frame) from a second run of
    the same scene stopped at the same steps, byte for byte."""
    name = "dfsph_dam_emitter"
    a = sph_gb300.Scene.load(scene_path(name), precision="f32")
    a.set_graph(True)
    a.set_frame_output(str(tmp_path / "a.json"), True)
    a.step(12)
    a.close()  # writes what is queued
    b = sph_gb300.Scene.load(scene_path(name), precision="f32")
    b.set_graph(True)
    frames = sorted(f for f in os.listdir(tmp_path) if f.startswith("a_"))
    assert len(frames) >= 3
    last_save, frame, fps = 0.0, 1, 200.0
    for _ in range(12):
        b.step(1)
        t = b.stats()["time"]
        if t - last_save >= 1.0 / fps:
            last_save = frame / fps
            b.write_frame(str(tmp_path / f"b_{frame:04d}.json"))
            frame += 1
    for f in frames:
        assert open(tmp_path / f, "rb").read() == open(tmp_path / ("b_" + f[2:]), "rb").read(), f
