"""Emitters on the GPU (Emitter.cpp, FluidModel::addEmitter): particle groups
appended on the device, against the reference's own results (golden
fixtures, 30 steps, every third stored) and the oracle.

Tolerances: as the other parity tests, FP64 fields within 1e-5 relative
after each stored step with identical active-particle and iteration counts.
FP32 against the FP64 reference over the 30 steps: the error grows about
linearly with the step count; measured on GB300 at step 30 (worst scene,
dfsph_emit with 2 ms steps) positions 1.1e-6 and densities 1.4e-5 relative,
velocities 2e-4 m/s; bounds 1e-5, 1.5e-4 and 2.5e-3 m/s, with identical
active-particle and iteration counts.
"""
import numpy as np
import pytest

import oracle
import sph_gb300
from scenes import EMIT_SCENES, EMIT_STEPS, emit_scene
from util import golden, relerr

pytestmark = pytest.mark.gpu

FIELDS64 = ("x", "v", "rho", "p", "alpha", "div", "pred", "k", "kv", "pacc")


def gpu_emit_scene(name, precision="f64", lists=64, graph=False):
    params, x, boxes, spheres, emitters = emit_scene(name)
    s = sph_gb300.Scene(precision=precision, neighbor_list_max=lists, **params)
    s.set_fluid(x)
    for mn, mx in boxes:
        s.add_boundary_box(mn, mx)
    for c, r in spheres:
        s.add_boundary_sphere(c, r)
    for e in emitters:
        s.add_emitter(e["type"], e["num"], e["position"], e["velocity"], e["rotation"], e["start"], e["width"],
                      e["height"], e["spacing"])
    s.init()
    if graph:
        s.set_graph(True)
    return s


@pytest.mark.parametrize("lists", [64, 0], ids=["pairlists", "cellwalk"])
@pytest.mark.parametrize("name", list(EMIT_SCENES))
def test_f64_emitter_scenes_match_reference(gpu_lib, name, lists):
    g = golden(name)
    s = gpu_emit_scene(name, lists=lists)
    total = x0 = s.n
    for e in EMIT_SCENES[name]["emitters"]:
        total += e["num"]
    assert s.stats()["num_fluid_total"] == total
    for step in range(1, EMIT_STEPS + 1):
        s.step(1)
        if f"s{step}.x" not in g:
            continue
        assert s.n == g[f"s{step}.rho"].size, (name, step)
        for f in FIELDS64:
            key = f"s{step}.{f}"
            if key in g:
                e = relerr(s.get(f), g[key])
                assert e <= 1e-5, (name, key, e)
        st = s.stats()
        assert abs(st["dt"] - g[f"s{step}.dt"][0]) <= 1e-12 * g[f"s{step}.dt"][0]
        assert st["iterations"] == int(g[f"s{step}.iterations"][0]), (name, step)
        assert st["num_fluid"] == s.n
    assert s.n > x0


@pytest.mark.parametrize("name", list(EMIT_SCENES))
def test_f32_emitter_scenes_against_reference(gpu_lib, name):
    g = golden(name)
    s = gpu_emit_scene(name, precision="f32")
    for step in range(1, EMIT_STEPS + 1):
        s.step(1)
        if f"s{step}.x" not in g:
            continue
        assert s.n == g[f"s{step}.rho"].size, (name, step)
        assert relerr(s.get("x"), g[f"s{step}.x"]) <= 1e-5
        assert relerr(s.get("rho"), g[f"s{step}.rho"]) <= 1.5e-4
        assert np.abs(s.get("v").ravel() - g[f"s{step}.v"]).max() <= 2.5e-3
        assert s.stats()["iterations"] == int(g[f"s{step}.iterations"][0])


@pytest.mark.parametrize("name", ["dfsph_emit", "pcisph_emit"])
def test_emitter_graph_mode_equals_stream_mode(gpu_lib, name):
    """The captured step (launch shapes fixed at the reserved capacity) gives
    the same bits as stream mode while the active count grows."""
    a = gpu_emit_scene(name, precision="f32")
    b = gpu_emit_scene(name, precision="f32", graph=True)
    a.step(24)
    b.step(24)
    assert a.n == b.n
    for f in ("x", "v", "rho"):
        assert np.array_equal(a.get(f), b.get(f)), f


def test_emitter_pause_and_resume_match_oracle(gpu_lib):
    """Simulation::setEmittersPause mid-run, FP64, against the oracle."""
    params, x, boxes, spheres, emitters = emit_scene("dfsph_emit")
    o = oracle.OracleScene(params, x, boxes=boxes, spheres=spheres, emitters=emitters)
    s = gpu_emit_scene("dfsph_emit")
    for k, pause in ((3, True), (15, False), (14, None)):
        o.step(k)
        s.step(k)
        assert s.n == o.n
        if pause is not None:
            o.pause_emitters(pause)
            s.pause_emitters(pause)
    for f in ("x", "v", "rho"):
        assert relerr(s.get(f), o.get(f)) <= 1e-5, f
    assert s.n == o.n > x.shape[0] + 19
