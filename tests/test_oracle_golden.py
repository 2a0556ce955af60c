"""The C restatement (oracle) against fixtures produced by the reference
simulator itself (tests/golden/, generated by make_golden.py from the
reference's own sources): every field of every step must be identical."""
import numpy as np
import pytest

import oracle
from scenes import EMIT_DUMP_EVERY, EMIT_SCENES, EMIT_STEPS, SCENES, emit_scene, scene, scene_extra
from util import golden

FIELDS = ("x", "v", "rho", "p", "alpha", "div", "pred", "k", "kv", "pacc", "normal", "bdens", "bpress")


def same(a, b):
    """Bit-identical, NaN where the reference has NaN (the PCISPH boundary
    model leaves NaN normals on particles that touched no boundary point)."""
    return np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(np.nan_to_num(a), np.nan_to_num(b))


@pytest.mark.parametrize("name", list(SCENES))
def test_oracle_reproduces_reference_bit_exact(name):
    params, x, boxes, spheres = scene(name)
    v, bh_boxes, bh_spheres = scene_extra(name, x)
    g = golden(name)
    assert np.array_equal(g["input.x"], x), "scene inputs changed; regenerate the fixtures"
    o = oracle.OracleScene(params, x, v, boxes=boxes, spheres=spheres, bh_boxes=bh_boxes, bh_spheres=bh_spheres)
    if params["boundary"] == 1:
        assert np.array_equal(o.get("bx").ravel(), g["b.x"])
    if "b.psi" in g:
        assert np.array_equal(o.get("bx").ravel(), g["b.x"])
        assert np.array_equal(o.get("psi"), g["b.psi"])
    if params["method"] == 2:
        assert np.array_equal(o.get("rho"), g["init.rho"])
        assert np.array_equal(o.get("alpha"), g["init.alpha"])
        nb = o.neighbors()
        assert np.array_equal(nb["cell"].ravel(), g["init.cell"])
        assert np.array_equal(nb["cell_rank"], g["init.cell_rank"])
        assert np.array_equal(nb["nbr_off"], g["init.nbr_off"])
        assert np.array_equal(nb["nbr"], g["init.nbr"])
        assert np.array_equal(nb["bnbr"], g["init.bnbr"])
    step = 1
    while f"s{step}.x" in g:
        o.step(1)
        for f in FIELDS:
            key = f"s{step}.{f}"
            if key in g:
                assert same(o.get(f).ravel(), g[key]), (name, key)
        assert o.scalar("dt") == g[f"s{step}.dt"][0]
        assert o.scalar("iterations") == g[f"s{step}.iterations"][0]
        step += 1
    assert step > 1


@pytest.mark.parametrize("name", list(EMIT_SCENES))
def test_oracle_reproduces_reference_with_emitters(name):
    """Emitter scenes: identical bits and identical active-particle counts at
    every stored step (every third of 30), with groups emitted on the way."""
    params, x, boxes, spheres, emitters = emit_scene(name)
    g = golden(name)
    assert np.array_equal(g["input.x"], x), "scene inputs changed; regenerate the fixtures"
    o = oracle.OracleScene(params, x, boxes=boxes, spheres=spheres, emitters=emitters)
    checked = 0
    for step in range(1, EMIT_STEPS + 1):
        o.step(1)
        if f"s{step}.x" not in g:
            continue
        assert o.n == g[f"s{step}.rho"].size, (name, step)
        for f in FIELDS:
            key = f"s{step}.{f}"
            if key in g:
                assert same(o.get(f).ravel(), g[key]), (name, key)
        assert o.scalar("dt") == g[f"s{step}.dt"][0]
        assert o.scalar("iterations") == g[f"s{step}.iterations"][0]
        checked += 1
    assert checked == EMIT_STEPS // EMIT_DUMP_EVERY
    assert o.n >= x.shape[0] + 2 * 19


def test_oracle_emitter_pause_restarts_the_clock():
    """Emitter::setPause: no group while paused; on resume the next group
    leaves at once with a zero time offset (nextTimeEmit = current time)."""
    params, x, boxes, spheres, emitters = emit_scene("dfsph_emit_only")
    o = oracle.OracleScene(params, x, boxes=boxes, spheres=spheres, emitters=emitters)
    o.step(1)
    assert o.n == 19
    o.pause_emitters(True)
    o.step(20)
    assert o.n == 19
    o.pause_emitters(False)
    o.step(1)
    assert o.n == 38
    # the resumed group sits exactly at the emitter's rotated group points
    e = emitters[0]
    grp = oracle.emitter_group(1, params["radius"], e["width"])
    w, qx, qy, qz = e["rotation"]
    u = np.array([qx, qy, qz])
    uv = np.cross(u, grp)
    rot = grp + 2.0 * (w * uv + np.cross(u, uv)) + np.array(e["position"])
    assert np.allclose(o.get("x")[19:38], rot, atol=1e-3)


def test_pcisph_model_cube_sampler():
    # PCISPHBoundaryModel::sampleCube: spacing <= 0.45 h, normals of the
    # faces / edges / corners pointing into the box when inverted
    pts, nrm = oracle.sample_bh_box(0.08, (0, 0, 0), (0.6, 0.6, 0.6), inverted=True)
    n = int(np.ceil(0.6 / (0.45 * 0.08)))
    assert pts.shape == ((n + 1) ** 3 - (n - 1) ** 3, 3)
    assert np.allclose(np.linalg.norm(nrm, axis=1), 1.0)
    centre = np.array([0.3, 0.3, 0.3])
    assert np.all(((centre - pts) * nrm).sum(1) > 0)
    _, out = oracle.sample_bh_box(0.08, (0, 0, 0), (0.6, 0.6, 0.6), inverted=False)
    assert np.array_equal(out, -nrm)


def test_samplers_match_reference_counts():
    # AkinciBoundaryModel::sampleCube at h/2 on the dam-break box, r = 0.01
    pts = oracle.sample_box(0.04, (0, 0, 0), (1.5, 0.8, 0.8))
    assert pts.shape == (15202, 3)
    # r = 0.005 variant of the same box
    assert oracle.sample_box(0.02, (0, 0, 0), (1.5, 0.8, 0.8)).shape == (60802, 3)
