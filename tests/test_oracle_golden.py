"""The C restatement (oracle) against fixtures produced by the reference
simulator itself (tests/golden/, generated by make_golden.py from the
reference's own sources): every field of every step must be identical."""
import numpy as np
import pytest

import oracle
from scenes import SCENES, scene, scene_extra
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
