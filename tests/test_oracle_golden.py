"""The C restatement (oracle) against fixtures produced by the reference
simulator itself (tests/golden/, generated by make_golden.py from the
reference's own sources): every field of every step must be identical."""
import numpy as np
import pytest

import oracle
from scenes import SCENES, scene
from util import golden

FIELDS = ("x", "v", "rho", "p", "alpha", "div", "pred", "k", "kv", "pacc")


@pytest.mark.parametrize("name", list(SCENES))
def test_oracle_reproduces_reference_bit_exact(name):
    params, x, boxes, spheres = scene(name)
    g = golden(name)
    assert np.array_equal(g["input.x"], x), "scene inputs changed; regenerate the fixtures"
    o = oracle.OracleScene(params, x, boxes=boxes, spheres=spheres)
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
                assert np.array_equal(o.get(f).ravel(), g[key]), (name, key)
        assert o.scalar("dt") == g[f"s{step}.dt"][0]
        assert o.scalar("iterations") == g[f"s{step}.iterations"][0]
        step += 1
    assert step > 1


def test_samplers_match_reference_counts():
    # AkinciBoundaryModel::sampleCube at h/2 on the dam-break box, r = 0.01
    pts = oracle.sample_box(0.04, (0, 0, 0), (1.5, 0.8, 0.8))
    assert pts.shape == (15202, 3)
    # r = 0.005 variant of the same box
    assert oracle.sample_box(0.02, (0, 0, 0), (1.5, 0.8, 0.8)).shape == (60802, 3)
