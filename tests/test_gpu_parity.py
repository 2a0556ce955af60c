"""GPU parity: the CUDA path (through the C ABI) against the reference's own
results (golden fixtures) and the C restatement, on the same inputs.

Tolerances:
  * grid: cell keys, in-cell ranks and per-particle neighbour lists are
    compared for equality (bit-exact);
  * FP64 form: fields after init within 1e-10 relative, after 1-3 steps within
    1e-5 relative (max |gpu - ref| / max |ref| per field), identical solver
    iteration counts;
  * FP32 form: errors against the FP64 reference are bounded per field
    (see test_f32_error_against_reference for the measured values).
"""
import numpy as np
import pytest

import oracle
import sph_gb300
from scenes import SCENES, jitter, scene, scene_extra
from util import golden, relerr

pytestmark = pytest.mark.gpu

DFSPH_SCENES = [n for n in SCENES if SCENES[n]["params"]["method"] == 2]
STEP_FIELDS = ("x", "v", "rho", "p", "alpha", "div", "pred", "k", "kv", "pacc")
# PCISPH boundary model: fluid normals (NaN where no boundary point was within
# h/2), boundary densities and pressures
BH_FIELDS = ("normal", "bdens", "bpress")


def nan_relerr(a, b):
    """relerr over the entries finite in both; inf when NaN patterns differ."""
    a, b = np.ravel(a), np.ravel(b)
    if not np.array_equal(np.isnan(a), np.isnan(b)):
        return np.inf
    m = ~np.isnan(b)
    return relerr(a[m], b[m]) if m.any() else 0.0


def gpu_scene(name, precision="f64", G=0, graph=False, lists=64):
    params, x, boxes, spheres = scene(name)
    v, bh_boxes, bh_spheres = scene_extra(name, x)
    s = sph_gb300.Scene(precision=precision, threads_per_particle=G, neighbor_list_max=lists, **params)
    s.set_fluid(x, v)
    for mn, mx in boxes:
        s.add_boundary_box(mn, mx)
    for c, r in spheres:
        s.add_boundary_sphere(c, r)
    for mn, mx, inv in bh_boxes:
        s.add_pcisph_box(mn, mx, inv)
    for c, r, inv in bh_spheres:
        s.add_pcisph_sphere(c, r, inv)
    s.init()
    if graph:
        s.set_graph(True)
    return s


@pytest.mark.parametrize("name", DFSPH_SCENES)
def test_f64_init_matches_reference(gpu_lib, name):
    g = golden(name)
    s = gpu_scene(name)
    if SCENES[name]["params"]["boundary"] == 1:
        assert np.array_equal(s.get("bx").ravel(), g["b.x"])
    if "b.psi" in g:
        assert np.array_equal(s.get("bx").ravel(), g["b.x"])
        assert relerr(s.get("psi"), g["b.psi"]) <= 1e-10
    assert relerr(s.get("rho"), g["init.rho"]) <= 1e-10
    assert relerr(s.get("alpha"), g["init.alpha"]) <= 1e-10


@pytest.mark.parametrize("name", DFSPH_SCENES)
def test_neighbour_sets_bit_exact(gpu_lib, name):
    g = golden(name)
    s = gpu_scene(name)
    nb = s.neighbors()
    assert np.array_equal(nb["cell"].ravel(), g["init.cell"])
    assert np.array_equal(nb["cell_rank"], g["init.cell_rank"])
    assert np.array_equal(nb["nbr_off"], g["init.nbr_off"])
    assert np.array_equal(nb["nbr"], g["init.nbr"])
    if SCENES[name]["params"]["boundary"] in (1, 2):
        # (the reference's cube model also files its two corner points as
        # boundary points in the grid; no walk ever reads them)
        assert np.array_equal(nb["bnbr_off"], g["init.bnbr_off"])
        assert np.array_equal(nb["bnbr"], g["init.bnbr"])


@pytest.mark.parametrize("lists", [64, 0], ids=["pairlists", "cellwalk"])
@pytest.mark.parametrize("name", list(SCENES))
def test_f64_steps_match_reference(gpu_lib, name, lists):
    g = golden(name)
    s = gpu_scene(name, lists=lists)
    step = 1
    while f"s{step}.x" in g:
        s.step(1)
        for f in STEP_FIELDS:
            key = f"s{step}.{f}"
            if key in g:
                e = relerr(s.get(f), g[key])
                assert e <= 1e-5, (name, key, e)
        for f in BH_FIELDS:
            key = f"s{step}.{f}"
            if key in g:
                e = nan_relerr(s.get(f), g[key])
                assert e <= 1e-5, (name, key, e)
        st = s.stats()
        assert abs(st["dt"] - g[f"s{step}.dt"][0]) <= 1e-12 * g[f"s{step}.dt"][0]
        assert st["iterations"] == int(g[f"s{step}.iterations"][0]), (name, step)
        if f"s{step}.iterationsV" in g:
            assert st["iterations_v"] == int(g[f"s{step}.iterationsV"][0]), (name, step)
        step += 1


@pytest.mark.parametrize("lists", [64, 0], ids=["pairlists", "cellwalk"])
@pytest.mark.parametrize("name", list(SCENES))
def test_f32_error_against_reference(gpu_lib, name, lists):
    """FP32 production form against the reference's FP64 results, 3 steps.
    Measured on GB300 (one lane per particle and the default 8 lanes of these
    small scenes alike): positions <= 2e-7 rel, densities <= 1.7e-6 rel,
    alpha <= 3.3e-6 rel, WCSPH/PCISPH pressures <= 1e-4 rel, velocities
    <= 5.2e-4 m/s abs, and identical iteration counts.  Bounds below leave
    ~5x headroom.  The velocity bound is loose because most of these scenes
    are exact lattices: neighbours at exactly h make the reference's
    20-neighbour rule and rho* >= rho0 clamp depend on the last bit, so
    single wall-layer particles get or miss a divergence correction; the
    jittered test below holds FP32 velocities to 1e-3 of the largest speed
    (measured 7e-5 for DFSPH, 1e-6 for WCSPH)."""
    g = golden(name)
    s = gpu_scene(name, precision="f32", lists=lists)
    for step in (1, 2, 3):
        s.step(1)
        assert relerr(s.get("x"), g[f"s{step}.x"]) <= 1e-6
        assert relerr(s.get("rho"), g[f"s{step}.rho"]) <= 1e-5
        assert np.abs(s.get("v").ravel() - g[f"s{step}.v"]).max() <= 2.5e-3
        if f"s{step}.alpha" in g:
            assert relerr(s.get("alpha"), g[f"s{step}.alpha"]) <= 2e-5
        if SCENES[name]["params"]["method"] != 2:
            assert relerr(s.get("p"), g[f"s{step}.p"]) <= 1e-3
        assert s.stats()["iterations"] == int(g[f"s{step}.iterations"][0])


@pytest.mark.parametrize("name", ["dfsph_akinci", "dfsph_artvisc", "dfsph_cube", "wcsph_akinci"])
def test_f32_error_on_jittered_lattice(gpu_lib, name):
    """FP32 against the oracle on the exact-lattice scenes jittered by
    U(-0.01 r, 0.01 r).  An exact lattice of spacing 2r with h = 4r puts
    neighbours at exactly h, where the reference's 20-neighbour rule and the
    rho* >= rho0 clamp let the last bit decide, so the bounds of the test
    above are loose; off the lattice FP32 must track the FP64 reference
    closely: velocities within 1e-3 of the largest speed, positions 1e-6
    and densities 1e-5 relative, equal iteration counts, 3 steps."""
    params, x, boxes, spheres = scene(name)
    x = jitter(x, params["radius"], 7)
    o = oracle.OracleScene(params, x, boxes=boxes, spheres=spheres)
    s = sph_gb300.Scene(precision="f32", **params)
    s.set_fluid(x)
    for mn, mx in boxes:
        s.add_boundary_box(mn, mx)
    for c, r in spheres:
        s.add_boundary_sphere(c, r)
    s.init()
    for step in (1, 2, 3):
        o.step(1)
        s.step(1)
        vr = o.get("v")
        dv = np.abs(s.get("v") - vr).max()
        vmax = np.sqrt((vr * vr).sum(1)).max()
        print(f"{name} step {step}: |dv| {dv:.3e} of |v|max {vmax:.3e}")
        assert dv <= 1e-3 * vmax
        assert relerr(s.get("x"), o.get("x")) <= 1e-6
        assert relerr(s.get("rho"), o.get("rho")) <= 1e-5
        if params["method"] == 2:
            assert s.stats()["iterations"] == int(o.scalar("iterations"))
            assert s.stats()["iterations_v"] == int(o.scalar("iterationsV"))


def test_f64_twenty_steps_match_oracle(gpu_lib):
    params, x, boxes, spheres = scene("dfsph_akinci")
    o = oracle.OracleScene(params, x, boxes=boxes, spheres=spheres)
    s = gpu_scene("dfsph_akinci")
    for _ in range(20):
        o.step(1)
        s.step(1)
        assert s.stats()["iterations"] == o.scalar("iterations")
    for f in ("x", "v", "rho", "alpha"):
        assert relerr(s.get(f), o.get(f)) <= 1e-5, f


@pytest.mark.parametrize("name", ["dfsph_akinci", "pcisph_drop", "wcsph_cube"])
def test_graph_mode_equals_stream_mode(gpu_lib, name):
    a = gpu_scene(name, precision="f32")
    b = gpu_scene(name, precision="f32", graph=True)
    a.step(5)
    b.step(5)
    for f in ("x", "v", "rho"):
        assert np.array_equal(a.get(f), b.get(f)), f
    sa, sb = a.stats(), b.stats()
    assert sa["sum_iterations"] == sb["sum_iterations"] and sa["steps"] == sb["steps"] == 5


@pytest.mark.parametrize("G", [2, 4, 8])
def test_threads_per_particle_variants(gpu_lib, G):
    a = gpu_scene("dfsph_forces", precision="f32", G=1, lists=0)
    b = gpu_scene("dfsph_forces", precision="f32", G=G, lists=0)
    a.step(2)
    b.step(2)
    assert relerr(b.get("rho"), a.get("rho")) <= 1e-4
    assert relerr(b.get("x"), a.get("x")) <= 1e-5


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_pair_list_overflow_falls_back_to_cell_walk(gpu_lib, precision):
    """With 8 slots every particle overflows its pair list and every solver
    walk takes the cell-walk fallback; results must agree with the full lists."""
    a = gpu_scene("dfsph_akinci", precision=precision, lists=64)
    b = gpu_scene("dfsph_akinci", precision=precision, lists=8)
    a.step(3)
    b.step(3)
    tol = 1e-12 if precision == "f64" else 1e-5
    for f in ("x", "rho", "alpha"):
        assert relerr(b.get(f), a.get(f)) <= tol, f
    assert b.stats()["list_overflow"] > 0 and a.stats()["list_overflow"] == 0
    assert a.stats()["list_pairs"] > 20 * a.n


@pytest.mark.parametrize("name", ["wcsph_bh", "pcisph_bh", "dfsph_bh"])
def test_pcisph_boundary_model_twelve_steps_match_oracle(gpu_lib, name):
    """PCISPH boundary model, FP64, 12 steps with particles colliding every
    step: positions, velocities, densities, normals (NaN where no boundary
    point was within h/2) and boundary densities / pressures against the
    oracle within 1e-5 relative, identical iteration counts."""
    params, x, boxes, spheres = scene(name)
    v, bh_boxes, bh_spheres = scene_extra(name, x)
    o = oracle.OracleScene(params, x, v, bh_boxes=bh_boxes, bh_spheres=bh_spheres)
    s = gpu_scene(name)
    for step in range(12):
        o.step(1)
        s.step(1)
        for f in ("x", "v", "rho", "normal", "bdens", "bpress"):
            e = nan_relerr(s.get(f), o.get(f))
            assert e <= 1e-5, (name, step, f, e)
        assert s.stats()["iterations"] == o.scalar("iterations"), (name, step)
