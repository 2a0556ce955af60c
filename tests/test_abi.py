"""CPU checks of the C ABI: the library loads, exports every function the
header declares, rejects bad arguments, and its host-side samplers reproduce
the reference's point sets (no GPU needed for any of these)."""
import ctypes
import os
import re

import numpy as np
import pytest

import oracle
import sph_gb300

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def L():
    sph_gb300.build()
    return sph_gb300.lib()


def header_functions():
    src = open(os.path.join(ROOT, "include", "sph_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_ ]+?[\s*]+(sph_[a-z0-9_]+)\s*\(", src, flags=re.M)))


def test_header_symbols_exported(L):
    names = header_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert {n for n, _, _ in sph_gb300.ABI} == set(names)


def test_desc_defaults_follow_reference(L):
    d = sph_gb300.make_desc()
    assert d.simulation_method == sph_gb300.DFSPH
    assert d.time_step == 0.0001 and d.density0 == 1000.0 and d.cfl_factor == 1.0
    assert d.min_iterations == -1 and d.viscosity_method == -1


def test_create_rejects_bad_arguments(L):
    h = ctypes.c_void_p()
    for bad in (dict(method=5), dict(boundary=7), dict(radius=0.0), dict(dt=-1.0)):
        d = sph_gb300.make_desc(**bad)
        rc = L.sph_ctx_create(ctypes.byref(d), ctypes.byref(h))
        assert rc == -1


def test_step_before_init_is_an_error(L):
    s = sph_gb300.Scene(method=2, radius=0.02)
    with pytest.raises(sph_gb300.SPHError):
        s.step(1)
    s.close()


def test_grid_growth_switch(L):
    """sph_ctx_set_grid_growth is accepted before init (host state only) and
    refuses a null context."""
    s = sph_gb300.Scene(method=2, radius=0.02)
    s.set_grid_growth(False)
    s.set_grid_growth(True)
    s.close()
    assert L.sph_ctx_set_grid_growth(None, 1) == -1


@pytest.mark.parametrize("r,mn,mx", [(0.02, (0, 0, 0), (0.6, 0.5, 0.5)), (0.005, (0, 0, 0), (1.5, 0.8, 0.8)),
                                     (0.01, (0.1, 0.2, 0.3), (1.3, 0.7, 0.9))])
def test_box_sampler_matches_oracle(L, r, mn, mx):
    assert np.array_equal(sph_gb300.sample_box(4 * r, mn, mx), oracle.sample_box(4 * r, mn, mx))


@pytest.mark.parametrize("r,c,R", [(0.01, (0.5, 0.5, 0.5), 0.1), (0.005, (0.3, 0.2, 0.1), 0.2), (0.01, (0, 0, 0), 0.05)])
def test_sphere_sampler_matches_oracle(L, r, c, R):
    assert np.array_equal(sph_gb300.sample_sphere(r, c, R), oracle.sample_sphere(r, c, R))


def test_fluid_block_matches_oracle(L):
    a = sph_gb300.fluid_block(0.01, (0, 0, 0), (0.5, 0.5, 0.5))
    assert a.shape == (15625, 3)
    assert np.array_equal(a, oracle.fluid_block(0.01, (0, 0, 0), (0.5, 0.5, 0.5)))


def test_pcisph_model_sampler_matches_oracle():
    """The library's PCISPHBoundaryModel::sampleCube (points and normals, both
    orientations) equals the oracle's bit for bit."""
    import oracle

    for mn, mx in [((0, 0, 0), (0.6, 0.6, 0.6)), ((-0.1, 0.2, 0.05), (0.7, 0.55, 0.33))]:
        for inv in (True, False):
            a, an = sph_gb300.sample_pcisph_box(0.08, mn, mx, inv)
            b, bn = oracle.sample_bh_box(0.08, mn, mx, inv)
            assert np.array_equal(a, b) and np.array_equal(an, bn)


@pytest.mark.parametrize("type_,r,w,h", [(1, 0.02, 0.1, 0.0), (1, 0.005, 0.3, 0.0), (1, 0.02, 0.01, 0.0),
                                         (0, 0.02, 0.24, 0.16), (0, 0.01, 0.5, 0.05), (0, 0.02, 0.03, 0.5)])
def test_emitter_group_matches_oracle(L, type_, r, w, h):
    """Emitter::buildCircleGroup / buildSquareGroup: the library's group
    equals the oracle's bit for bit (including the degenerate cases: a circle
    narrower than one ring is its centre, a square narrower than one
    particle is empty)."""
    a = sph_gb300.emitter_group(type_, r, w, h)
    b = oracle.emitter_group(type_, r, w, h)
    assert a.shape == b.shape and np.array_equal(a, b)
    if type_ == 1 and w < 3 * r:
        assert a.shape == (1, 3)
    if type_ == 0 and w < 2 * r:
        assert a.shape == (0, 3)


def test_circle_group_rings():
    g = sph_gb300.emitter_group(sph_gb300.EMITTER_CIRCLE, 0.02, 0.1)
    # centre + floor(2 pi R / 2r) points on rings R = 0.04, 0.08
    assert g.shape == (1 + 6 + 12, 3)
    rr = np.sqrt((g[:, :2] ** 2).sum(1))
    assert np.allclose(sorted(set(np.round(rr, 12))), [0.0, 0.04, 0.08])


def test_add_emitter_rejects_bad_arguments(L):
    s = sph_gb300.Scene(method=2, radius=0.02)
    with pytest.raises(sph_gb300.SPHError):
        s.add_emitter(2, 10, (0, 0, 0), 1.0, width=0.1)
    with pytest.raises(sph_gb300.SPHError):
        s.add_emitter(1, 10, (0, 0, float("nan")), 1.0, width=0.1)
    for _ in range(64):
        s.add_emitter(1, 10, (0, 0, 0), 1.0, width=0.1)
    with pytest.raises(sph_gb300.SPHError):
        s.add_emitter(1, 10, (0, 0, 0), 1.0, width=0.1)
    with pytest.raises(sph_gb300.SPHError):
        s.pause_emitters(True)  # before init
    s.close()


MESH_DIR = os.path.join(ROOT, "tests", "golden", "meshes")


def test_mesh_sampler_matches_reference(L):
    """AkinciBoundaryModel::addGeometry's samples (OBJ reader, regular
    triangle sampling in FP32, rotation by pi/2 about x): the library's
    points equal the reference build's bit for bit, for a ramp with a wedge
    and a tetrahedron with texture coordinates and normals, at several
    spacings."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "meshes.npz"))
    assert len(g.files) >= 4
    for key in g.files:
        mesh, sp = key.split("/")
        pts = sph_gb300.sample_mesh(os.path.join(MESH_DIR, mesh + ".obj"), float(sp) * 0.02 * 2.0)
        assert pts.shape == g[key].shape and np.array_equal(pts, g[key]), key


def test_mesh_sampler_rejects_bad_files(L, tmp_path):
    assert L.sph_sample_mesh(str(tmp_path / "none.obj").encode(), 0.04, None) == -1
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nf 1 2 3\n")
    assert L.sph_sample_mesh(str(bad).encode(), 0.04, None) == -1
    assert L.sph_sample_mesh(os.path.join(MESH_DIR, "ramp.obj").encode(), 0.0, None) == -1
    # a distance that would need more than 2^28 samples is refused before sampling
    assert L.sph_sample_mesh(os.path.join(MESH_DIR, "ramp.obj").encode(), 1e-9, None) == -1
    s = sph_gb300.Scene(method=2, boundary=1, radius=0.02)
    with pytest.raises(sph_gb300.SPHError, match="Akinci"):
        s.add_boundary_mesh(os.path.join(MESH_DIR, "ramp.obj"), 0.02)
    s.close()


def test_pool_capacity_from_an_hbm_budget(L):
    """sph_pool_desc_from_budget (host arithmetic only): one boundary particle
    and sixteen grid keys per fluid particle, about 1.5 KB per fluid particle
    at 64 pair-list slots, linear in the budget; budgets under 1 MiB are
    refused."""
    d = sph_gb300.PoolDesc()
    assert L.sph_pool_desc_from_budget(80 * 10**9, 64, ctypes.byref(d)) == 0
    assert d.max_boundary == d.max_particles and d.max_keys == 16 * d.max_particles
    assert d.neighbor_list_max == 64
    assert 1400 <= 80 * 10**9 / d.max_particles <= 1600
    d2 = sph_gb300.PoolDesc()
    assert L.sph_pool_desc_from_budget(160 * 10**9, 64, ctypes.byref(d2)) == 0
    assert abs(d2.max_particles - 2 * d.max_particles) <= 1
    d3 = sph_gb300.PoolDesc()
    assert L.sph_pool_desc_from_budget(80 * 10**9, 32, ctypes.byref(d3)) == 0
    assert d3.max_particles > d.max_particles          # fewer slots, more particles
    assert L.sph_pool_desc_from_budget(1000, 64, ctypes.byref(d3)) == -1
