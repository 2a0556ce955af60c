"""sph_ctx_download_noalloc: the field download for callers that cannot
allocate device memory (a frame-export hook in a serving process whose device
memory is fully reserved, or a real-time driver that must not call cudaFree,
which waits for the whole device).  It stages through a fixed 4 MiB device
array in the library instead of a per-call cudaMalloc.

Checked through the C ABI against sph_ctx_download (same conversion, so the
results must be identical), on two calls in a row, and for the size limit.
Kept in a file of its own, collected last."""
import ctypes

import numpy as np
import pytest

import sph_gb300
from scenes import scene

pytestmark = pytest.mark.gpu

LIMIT = 524288


def build(name, precision):
    params, x, boxes, spheres = scene(name)
    s = sph_gb300.Scene(precision=precision, **params)
    s.set_fluid(x)
    for mn, mx in boxes:
        s.add_boundary_box(mn, mx)
    for c, r in spheres:
        s.add_boundary_sphere(c, r)
    s.init()
    return s


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_noalloc_download_matches_download_on_two_calls(gpu_lib, precision):
    s = build("dfsph_forces", precision)
    s.step(2)
    # two calls in a row, different fields, then the first field again
    for field in ("x", "rho", "x"):
        a = s.get(field)
        b = s.get_noalloc(field)
        assert np.array_equal(a, b), field
    s.step(1)
    for field in ("v", "bx"):
        assert np.array_equal(s.get(field), s.get_noalloc(field)), field


def test_noalloc_download_rejects_fields_over_the_limit(gpu_lib):
    n = LIMIT // 3 + 1000          # 3-component field just over the limit
    side = int(np.ceil(n ** (1 / 3)))
    r = 0.002
    s = sph_gb300.Scene(method=2, boundary=0, radius=r, has_cube=1, cube_min=(0, 0, 0),
                        cube_max=(side * 2 * r + 0.01,) * 3, precision="f32")
    s.add_fluid_block((0, 0, 0), (side * 2 * r, side * 2 * r, side * 2 * r))
    s.init()
    assert 3 * s.n > LIMIT
    out = np.zeros((s.n, 3))
    rc = sph_gb300.lib().sph_ctx_download_noalloc(s._h, 0, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == -4
    assert b"at most" in sph_gb300.lib().sph_ctx_last_error(s._h)
    # scalar field of the same scene fits
    assert np.array_equal(s.get_noalloc("rho"), s.get("rho"))
