"""Test oracles for the per-step SPH particle loop.

TEST INFRASTRUCTURE ONLY.  This package is the checker: it is imported by the
tests, by ``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg,
never by the product (``sph_gb300``).

Two oracles live here:

* ``liboracle.so`` (``sph_oracle.c``): the project's C restatement of the
  reference's solvers, FP64, in the reference's own evaluation order.  It
  builds on any host (``make -C oracle oracle``), with or without the
  reference tree.
* ``_ref/ref_parity`` / ``_ref/ref_timed``: the reference simulator's own
  sources compiled headless against the project's GLM shim, driven by
  ``ref_driver.cpp`` (``make -C oracle ref``).  It needs the reference tree,
  so it exists only where that tree is mounted; ``run_reference`` uses it to
  pin the restatement and to generate the golden fixtures in tests/golden/.
"""
from __future__ import annotations

import ctypes
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PARITY = os.path.join(HERE, "_ref", "ref_parity")
REF_TIMED = os.path.join(HERE, "_ref", "ref_timed")


class OrcParams(ctypes.Structure):
    _fields_ = [
        ("method", ctypes.c_int),
        ("boundary", ctypes.c_int),
        ("radius", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("dt", ctypes.c_double),
        ("min_dt", ctypes.c_double),
        ("max_dt", ctypes.c_double),
        ("fps", ctypes.c_double),
        ("density0", ctypes.c_double),
        ("stiffness", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("eta", ctypes.c_double),
        ("eta_v", ctypes.c_double),
        ("cfl", ctypes.c_double),
        ("min_it", ctypes.c_int),
        ("max_it", ctypes.c_int),
        ("min_it_v", ctypes.c_int),
        ("max_it_v", ctypes.c_int),
        ("visc_method", ctypes.c_int),
        ("visc", ctypes.c_double),
        ("bvisc", ctypes.c_double),
        ("st_method", ctypes.c_int),
        ("st", ctypes.c_double),
        ("adh_method", ctypes.c_int),
        ("adh", ctypes.c_double),
        ("cube_min", ctypes.c_double * 3),
        ("cube_max", ctypes.c_double * 3),
        ("has_cube", ctypes.c_int),
        ("bh_normal_fct", ctypes.c_double),
        ("bh_tang_fct", ctypes.c_double),
    ]


DEFAULTS = dict(
    method=2, boundary=2, radius=0.025, gravity=(0.0, -9.81, 0.0), dt=1e-4, min_dt=1e-5,
    max_dt=5e-3, fps=60.0, density0=1000.0, stiffness=1000.0, gamma=7.0, eta=0.001, eta_v=0.001,
    cfl=1.0, min_it=-1, max_it=-1, min_it_v=-1, max_it_v=-1, visc_method=-1, visc=0.0, bvisc=0.0,
    st_method=-1, st=0.0, adh_method=-1, adh=0.0, cube_min=(0.0, 0.0, 0.0), cube_max=(1.0, 1.0, 1.0),
    has_cube=0, bh_normal_fct=0.0, bh_tang_fct=1.0,
)

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
        os.path.getmtime(os.path.join(HERE, f)) for f in ("sph_oracle.c", "sph_oracle.h")
    ):
        subprocess.run(["make", "-C", HERE, "oracle"], check=True, capture_output=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = vp
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_fluid.argtypes = [vp, dp, dp, ctypes.c_uint]
        L.orc_add_box.argtypes = [vp, dp, dp]
        L.orc_add_sphere.argtypes = [vp, dp, ctypes.c_double]
        L.orc_add_points.argtypes = [vp, dp, ctypes.c_uint]
        L.orc_add_bh_box.argtypes = [vp, dp, dp, ctypes.c_int]
        L.orc_add_bh_sphere.argtypes = [vp, dp, ctypes.c_double, ctypes.c_int]
        L.orc_sample_bh_box.argtypes = [ctypes.c_double, dp, dp, ctypes.c_int, dp, dp]
        L.orc_sample_bh_box.restype = ctypes.c_longlong
        L.orc_perturb.argtypes = [vp, ctypes.c_double, ctypes.c_double, ctypes.c_ulonglong]
        L.orc_add_emitter.argtypes = [vp, ctypes.c_int, ctypes.c_uint, dp, ctypes.c_double, dp, ctypes.c_double,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_pause_emitters.argtypes = [vp, ctypes.c_int]
        L.orc_emitter_group.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
        L.orc_emitter_group.restype = ctypes.c_longlong
        L.orc_init.argtypes = [vp]
        L.orc_step.argtypes = [vp, ctypes.c_int]
        L.orc_num_fluid.argtypes = [vp]
        L.orc_num_fluid.restype = ctypes.c_uint
        L.orc_num_boundary.argtypes = [vp]
        L.orc_num_boundary.restype = ctypes.c_uint
        L.orc_get.argtypes = [vp, ctypes.c_char_p, dp]
        L.orc_get_scalar.argtypes = [vp, ctypes.c_char_p, dp]
        L.orc_neighbors.argtypes = [vp, ip, ip, ip, ip, ip, ip, ctypes.POINTER(ctypes.c_longlong)]
        L.orc_sample_box.argtypes = [ctypes.c_double, dp, dp, dp]
        L.orc_sample_box.restype = ctypes.c_longlong
        L.orc_sample_sphere.argtypes = [ctypes.c_double, dp, ctypes.c_double, dp]
        L.orc_sample_sphere.restype = ctypes.c_longlong
        L.orc_fluid_block.argtypes = [ctypes.c_double, dp, dp, dp]
        L.orc_fluid_block.restype = ctypes.c_longlong
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _iptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _vec3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(3))


def make_params(**kw) -> OrcParams:
    d = dict(DEFAULTS)
    for k, v in kw.items():
        if k not in d:
            raise KeyError(f"unknown oracle parameter {k}")
        d[k] = v
    p = OrcParams()
    for k, v in d.items():
        if k in ("gravity", "cube_min", "cube_max"):
            getattr(p, k)[:] = [float(t) for t in v]
        else:
            setattr(p, k, v)
    return p


def sample_bh_box(h, mn, mx, inverted=True):
    """PCISPHBoundaryModel::sampleCube: (points, normals)."""
    L = lib()
    mn, mx = _vec3(mn), _vec3(mx)
    n = L.orc_sample_bh_box(h, _dptr(mn), _dptr(mx), int(inverted), None, None)
    pts = np.zeros((n, 3))
    nrm = np.zeros((n, 3))
    L.orc_sample_bh_box(h, _dptr(mn), _dptr(mx), int(inverted), _dptr(pts), _dptr(nrm))
    return pts, nrm


def emitter_group(type, particle_radius, width, height=0.0):
    """Emitter::buildSquareGroup (type 0) / buildCircleGroup (type 1)."""
    L = lib()
    n = L.orc_emitter_group(int(type), float(particle_radius), float(width), float(height), None)
    out = np.zeros((n, 3))
    if n:
        L.orc_emitter_group(int(type), float(particle_radius), float(width), float(height), _dptr(out))
    return out


EMITTER_KEYS = ("type", "num", "position", "velocity", "rotation", "start", "width", "height", "spacing")


def _emitter_args(e):
    """An emitter dict (EMITTER_KEYS; rotation (w, x, y, z)) as flat values."""
    rot = e.get("rotation", (1.0, 0.0, 0.0, 0.0))
    return (int(e["type"]), int(e["num"]), [float(t) for t in e["position"]], float(e["velocity"]),
            [float(t) for t in rot], float(e.get("start", 0.0)), float(e.get("width", 0.0)),
            float(e.get("height", 0.0)), float(e.get("spacing", 1.0)))


def fluid_block(radius, mn, mx):
    """Lattice of Simulation::buildFluidBlock (spacing 2r from min + r)."""
    L = lib()
    mn, mx = _vec3(mn), _vec3(mx)
    n = L.orc_fluid_block(radius, _dptr(mn), _dptr(mx), None)
    out = np.zeros((n, 3))
    L.orc_fluid_block(radius, _dptr(mn), _dptr(mx), _dptr(out))
    return out


def sample_box(support_radius, mn, mx):
    L = lib()
    mn, mx = _vec3(mn), _vec3(mx)
    n = L.orc_sample_box(support_radius, _dptr(mn), _dptr(mx), None)
    out = np.zeros((n, 3))
    L.orc_sample_box(support_radius, _dptr(mn), _dptr(mx), _dptr(out))
    return out


def sample_sphere(particle_radius, c, radius):
    L = lib()
    c = _vec3(c)
    n = L.orc_sample_sphere(particle_radius, _dptr(c), radius, None)
    out = np.zeros((n, 3))
    L.orc_sample_sphere(particle_radius, _dptr(c), radius, _dptr(out))
    return out


class OracleScene:
    """One scene of the C restatement (one fluid model, one boundary model)."""

    def __init__(self, params: dict, x, v=None, boxes=(), spheres=(), points=None, bh_boxes=(), bh_spheres=(),
                 emitters=()):
        L = lib()
        self.params = dict(params)
        self._p = make_params(**params)
        self.h = L.orc_create(ctypes.byref(self._p))
        if not self.h:
            raise ValueError("oracle rejected the scene parameters")
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        v = np.zeros_like(x) if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        if L.orc_set_fluid(self.h, _dptr(x), _dptr(v), x.shape[0]) != 0:
            raise RuntimeError("orc_set_fluid failed")
        for e in emitters:
            t, num, pos, vel, rot, start, w, hgt, sp = _emitter_args(e)
            rot = np.array(rot)
            if L.orc_add_emitter(self.h, t, num, _dptr(_vec3(pos)), vel, _dptr(rot), start, w, hgt, sp) != 0:
                raise RuntimeError("orc_add_emitter failed")
        for mn, mx in boxes:
            L.orc_add_box(self.h, _dptr(_vec3(mn)), _dptr(_vec3(mx)))
        for c, r in spheres:
            L.orc_add_sphere(self.h, _dptr(_vec3(c)), float(r))
        for mn, mx, inv in bh_boxes:
            if L.orc_add_bh_box(self.h, _dptr(_vec3(mn)), _dptr(_vec3(mx)), int(inv)) != 0:
                raise RuntimeError("orc_add_bh_box failed (boundary must be 1)")
        for c, r, inv in bh_spheres:
            if L.orc_add_bh_sphere(self.h, _dptr(_vec3(c)), float(r), int(inv)) != 0:
                raise RuntimeError("orc_add_bh_sphere failed (boundary must be 1)")
        if points is not None and len(points):
            pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
            L.orc_add_points(self.h, _dptr(pts), pts.shape[0])
        if L.orc_init(self.h) != 0:
            raise RuntimeError("orc_init failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    @property
    def n(self):
        return lib().orc_num_fluid(self.h)

    @property
    def nb(self):
        return lib().orc_num_boundary(self.h)

    def step(self, n=1):
        if lib().orc_step(self.h, n) != 0:
            raise RuntimeError("orc_step failed")

    def get(self, field):
        vec = field in ("x", "v", "a", "pacc", "normal", "bx", "bn")
        count = self.nb if field in ("bx", "psi", "bn", "bdens", "bpress") else self.n
        out = np.zeros((count, 3) if vec else count)
        rc = lib().orc_get(self.h, field.encode(), _dptr(out))
        if rc != 0:
            raise KeyError(field)
        return out

    def pause_emitters(self, pause=True):
        if lib().orc_pause_emitters(self.h, int(bool(pause))) != 0:
            raise RuntimeError("orc_pause_emitters failed")

    def perturb(self, dx, dv, seed):
        """Test instrument: add U(-dx, dx) to positions, U(-dv, dv) to velocities."""
        if lib().orc_perturb(self.h, float(dx), float(dv), int(seed)) != 0:
            raise RuntimeError("orc_perturb failed")

    def scalar(self, name):
        out = ctypes.c_double()
        if lib().orc_get_scalar(self.h, name.encode(), ctypes.byref(out)) != 0:
            raise KeyError(name)
        return out.value

    def neighbors(self):
        """Per-particle neighbour sets (CSR) as the reference's walks see them."""
        L = lib()
        tot = (ctypes.c_longlong * 2)()
        L.orc_neighbors(self.h, None, None, None, None, None, None, tot)
        n = self.n
        cells = np.zeros(3 * n, np.int32)
        rank = np.zeros(n, np.int32)
        off = np.zeros(n + 1, np.int32)
        nbr = np.zeros(max(tot[0], 1), np.int32)
        boff = np.zeros(n + 1, np.int32)
        bnbr = np.zeros(max(tot[1], 1), np.int32)
        L.orc_neighbors(self.h, _iptr(cells), _iptr(rank), _iptr(off), _iptr(nbr), _iptr(boff), _iptr(bnbr), tot)
        return dict(cell=cells.reshape(n, 3), cell_rank=rank, nbr_off=off, nbr=nbr[: tot[0]],
                    bnbr_off=boff, bnbr=bnbr[: tot[1]])


# ---------------------------------------------------------------------------
# The reference itself (only where the reference tree has been built)
# ---------------------------------------------------------------------------

def reference_available(timed: bool = False) -> bool:
    return os.path.exists(REF_TIMED if timed else REF_PARITY)


def build_reference(ref_tree: str | None = None) -> bool:
    """Compile the reference headless into _ref/ with the Makefile's `ref`
    recipe.  The tree is `ref_tree`, else the environment's
    SPH_REFERENCE_TREE, else the recipe's default; where none holds the
    reference's sources nothing is built.  Returns whether the build exists."""
    # the reference's own build, and the GPU drop-in solvers built with it
    # (they link to sph_gb300/lib/libsph_gb300.so, built first)
    cmd = ["make", "-C", HERE, "ref", "adapter", "-j8"]
    if ref_tree:
        cmd.append(f"REF={ref_tree}")
    subprocess.run(cmd, check=True, capture_output=True)
    return reference_available()


def read_dump(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            hdr = f.read(48)
            if len(hdr) < 48:
                break
            name = hdr.split(b"\0", 1)[0].decode()
            t = f.read(1)
            (count,) = struct.unpack("<Q", f.read(8))
            dt = {b"d": np.float64, b"i": np.int32, b"u": np.uint32}[t]
            arr = np.frombuffer(f.read(count * np.dtype(dt).itemsize), dtype=dt).copy()
            out[name] = arr
    return out


def read_frames(directory, stem="scene"):
    """Frame files SceneLoader::writeFluid wrote next to `stem`.json, as
    arrays: frame{N}.positions / .velocities (flat xyz), .time, .timeStep,
    .numParticles, .numActiveParticles, and .raw (the file's bytes)."""
    import glob
    import json

    out = {}
    for path in sorted(glob.glob(os.path.join(directory, f"{stem}_*.json"))):
        num = int(os.path.basename(path)[len(stem) + 1:-5])
        raw = open(path, "rb").read()
        st = json.loads(raw)
        tag = f"frame{num}"
        for key in ("positions", "velocities"):
            out[f"{tag}.{key}"] = np.asarray(st.get(key, []), dtype=np.float64).ravel()
        for key in ("time", "timeStep", "numParticles", "numActiveParticles"):
            out[f"{tag}.{key}"] = np.array([st[key]], dtype=np.float64)
        out[f"{tag}.raw"] = np.frombuffer(raw, dtype=np.uint8).copy()
    return out


def run_reference_json(scene: dict, steps=1, dump_every=1, dump_neighbors=False, save=False, workdir=None):
    """Run the reference's own scene-file path (Simulation::importScene on
    `scene` written as JSON) and return its dump plus, with save, the frame
    files SceneLoader::writeFluid wrote (see read_frames)."""
    import json

    if not os.path.exists(REF_PARITY):
        raise FileNotFoundError(REF_PARITY)
    with tempfile.TemporaryDirectory(dir=workdir) as td:
        path = os.path.join(td, "scene.json")
        with open(path, "w") as f:
            json.dump(scene, f)
        out = os.path.join(td, "out.bin")
        spec = os.path.join(td, "spec.txt")
        with open(spec, "w") as f:
            f.write(f"json {path}\nout {out}\nsteps {steps}\ndump_every {dump_every}\n"
                    f"dump_neighbors {int(dump_neighbors)}\nsave {int(save)}\n")
        env = dict(os.environ, OMP_NUM_THREADS="1")
        with open(os.devnull, "rb") as devnull_in, open(os.devnull, "wb") as devnull_out:
            subprocess.run([REF_PARITY, spec], stdin=devnull_in, stdout=devnull_out, env=env, check=True, cwd=td)
        res = read_dump(out)
        res.update(read_frames(td))
        return res


def run_reference(params: dict, x, v=None, boxes=(), spheres=(), steps=1, dump_neighbors=False,
                  dump_every=1, timed=False, threads=1, workdir=None, bh_boxes=(), bh_spheres=(), emitters=(),
                  geometries=()):
    """Run the reference's own solver on the scene and return its dump."""
    exe = REF_TIMED if timed else REF_PARITY
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    d = dict(DEFAULTS)
    d.update(params)
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
    v = np.zeros_like(x) if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
    with tempfile.TemporaryDirectory(dir=workdir) as td:
        fluid = os.path.join(td, "fluid.bin")
        with open(fluid, "wb") as f:
            f.write(struct.pack("<Q", x.shape[0]))
            f.write(x.tobytes())
            f.write(v.tobytes())
        out = os.path.join(td, "out.bin")
        lines = [
            f"method {d['method']}", f"boundary {d['boundary']}", f"radius {d['radius']!r}",
            "gravity " + " ".join(repr(float(t)) for t in d["gravity"]),
            f"dt {d['dt']!r}", f"min_dt {d['min_dt']!r}", f"max_dt {d['max_dt']!r}", f"fps {d['fps']!r}",
            f"density0 {d['density0']!r}", f"stiffness {d['stiffness']!r}", f"gamma {d['gamma']!r}",
            f"eta {d['eta']!r}", f"eta_v {d['eta_v']!r}", f"cfl {d['cfl']!r}",
            f"min_it {d['min_it']}", f"max_it {d['max_it']}", f"min_it_v {d['min_it_v']}",
            f"max_it_v {d['max_it_v']}", f"visc_method {d['visc_method']}", f"visc {d['visc']!r}",
            f"bvisc {d['bvisc']!r}", f"st_method {d['st_method']}", f"st {d['st']!r}",
            f"adh_method {d['adh_method']}", f"adh {d['adh']!r}",
            f"fluid {fluid}", f"out {out}", f"steps {steps}", f"dump_neighbors {int(dump_neighbors)}",
            f"dump_every {dump_every}",
            f"bh_normal_fct {d['bh_normal_fct']!r}", f"bh_tang_fct {d['bh_tang_fct']!r}",
        ]
        if d["has_cube"]:
            lines.append("cube " + " ".join(repr(float(t)) for t in list(d["cube_min"]) + list(d["cube_max"])))
        for mn, mx in boxes:
            lines.append("box " + " ".join(repr(float(t)) for t in list(mn) + list(mx)))
        for c, r in spheres:
            lines.append("sphere " + " ".join(repr(float(t)) for t in list(c) + [r]))
        for mn, mx, inv in bh_boxes:
            lines.append("bh_box " + " ".join(repr(float(t)) for t in list(mn) + list(mx)) + f" {int(inv)}")
        for c, r, inv in bh_spheres:
            lines.append("bh_sphere " + " ".join(repr(float(t)) for t in list(c) + [r]) + f" {int(inv)}")
        for path, spacing in geometries:
            lines.append(f"geometry {os.path.abspath(path)} {float(spacing)!r}")
        for e in emitters:
            t, num, pos, vel, rot, start, w, hgt, sp = _emitter_args(e)
            lines.append("emitter " + " ".join([str(t), str(num)] + [repr(float(q)) for q in list(pos) + [vel] + list(rot)
                                                                     + [start, w, hgt, sp]]))
        scene = os.path.join(td, "scene.txt")
        with open(scene, "w") as f:
            f.write("\n".join(lines) + "\n")
        env = dict(os.environ, OMP_NUM_THREADS=str(threads))
        with open(os.devnull, "rb") as devnull_in, open(os.devnull, "wb") as devnull_out:
            subprocess.run([exe, scene], stdin=devnull_in, stdout=devnull_out, env=env, check=True)
        return read_dump(out)
