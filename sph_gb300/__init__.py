"""sph_gb300: GB300 (sm_103a) per-step SPH particle loop behind a C ABI.

This module is a thin ctypes layer over ``lib/libsph_gb300.so`` (declared in
``include/sph_gb300.h``).  All computation happens in the library's CUDA
kernels; if the library is missing or fails to load, every entry point raises
-- there is no CPU fallback.

Vocabulary follows the reference simulator (josemanuel28v/SPH):
``Scene`` bundles what the reference's ``Simulation`` singleton holds for one
fluid model and one boundary model -- ``add_fluid_block`` is
``Simulation::buildFluidBlock``, ``add_boundary_box`` / ``add_boundary_sphere``
are ``AkinciBoundaryModel::addCube`` / ``addSphere``, ``init`` is
``Simulation::init`` and ``step`` is ``Simulation::step``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsph_gb300.so")

# Method ids (src/Simulation.cpp:21-43 of the reference)
WCSPH, PCISPH, DFSPH = 0, 1, 2
BOUNDARY_CUBE, BOUNDARY_PCISPH, BOUNDARY_AKINCI = 0, 1, 2
VISCOSITY_STANDARD, VISCOSITY_ARTIFICIAL, VISCOSITY_XSPH = 0, 1, 2
SURFACE_TENSION_AKINCI, ADHESION_AKINCI = 3, 4
PRECISION_F32, PRECISION_F64 = 0, 1

FIELDS = {
    "x": (0, 3), "v": (1, 3), "a": (2, 3), "rho": (3, 1), "p": (4, 1), "alpha": (5, 1), "pred": (6, 1),
    "div": (7, 1), "k": (8, 1), "kv": (9, 1), "pacc": (10, 3), "normal": (11, 3), "bx": (12, 3), "psi": (13, 1),
    "bdens": (14, 1), "bpress": (15, 1),
}

STATUS_OUT_OF_GRID, STATUS_NONFINITE, STATUS_ITER_CAP, STATUS_ITER_CAP_V, STATUS_DIVERGED = 1, 2, 4, 8, 16
STATUS_BOUNDS = 32  # bounds-checked build only
ERR_CAPACITY = -4   # SPH_ERR_CAPACITY


def _phases(fn, handle, check, what):
    """Parse "name<TAB>count<TAB>total_ms" lines of a phase profile."""
    buf = ctypes.create_string_buffer(1 << 14)
    n = fn(handle, buf, len(buf))
    if n < 0:
        check(n, what)
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split("\t")
        out[name] = (int(cnt), float(ms))
    return out


class SceneDesc(ctypes.Structure):
    _fields_ = [
        ("simulation_method", ctypes.c_int),
        ("boundary_method", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("particle_radius", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("time_step", ctypes.c_double),
        ("min_time_step", ctypes.c_double),
        ("max_time_step", ctypes.c_double),
        ("fps", ctypes.c_double),
        ("density0", ctypes.c_double),
        ("stiffness", ctypes.c_double),
        ("gamma", ctypes.c_double),
        ("max_error", ctypes.c_double),
        ("max_error_v", ctypes.c_double),
        ("cfl_factor", ctypes.c_double),
        ("min_iterations", ctypes.c_int),
        ("max_iterations", ctypes.c_int),
        ("min_iterations_v", ctypes.c_int),
        ("max_iterations_v", ctypes.c_int),
        ("viscosity_method", ctypes.c_int),
        ("viscosity", ctypes.c_double),
        ("boundary_viscosity", ctypes.c_double),
        ("surface_tension_method", ctypes.c_int),
        ("surface_tension", ctypes.c_double),
        ("adhesion_method", ctypes.c_int),
        ("adhesion", ctypes.c_double),
        ("has_cube", ctypes.c_int),
        ("cube_min", ctypes.c_double * 3),
        ("cube_max", ctypes.c_double * 3),
        ("domain_min", ctypes.c_double * 3),
        ("domain_max", ctypes.c_double * 3),
        ("threads_per_particle", ctypes.c_int),
        ("neighbor_list_max", ctypes.c_int),
        ("bh_normal_fct", ctypes.c_double),
        ("bh_tangential_fct", ctypes.c_double),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("time", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("avg_density_error", ctypes.c_double),
        ("avg_divergence_error", ctypes.c_double),
        ("max_density_error", ctypes.c_double),
        ("max_velocity", ctypes.c_double),
        ("iterations", ctypes.c_uint),
        ("iterations_v", ctypes.c_uint),
        ("steps", ctypes.c_uint),
        ("status", ctypes.c_uint),
        ("sum_iterations", ctypes.c_ulonglong),
        ("sum_iterations_v", ctypes.c_ulonglong),
        ("num_fluid", ctypes.c_uint),
        ("num_boundary", ctypes.c_uint),
        ("list_pairs", ctypes.c_ulonglong),
        ("list_overflow", ctypes.c_uint),
        ("num_fluid_total", ctypes.c_uint),
        ("grid_growths", ctypes.c_uint),
    ]


class PoolDesc(ctypes.Structure):
    _fields_ = [
        ("max_particles", ctypes.c_ulonglong),
        ("max_boundary", ctypes.c_ulonglong),
        ("max_keys", ctypes.c_ulonglong),
        ("max_scenes", ctypes.c_uint),
        ("neighbor_list_max", ctypes.c_int),
    ]


class PoolTuning(ctypes.Structure):
    _fields_ = [
        ("build_block", ctypes.c_int),
        ("build_occupancy", ctypes.c_int),
        ("queue_depth", ctypes.c_int),
        ("solver_block", ctypes.c_int),
        ("solver_occupancy", ctypes.c_int),
        ("scan_width", ctypes.c_int),
        ("source", ctypes.c_int),
        ("steps_left", ctypes.c_int),
    ]


class ServerDesc(ctypes.Structure):
    _fields_ = [("epoch_steps", ctypes.c_uint), ("lookahead", ctypes.c_uint), ("keep_results", ctypes.c_int),
                ("max_queued_bytes", ctypes.c_ulonglong)]


class RequestInfo(ctypes.Structure):
    _fields_ = [
        ("id", ctypes.c_longlong),
        ("state", ctypes.c_int),
        ("num_fluid", ctypes.c_uint),
        ("steps", ctypes.c_uint),
        ("steps_done", ctypes.c_uint),
        ("status", ctypes.c_uint),
        ("latency_s", ctypes.c_double),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_ulonglong),
        ("admitted", ctypes.c_ulonglong),
        ("completed", ctypes.c_ulonglong),
        ("failed", ctypes.c_ulonglong),
        ("queued", ctypes.c_ulonglong),
        ("resident", ctypes.c_ulonglong),
        ("epochs", ctypes.c_ulonglong),
        ("wall_s", ctypes.c_double),
        ("particle_steps", ctypes.c_double),
        ("particle_steps_per_s", ctypes.c_double),
        ("p50_latency_s", ctypes.c_double),
        ("p99_latency_s", ctypes.c_double),
        ("mean_latency_s", ctypes.c_double),
        ("rejected", ctypes.c_ulonglong),
        ("queued_bytes", ctypes.c_ulonglong),
    ]


REQUEST_QUEUED, REQUEST_RESIDENT, REQUEST_DONE, REQUEST_FAILED = 0, 1, 2, 3

# The C ABI, as (name, restype, argtypes); the CPU tests check that the
# library exports each of these.
_vp, _dp, _ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
ABI = [
    ("sph_scene_desc_init", ctypes.c_int, [ctypes.POINTER(SceneDesc)]),
    ("sph_ctx_create", ctypes.c_int, [ctypes.POINTER(SceneDesc), ctypes.POINTER(_vp)]),
    ("sph_ctx_destroy", ctypes.c_int, [_vp]),
    ("sph_ctx_set_fluid", ctypes.c_int, [_vp, _dp, _dp, ctypes.c_uint]),
    ("sph_ctx_add_fluid_block", ctypes.c_int, [_vp, _dp, _dp]),
    ("sph_ctx_add_boundary_box", ctypes.c_int, [_vp, _dp, _dp]),
    ("sph_ctx_add_boundary_sphere", ctypes.c_int, [_vp, _dp, ctypes.c_double]),
    ("sph_ctx_add_boundary_points", ctypes.c_int, [_vp, _dp, ctypes.c_uint]),
    ("sph_ctx_add_pcisph_box", ctypes.c_int, [_vp, _dp, _dp, ctypes.c_int]),
    ("sph_ctx_add_pcisph_sphere", ctypes.c_int, [_vp, _dp, ctypes.c_double, ctypes.c_int]),
    ("sph_ctx_add_pcisph_points", ctypes.c_int, [_vp, _dp, _dp, ctypes.c_uint]),
    ("sph_ctx_add_emitter", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_uint, _dp, ctypes.c_double, _dp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    ("sph_ctx_pause_emitters", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_ctx_add_boundary_mesh", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double]),
    ("sph_sample_mesh", ctypes.c_longlong, [ctypes.c_char_p, ctypes.c_double, _dp]),
    ("sph_ctx_load_scene", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(SceneDesc), ctypes.POINTER(_vp)]),
    ("sph_ctx_import_scene", ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(SceneDesc), ctypes.POINTER(_vp)]),
    ("sph_scene_load_error", ctypes.c_char_p, []),
    ("sph_ctx_get_desc", ctypes.c_int, [_vp, ctypes.POINTER(SceneDesc)]),
    ("sph_ctx_set_time_window", ctypes.c_int, [_vp, ctypes.c_double, ctypes.c_double]),
    ("sph_ctx_set_frame_output", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int]),
    ("sph_ctx_get_frame", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint)]),
    ("sph_ctx_write_frame", ctypes.c_int, [_vp, ctypes.c_char_p]),
    ("sph_ctx_run", ctypes.c_int, [_vp, ctypes.c_ulonglong, ctypes.POINTER(ctypes.c_ulonglong)]),
    ("sph_ctx_init", ctypes.c_int, [_vp]),
    ("sph_ctx_step", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_ctx_step_timed", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    ("sph_ctx_synchronize", ctypes.c_int, [_vp]),
    ("sph_ctx_set_graph", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_ctx_set_grid_growth", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_ctx_num_particles", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint), ctypes.POINTER(ctypes.c_uint)]),
    ("sph_ctx_download", ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    ("sph_ctx_download_noalloc", ctypes.c_int, [_vp, ctypes.c_int, _dp]),
    ("sph_ctx_get_stats", ctypes.c_int, [_vp, ctypes.POINTER(Stats)]),
    ("sph_ctx_last_error", ctypes.c_char_p, [_vp]),
    ("sph_ctx_neighbors", ctypes.c_int, [_vp, _ip, _ip, _ip, _ip, _ip, _ip, ctypes.POINTER(ctypes.c_longlong)]),
    ("sph_ctx_pair_lists", ctypes.c_int, [_vp, _ip, _ip, _ip, ctypes.POINTER(ctypes.c_longlong)]),
    ("sph_ctx_get_launch_count", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
    ("sph_ctx_set_profiling", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_ctx_get_profile", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_ulonglong]),
    ("sph_ctx_get_phase_profile", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_ulonglong]),
    ("sph_select_device", ctypes.c_int, [ctypes.c_int]),
    ("sph_sample_box", ctypes.c_longlong, [ctypes.c_double, _dp, _dp, _dp]),
    ("sph_sample_sphere", ctypes.c_longlong, [ctypes.c_double, _dp, ctypes.c_double, _dp]),
    ("sph_sample_pcisph_box", ctypes.c_longlong, [ctypes.c_double, _dp, _dp, ctypes.c_int, _dp, _dp]),
    ("sph_fluid_block", ctypes.c_longlong, [ctypes.c_double, _dp, _dp, _dp]),
    ("sph_emitter_group", ctypes.c_longlong, [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp]),
    ("sph_version", ctypes.c_char_p, []),
    ("sph_pool_desc_from_budget", ctypes.c_int, [ctypes.c_ulonglong, ctypes.c_int, ctypes.POINTER(PoolDesc)]),
    ("sph_pool_create", ctypes.c_int, [ctypes.POINTER(PoolDesc), ctypes.POINTER(_vp)]),
    ("sph_pool_destroy", ctypes.c_int, [_vp]),
    ("sph_pool_add_scene", ctypes.c_int, [_vp, ctypes.POINTER(SceneDesc), _dp, _dp, ctypes.c_uint, _dp, ctypes.c_uint,
                                          ctypes.c_uint, ctypes.POINTER(ctypes.c_int)]),
    ("sph_pool_remove_scene", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_pool_step", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_pool_set_graph", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_pool_synchronize", ctypes.c_int, [_vp]),
    ("sph_pool_query", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(Stats), ctypes.POINTER(ctypes.c_int)]),
    ("sph_pool_poll", ctypes.c_int, [_vp, _ip, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    ("sph_pool_download", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _dp]),
    ("sph_pool_usage", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_ulonglong),
                                      ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_uint)]),
    ("sph_pool_get_launch_count", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
    ("sph_pool_step_timed", ctypes.c_int, [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_float)]),
    ("sph_pool_set_profiling", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_pool_get_profile", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_ulonglong]),
    ("sph_pool_get_phase_profile", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_ulonglong]),
    ("sph_pool_set_autotune", ctypes.c_int, [_vp, ctypes.c_int]),
    ("sph_pool_get_tuning", ctypes.c_int, [_vp, ctypes.POINTER(PoolTuning)]),
    ("sph_pool_set_tuning", ctypes.c_int, [_vp, ctypes.POINTER(PoolTuning)]),
    ("sph_pool_get_tuning_log", ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_ulonglong]),
    ("sph_pool_list_pairs", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_ulonglong), ctypes.POINTER(ctypes.c_uint)]),
    ("sph_pool_count_work", ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_ulonglong)]),
    ("sph_pool_pair_lists", ctypes.c_int, [_vp, ctypes.c_int, _ip, _ip, _ip, ctypes.POINTER(ctypes.c_longlong)]),
    ("sph_pool_snapshot", ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_void_p, ctypes.c_ulonglong,
                                         ctypes.POINTER(ctypes.c_ulonglong)]),
    ("sph_pool_restore", ctypes.c_int, [_vp, ctypes.c_void_p, ctypes.c_ulonglong, ctypes.c_uint,
                                        ctypes.POINTER(ctypes.c_int)]),
    ("sph_pool_last_error", ctypes.c_char_p, [_vp]),
    ("sph_server_desc_init", ctypes.c_int, [ctypes.POINTER(ServerDesc)]),
    ("sph_server_create", ctypes.c_int, [_vp, ctypes.POINTER(ServerDesc), ctypes.POINTER(_vp)]),
    ("sph_server_destroy", ctypes.c_int, [_vp]),
    ("sph_server_submit", ctypes.c_int, [_vp, ctypes.POINTER(SceneDesc), _dp, _dp, ctypes.c_uint, _dp, ctypes.c_uint,
                                         ctypes.c_uint, ctypes.POINTER(ctypes.c_longlong)]),
    ("sph_server_completed", ctypes.c_int, [_vp, ctypes.POINTER(RequestInfo), ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    ("sph_server_query", ctypes.c_int, [_vp, ctypes.c_longlong, ctypes.POINTER(RequestInfo)]),
    ("sph_server_fetch", ctypes.c_int, [_vp, ctypes.c_longlong, ctypes.c_int, _dp]),
    ("sph_server_release", ctypes.c_int, [_vp, ctypes.c_longlong]),
    ("sph_server_drain", ctypes.c_int, [_vp, ctypes.c_double, ctypes.POINTER(ctypes.c_int)]),
    ("sph_server_get_stats", ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    ("sph_server_last_error", ctypes.c_char_p, [_vp]),
]

_lib = None


class SPHError(RuntimeError):
    pass


def build(verbose: bool = False, force: bool = False) -> str:
    from . import buildlib as _b

    return _b.build(verbose=verbose, force=force)


def lib():
    """Load the CUDA library (raises if it is missing: no fallback).
    SPH_GB300_LIBRARY names another build of it (the bounds-checked one)."""
    global _lib
    if _lib is None:
        path = os.environ.get("SPH_GB300_LIBRARY") or LIB_PATH
        if not os.path.exists(path):
            raise SPHError(f"{path} is missing; build it with sph_gb300.build()")
        L = ctypes.CDLL(path)
        for name, res, args in ABI:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _v3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(3))


# parameter names shared with the oracle's scene parameters
_PARAM_MAP = {
    "method": "simulation_method", "boundary": "boundary_method", "radius": "particle_radius",
    "dt": "time_step", "min_dt": "min_time_step", "max_dt": "max_time_step", "fps": "fps",
    "density0": "density0", "stiffness": "stiffness", "gamma": "gamma", "eta": "max_error",
    "eta_v": "max_error_v", "cfl": "cfl_factor", "min_it": "min_iterations", "max_it": "max_iterations",
    "min_it_v": "min_iterations_v", "max_it_v": "max_iterations_v", "visc_method": "viscosity_method",
    "visc": "viscosity", "bvisc": "boundary_viscosity", "st_method": "surface_tension_method",
    "st": "surface_tension", "adh_method": "adhesion_method", "adh": "adhesion", "has_cube": "has_cube",
    "precision": "precision", "threads_per_particle": "threads_per_particle",
    "neighbor_list_max": "neighbor_list_max", "bh_normal_fct": "bh_normal_fct", "bh_tang_fct": "bh_tangential_fct",
}
_VEC = {"gravity", "cube_min", "cube_max", "domain_min", "domain_max"}


def make_desc(**params) -> SceneDesc:
    d = SceneDesc()
    lib().sph_scene_desc_init(ctypes.byref(d))
    for k, v in params.items():
        if k in _VEC:
            getattr(d, k)[:] = [float(t) for t in v]
            continue
        name = _PARAM_MAP.get(k, k)
        if not hasattr(d, name):
            raise KeyError(f"unknown scene parameter {k}")
        if k == "precision" and isinstance(v, str):
            v = PRECISION_F64 if v in ("f64", "fp64", "double") else PRECISION_F32
        setattr(d, name, v)
    return d


class Scene:
    """One device-resident scene (one fluid model, one boundary model)."""

    def __init__(self, **params):
        L = lib()
        self._desc = make_desc(**params)
        self._h = ctypes.c_void_p()
        rc = L.sph_ctx_create(ctypes.byref(self._desc), ctypes.byref(self._h))
        if rc != 0:
            raise SPHError(f"sph_ctx_create failed ({rc})")
        self._inited = False

    @classmethod
    def load(cls, path, init=True, **params):
        """A scene file (Simulation::importScene): the reference's settings,
        fluid blocks, emitters and boundary shapes from the JSON file at
        `path`; `params` set this library's own (precision,
        threads_per_particle, neighbor_list_max, domain_min/max).  With
        init=False the scene is returned before sph_ctx_init."""
        L = lib()
        self = cls.__new__(cls)
        self._desc = make_desc(**params)
        self._h = ctypes.c_void_p()
        fn = L.sph_ctx_import_scene if init else L.sph_ctx_load_scene
        rc = fn(os.fsencode(path), ctypes.byref(self._desc), ctypes.byref(self._h))
        if rc != 0:
            msg = L.sph_scene_load_error()
            raise SPHError(f"loading {path} failed ({rc}): {msg.decode() if msg else ''}")
        L.sph_ctx_get_desc(self._h, ctypes.byref(self._desc))
        self._inited = bool(init)
        return self

    def desc(self) -> dict:
        d = SceneDesc()
        self._check(lib().sph_ctx_get_desc(self._h, ctypes.byref(d)), "sph_ctx_get_desc")
        out = {}
        for name, _ in SceneDesc._fields_:
            v = getattr(d, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out

    def set_time_window(self, start, end):
        self._check(lib().sph_ctx_set_time_window(self._h, float(start), float(end)), "sph_ctx_set_time_window")

    def set_frame_output(self, scene_path=None, active=True):
        """Simulation::activateSave: write frame files named after scene_path."""
        p = None if scene_path is None else os.fsencode(scene_path)
        self._check(lib().sph_ctx_set_frame_output(self._h, p, int(bool(active))), "sph_ctx_set_frame_output")

    @property
    def frame(self):
        f = ctypes.c_uint()
        self._check(lib().sph_ctx_get_frame(self._h, ctypes.byref(f)), "sph_ctx_get_frame")
        return f.value

    def write_frame(self, path):
        """SceneLoader::writeFluid to `path`."""
        self._check(lib().sph_ctx_write_frame(self._h, os.fsencode(path)), "sph_ctx_write_frame")

    def run(self, max_steps=2**63):
        """Simulation::run: step while the time is inside the window (at most max_steps)."""
        done = ctypes.c_ulonglong()
        self._check(lib().sph_ctx_run(self._h, int(max_steps), ctypes.byref(done)), "sph_ctx_run")
        return done.value

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sph_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            msg = lib().sph_ctx_last_error(self._h)
            raise SPHError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    # -- construction -------------------------------------------------------
    def set_fluid(self, x, v=None):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        self._check(lib().sph_ctx_set_fluid(self._h, _d(x), None if vv is None else _d(vv), x.shape[0]),
                    "sph_ctx_set_fluid")
        return self

    def add_fluid_block(self, mn, mx):
        self._check(lib().sph_ctx_add_fluid_block(self._h, _d(_v3(mn)), _d(_v3(mx))), "sph_ctx_add_fluid_block")
        return self

    def add_boundary_box(self, mn, mx):
        self._check(lib().sph_ctx_add_boundary_box(self._h, _d(_v3(mn)), _d(_v3(mx))), "sph_ctx_add_boundary_box")
        return self

    def add_boundary_sphere(self, c, radius):
        self._check(lib().sph_ctx_add_boundary_sphere(self._h, _d(_v3(c)), float(radius)),
                    "sph_ctx_add_boundary_sphere")
        return self

    def add_pcisph_box(self, mn, mx, inverted=True):
        self._check(lib().sph_ctx_add_pcisph_box(self._h, _d(_v3(mn)), _d(_v3(mx)), int(bool(inverted))),
                    "sph_ctx_add_pcisph_box")
        return self

    def add_pcisph_sphere(self, c, radius, inverted=False):
        self._check(lib().sph_ctx_add_pcisph_sphere(self._h, _d(_v3(c)), float(radius), int(bool(inverted))),
                    "sph_ctx_add_pcisph_sphere")
        return self

    def add_boundary_mesh(self, obj_path, max_distance):
        """AkinciBoundaryModel::addGeometry: an OBJ mesh's surface samples as boundary points."""
        self._check(lib().sph_ctx_add_boundary_mesh(self._h, os.fsencode(obj_path), float(max_distance)),
                    "sph_ctx_add_boundary_mesh")
        return self

    def add_emitter(self, type, num_particles, position, velocity, rotation=(1.0, 0.0, 0.0, 0.0), start_time=0.0,
                    width=0.0, height=0.0, spacing=1.0):
        """FluidModel::addEmitter: type EMITTER_SQUARE (0) or EMITTER_CIRCLE (1);
        rotation is the unit quaternion (w, x, y, z)."""
        q = np.ascontiguousarray(np.asarray(rotation, dtype=np.float64).reshape(4))
        self._check(lib().sph_ctx_add_emitter(self._h, int(type), int(num_particles), _d(_v3(position)), float(velocity),
                                              _d(q), float(start_time), float(width), float(height), float(spacing)),
                    "sph_ctx_add_emitter")
        return self

    def pause_emitters(self, pause=True):
        """Simulation::setEmittersPause: pause or resume every emitter (both restart its clock now)."""
        self._check(lib().sph_ctx_pause_emitters(self._h, int(bool(pause))), "sph_ctx_pause_emitters")

    def add_boundary_points(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        self._check(lib().sph_ctx_add_boundary_points(self._h, _d(x), x.shape[0]), "sph_ctx_add_boundary_points")
        return self

    def init(self):
        self._check(lib().sph_ctx_init(self._h), "sph_ctx_init")
        self._inited = True
        return self

    # -- running ------------------------------------------------------------
    def step(self, n=1):
        self._check(lib().sph_ctx_step(self._h, int(n)), "sph_ctx_step")

    def step_timed(self, n=1):
        """Run n steps; return their device time in ms (CUDA events)."""
        ms = ctypes.c_float()
        self._check(lib().sph_ctx_step_timed(self._h, int(n), ctypes.byref(ms)), "sph_ctx_step_timed")
        return ms.value

    def synchronize(self):
        self._check(lib().sph_ctx_synchronize(self._h), "sph_ctx_synchronize")

    def set_graph(self, enable=True):
        self._check(lib().sph_ctx_set_graph(self._h, int(bool(enable))), "sph_ctx_set_graph")

    def set_grid_growth(self, enable=True):
        """Grow the grid box when particles leave it (the default), or keep it
        fixed (particles outside stay in its border cells)."""
        self._check(lib().sph_ctx_set_grid_growth(self._h, int(bool(enable))), "sph_ctx_set_grid_growth")

    # -- results ------------------------------------------------------------
    def counts(self):
        nf, nb = ctypes.c_uint(), ctypes.c_uint()
        lib().sph_ctx_num_particles(self._h, ctypes.byref(nf), ctypes.byref(nb))
        return nf.value, nb.value

    @property
    def n(self):
        return self.counts()[0]

    @property
    def nb(self):
        return self.counts()[1]

    def get(self, field):
        fid, width = FIELDS[field]
        count = self.nb if field in ("bx", "psi", "bdens", "bpress") else self.n
        out = np.zeros((count, 3) if width == 3 else count)
        if count:
            self._check(lib().sph_ctx_download(self._h, fid, _d(out)), f"sph_ctx_download({field})")
        return out

    def get_noalloc(self, field):
        """get() through sph_ctx_download_noalloc (fixed device staging array)."""
        fid, width = FIELDS[field]
        count = self.nb if field in ("bx", "psi", "bdens", "bpress") else self.n
        out = np.zeros((count, 3) if width == 3 else count)
        if count:
            self._check(lib().sph_ctx_download_noalloc(self._h, fid, _d(out)), f"sph_ctx_download_noalloc({field})")
        return out

    def stats(self) -> dict:
        s = Stats()
        self._check(lib().sph_ctx_get_stats(self._h, ctypes.byref(s)), "sph_ctx_get_stats")
        return {name: getattr(s, name) for name, _ in Stats._fields_}

    def launch_count(self):
        n = ctypes.c_ulonglong()
        self._check(lib().sph_ctx_get_launch_count(self._h, ctypes.byref(n)), "sph_ctx_get_launch_count")
        return n.value

    def set_profiling(self, enable=True):
        self._check(lib().sph_ctx_set_profiling(self._h, int(bool(enable))), "sph_ctx_set_profiling")

    def profile(self):
        """{kernel name: (launches, total ms)} since the previous call."""
        buf = ctypes.create_string_buffer(1 << 16)
        n = lib().sph_ctx_get_profile(self._h, buf, len(buf))
        if n < 0:
            self._check(n, "sph_ctx_get_profile")
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split()
            out[name] = (int(cnt), float(ms))
        return out

    def phase_profile(self):
        """{phase name: (count, total ms)} since the previous call, under the
        reference's phase-timer names (profiling on, host-driven steps; a
        graph step is one "Step computation")."""
        return _phases(lib().sph_ctx_get_phase_profile, self._h, self._check, "sph_ctx_get_phase_profile")

    def neighbors(self):
        L = lib()
        tot = (ctypes.c_longlong * 2)()
        self._check(L.sph_ctx_neighbors(self._h, None, None, None, None, None, None, tot), "sph_ctx_neighbors")
        n = self.n
        cells = np.zeros(3 * n, np.int32)
        rank = np.zeros(n, np.int32)
        off = np.zeros(n + 1, np.int32)
        nbr = np.zeros(max(tot[0], 1), np.int32)
        boff = np.zeros(n + 1, np.int32)
        bnbr = np.zeros(max(tot[1], 1), np.int32)
        self._check(L.sph_ctx_neighbors(self._h, _i(cells), _i(rank), _i(off), _i(nbr), _i(boff), _i(bnbr), tot),
                    "sph_ctx_neighbors")
        return dict(cell=cells.reshape(n, 3), cell_rank=rank, nbr_off=off, nbr=nbr[: tot[0]], bnbr_off=boff,
                    bnbr=bnbr[: tot[1]])

    def pair_lists(self):
        """The DFSPH pair lists the solver passes read: dict(count, off, nbr)
        by original index (count above the list width: overflowed, not stored)."""
        def call(c, o, nb, t):
            self._check(lib().sph_ctx_pair_lists(self._h, c, o, nb, t), "sph_ctx_pair_lists")

        return _pair_lists(call, self.n)


def _pair_lists(call, n):
    """CSR pair lists through a (count, off, nbr, total) dump call: dict of
    count, off, nbr (original indices)."""
    tot = ctypes.c_longlong()
    cnt = np.zeros(max(n, 1), np.int32)
    off = np.zeros(n + 1, np.int32)
    call(_i(cnt), _i(off), None, ctypes.byref(tot))
    nbr = np.zeros(max(tot.value, 1), np.int32)
    call(_i(cnt), _i(off), _i(nbr), ctypes.byref(tot))
    return dict(count=cnt[:n], off=off, nbr=nbr[: tot.value])


def select_device(device: int):
    rc = lib().sph_select_device(int(device))
    if rc != 0:
        raise SPHError(f"sph_select_device({device}) failed ({rc})")


def sample_box(support_radius, mn, mx):
    L = lib()
    m = L.sph_sample_box(support_radius, _d(_v3(mn)), _d(_v3(mx)), None)
    out = np.zeros((m, 3))
    L.sph_sample_box(support_radius, _d(_v3(mn)), _d(_v3(mx)), _d(out))
    return out


def sample_sphere(particle_radius, c, radius):
    L = lib()
    m = L.sph_sample_sphere(particle_radius, _d(_v3(c)), radius, None)
    out = np.zeros((m, 3))
    L.sph_sample_sphere(particle_radius, _d(_v3(c)), radius, _d(out))
    return out


def sample_pcisph_box(h, mn, mx, inverted=True):
    """PCISPHBoundaryModel::sampleCube as the library samples it: (points, normals)."""
    L = lib()
    n = L.sph_sample_pcisph_box(float(h), _d(_v3(mn)), _d(_v3(mx)), int(bool(inverted)), None, None)
    pts, nrm = np.zeros((n, 3)), np.zeros((n, 3))
    L.sph_sample_pcisph_box(float(h), _d(_v3(mn)), _d(_v3(mx)), int(bool(inverted)), _d(pts), _d(nrm))
    return pts, nrm


EMITTER_SQUARE, EMITTER_CIRCLE = 0, 1


def sample_mesh(obj_path, max_distance):
    """The boundary points AkinciBoundaryModel::addGeometry makes of an OBJ mesh."""
    L = lib()
    m = L.sph_sample_mesh(os.fsencode(obj_path), float(max_distance), None)
    if m < 0:
        raise SPHError(f"cannot sample {obj_path}")
    out = np.zeros((m, 3))
    if m:
        L.sph_sample_mesh(os.fsencode(obj_path), float(max_distance), _d(out))
    return out


def emitter_group(type, particle_radius, width, height=0.0):
    """Emitter::buildSquareGroup / buildCircleGroup: the group emitted each time, emitter frame."""
    L = lib()
    m = L.sph_emitter_group(int(type), float(particle_radius), float(width), float(height), None)
    if m < 0:
        raise SPHError("invalid emitter group arguments")
    out = np.zeros((m, 3))
    if m:
        L.sph_emitter_group(int(type), float(particle_radius), float(width), float(height), _d(out))
    return out


def fluid_block(particle_radius, mn, mx):
    L = lib()
    m = L.sph_fluid_block(particle_radius, _d(_v3(mn)), _d(_v3(mx)), None)
    out = np.zeros((m, 3))
    L.sph_fluid_block(particle_radius, _d(_v3(mn)), _d(_v3(mx)), _d(out))
    return out


class PoolFull(SPHError):
    """The scene does not fit beside the resident and queued scenes."""


class Pool:
    """Many independent DFSPH scenes resident on the GPU, advanced together."""

    def __init__(self, budget_bytes=None, max_particles=None, max_boundary=None, max_keys=None, max_scenes=4096,
                 neighbor_list_max=64):
        L = lib()
        d = PoolDesc()
        if budget_bytes is not None:
            L.sph_pool_desc_from_budget(int(budget_bytes), int(neighbor_list_max), ctypes.byref(d))
        else:
            d.max_particles = int(max_particles)
            d.max_boundary = int(max_boundary if max_boundary is not None else max_particles)
            d.max_keys = int(max_keys if max_keys is not None else 16 * max_particles)
            d.max_scenes = int(max_scenes)
            d.neighbor_list_max = int(neighbor_list_max)
        self.desc = d
        self._h = ctypes.c_void_p()
        rc = L.sph_pool_create(ctypes.byref(d), ctypes.byref(self._h))
        if rc != 0:
            raise SPHError(f"sph_pool_create failed ({rc})")
        self._n = {}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sph_pool_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            msg = lib().sph_pool_last_error(self._h)
            text = f"{what} failed ({rc}): {msg.decode() if msg else ''}"
            raise (PoolFull if rc == -4 else SPHError)(text)

    def _desc(self, params):
        """The scene descriptor of these parameters (built once per distinct
        parameter set: a mix of scenes usually shares one)."""
        key = tuple(sorted((k, tuple(v) if isinstance(v, (list, tuple)) else v) for k, v in params.items()))
        cache = self.__dict__.setdefault("_descs", {})
        d = cache.get(key)
        if d is None:
            d = cache[key] = make_desc(**params)
        return d

    def add_scene(self, x, v=None, boundary_points=None, steps=1, **params):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        b = None if boundary_points is None else np.ascontiguousarray(boundary_points, dtype=np.float64).reshape(-1, 3)
        d = self._desc(params)
        sid = ctypes.c_int()
        rc = lib().sph_pool_add_scene(self._h, ctypes.byref(d), _d(x), None if vv is None else _d(vv), x.shape[0],
                                      None if b is None else _d(b), 0 if b is None else b.shape[0], int(steps),
                                      ctypes.byref(sid))
        self._check(rc, "sph_pool_add_scene")
        self._n[sid.value] = (x.shape[0], 0 if b is None else b.shape[0])
        return sid.value

    def remove(self, sid):
        self._check(lib().sph_pool_remove_scene(self._h, int(sid)), "sph_pool_remove_scene")

    def step(self, n=1):
        self._check(lib().sph_pool_step(self._h, int(n)), "sph_pool_step")

    def set_graph(self, enable=True):
        self._check(lib().sph_pool_set_graph(self._h, int(bool(enable))), "sph_pool_set_graph")

    def synchronize(self):
        self._check(lib().sph_pool_synchronize(self._h), "sph_pool_synchronize")

    def query(self, sid):
        st = Stats()
        done = ctypes.c_int()
        self._check(lib().sph_pool_query(self._h, int(sid), ctypes.byref(st), ctypes.byref(done)), "sph_pool_query")
        return {name: getattr(st, name) for name, _ in Stats._fields_}, bool(done.value)

    def poll(self):
        n = ctypes.c_int()
        self._check(lib().sph_pool_poll(self._h, None, 0, ctypes.byref(n)), "sph_pool_poll")
        if n.value == 0:
            return []
        ids = np.zeros(n.value, np.int32)
        self._check(lib().sph_pool_poll(self._h, _i(ids), n.value, ctypes.byref(n)), "sph_pool_poll")
        return [int(t) for t in ids[: n.value]]

    def get(self, sid, field, out=None):
        fid, width = FIELDS[field]
        nf, nb = self._n[sid]
        count = nb if field in ("bx", "psi", "bdens", "bpress") else nf
        shape = (count, 3) if width == 3 else (count,)
        if out is None:
            out = np.zeros(shape)
        elif out.shape != shape or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError(f"out must be a C-contiguous float64 array of shape {shape}")
        if count:
            self._check(lib().sph_pool_download(self._h, int(sid), fid, _d(out)), f"sph_pool_download({field})")
        return out

    def usage(self):
        p, b, k = ctypes.c_ulonglong(), ctypes.c_ulonglong(), ctypes.c_ulonglong()
        s = ctypes.c_uint()
        lib().sph_pool_usage(self._h, ctypes.byref(p), ctypes.byref(b), ctypes.byref(k), ctypes.byref(s))
        return dict(particles=p.value, boundary=b.value, keys=k.value, scenes=s.value)

    def launch_count(self):
        n = ctypes.c_ulonglong()
        self._check(lib().sph_pool_get_launch_count(self._h, ctypes.byref(n)), "sph_pool_get_launch_count")
        return n.value

    def step_timed(self, n=1):
        ms = ctypes.c_float()
        self._check(lib().sph_pool_step_timed(self._h, int(n), ctypes.byref(ms)), "sph_pool_step_timed")
        return ms.value

    def set_profiling(self, enable=True):
        self._check(lib().sph_pool_set_profiling(self._h, int(bool(enable))), "sph_pool_set_profiling")

    def profile(self):
        buf = ctypes.create_string_buffer(1 << 16)
        n = lib().sph_pool_get_profile(self._h, buf, len(buf))
        if n < 0:
            self._check(n, "sph_pool_get_profile")
        out = {}
        for line in buf.value.decode().splitlines():
            name, cnt, ms = line.split()
            out[name] = (int(cnt), float(ms))
        return out

    def phase_profile(self):
        """As Scene.phase_profile, for the pool's steps."""
        return _phases(lib().sph_pool_get_phase_profile, self._h, self._check, "sph_pool_get_phase_profile")

    def set_autotune(self, mode=1):
        """0 off, 1 cached-or-measured after each re-layout (default), 2 measure again."""
        self._check(lib().sph_pool_set_autotune(self._h, int(mode)), "sph_pool_set_autotune")

    def tuning(self):
        t = PoolTuning()
        self._check(lib().sph_pool_get_tuning(self._h, ctypes.byref(t)), "sph_pool_get_tuning")
        return {name: getattr(t, name) for name, _ in PoolTuning._fields_}

    def set_tuning(self, build_block=256, build_occupancy=768, queue_depth=48, solver_block=128, solver_occupancy=1024,
                   scan_width=16):
        t = PoolTuning(build_block, build_occupancy, queue_depth, solver_block, solver_occupancy, scan_width, 0, 0)
        self._check(lib().sph_pool_set_tuning(self._h, ctypes.byref(t)), "sph_pool_set_tuning")

    def tuning_log(self):
        buf = ctypes.create_string_buffer(1 << 14)
        lib().sph_pool_get_tuning_log(self._h, buf, len(buf))
        return buf.value.decode()

    def tune(self):
        """Run the pending tuning steps now (ordinary steps of every resident
        scene); returns how many steps were taken."""
        k = 0
        self.step(1)
        k += 1
        while self.tuning()["steps_left"] > 0:
            self.step(1)
            k += 1
        return k

    def list_pairs(self):
        p, o = ctypes.c_ulonglong(), ctypes.c_uint()
        self._check(lib().sph_pool_list_pairs(self._h, ctypes.byref(p), ctypes.byref(o)), "sph_pool_list_pairs")
        return p.value, o.value

    def pair_lists(self, sid):
        """A resident scene's pair lists, as Scene.pair_lists."""
        def call(c, o, nb, t):
            self._check(lib().sph_pool_pair_lists(self._h, int(sid), c, o, nb, t), "sph_pool_pair_lists")

        return _pair_lists(call, self._n[sid][0])

    def snapshot(self, sid):
        """A resident scene's snapshot (bytes): everything its future steps
        depend on, for sph_pool_restore."""
        size = ctypes.c_ulonglong()
        self._check(lib().sph_pool_snapshot(self._h, int(sid), None, 0, ctypes.byref(size)), "sph_pool_snapshot")
        buf = ctypes.create_string_buffer(size.value)
        self._check(lib().sph_pool_snapshot(self._h, int(sid), buf, size.value, ctypes.byref(size)), "sph_pool_snapshot")
        return buf.raw

    def restore(self, snap, steps=0):
        """Admit a scene from a snapshot; `steps` more steps (0: the steps it
        had left).  Returns its scene id."""
        buf = ctypes.create_string_buffer(bytes(snap), len(snap))
        sid = ctypes.c_int()
        self._check(lib().sph_pool_restore(self._h, buf, len(snap), int(steps), ctypes.byref(sid)), "sph_pool_restore")
        import struct
        # header: magic[8], version, desc_size, scalars_size, n, nb, steps_left (uint32)
        n, nb = struct.unpack_from("<II", bytes(snap), 20)
        self._n[sid.value] = (n, nb)
        return sid.value

    def count_work(self):
        """The list build's work at the current positions: candidates its walks
        visit and pairs within h, fluid and boundary."""
        out = (ctypes.c_ulonglong * 4)()
        self._check(lib().sph_pool_count_work(self._h, out), "sph_pool_count_work")
        return dict(fluid_candidates=out[0], fluid_pairs=out[1], boundary_candidates=out[2], boundary_pairs=out[3])


class Server:
    """The library's request loop over a pool (sph_server_*): submit scenes
    from any thread; a driver thread in the library steps the pool in epochs,
    admits queued scenes as capacity frees up and retires completed ones.
    While it exists, nothing else steps the pool."""

    def __init__(self, pool, epoch_steps=10, lookahead=8, keep_results=False, max_queued_bytes=0):
        L = lib()
        d = ServerDesc()
        L.sph_server_desc_init(ctypes.byref(d))
        d.epoch_steps, d.lookahead, d.keep_results = int(epoch_steps), int(lookahead), int(bool(keep_results))
        d.max_queued_bytes = int(max_queued_bytes)
        self.pool = pool
        self._h = ctypes.c_void_p()
        rc = L.sph_server_create(pool._h, ctypes.byref(d), ctypes.byref(self._h))
        if rc != 0:
            raise SPHError(f"sph_server_create failed ({rc})")
        self._n = {}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().sph_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            msg = lib().sph_server_last_error(self._h)
            raise SPHError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def submit(self, x, v=None, boundary_points=None, steps=1, **params):
        """Queue a scene; returns its request id, or None when the queue
        already holds max_queued_bytes (the request is not queued)."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, 3)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64).reshape(-1, 3)
        b = None if boundary_points is None else np.ascontiguousarray(boundary_points, dtype=np.float64).reshape(-1, 3)
        d = make_desc(**params)
        rid = ctypes.c_longlong()
        rc = lib().sph_server_submit(self._h, ctypes.byref(d), _d(x), None if vv is None else _d(vv), x.shape[0],
                                     None if b is None else _d(b), 0 if b is None else b.shape[0], int(steps),
                                     ctypes.byref(rid))
        if rc == ERR_CAPACITY:
            return None
        self._check(rc, "sph_server_submit")
        self._n[rid.value] = x.shape[0]
        return rid.value

    @staticmethod
    def _info(r):
        return {name: getattr(r, name) for name, _ in RequestInfo._fields_}

    def completed(self, max_n=4096):
        buf = (RequestInfo * max_n)()
        n = ctypes.c_int()
        self._check(lib().sph_server_completed(self._h, buf, max_n, ctypes.byref(n)), "sph_server_completed")
        return [self._info(buf[k]) for k in range(n.value)]

    def query(self, rid):
        r = RequestInfo()
        self._check(lib().sph_server_query(self._h, int(rid), ctypes.byref(r)), "sph_server_query")
        return self._info(r)

    def fetch(self, rid, field):
        fid, _ = FIELDS[field]
        out = np.zeros((self._n[rid], 3))
        self._check(lib().sph_server_fetch(self._h, int(rid), fid, _d(out)), f"sph_server_fetch({field})")
        return out

    def release(self, rid):
        lib().sph_server_release(self._h, int(rid))

    def drain(self, timeout_s=600.0):
        idle = ctypes.c_int()
        self._check(lib().sph_server_drain(self._h, float(timeout_s), ctypes.byref(idle)), "sph_server_drain")
        return bool(idle.value)

    def stats(self):
        st = ServerStats()
        self._check(lib().sph_server_get_stats(self._h, ctypes.byref(st)), "sph_server_get_stats")
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}
