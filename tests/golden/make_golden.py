"""Generate the golden fixtures from the reference simulator itself.

Runs the reference's own solver (its sources compiled headless with the
project's GLM shim, `make -C oracle ref`, parity build, one OpenMP thread) on
every scene of tests/scenes.py and stores inputs and per-step outputs as
compressed .npz files in this directory.  Needs the reference tree, so it
runs only where that tree is mounted:

    python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from scenes import EMIT_DUMP_EVERY, EMIT_SCENES, EMIT_STEPS, SCENES, emit_scene, scene, scene_extra  # noqa: E402

STEPS = 3
SCENE_FILE_STEPS = 12
# read before the reference first sets them (uninitialised solver members)
UNSET_AT_INIT = ("init.iterationsV", "init.avgDensError", "init.avgDivError")
KEEP = ("x", "v", "a", "rho", "p", "alpha", "div", "pred", "k", "kv", "pacc", "time", "dt", "iterations",
        "iterationsV", "avgDensError", "avgDivError", "maxDensityError", "scaling", "normal", "bdens", "bpress")


def resolve_mesh_paths(sc, base):
    """Mesh paths in a scene file are relative to the file; the reference
    reads them relative to its working directory, so make them absolute."""
    for b in sc.get("Boundary", []):
        for g in b.get("geometry", []):
            g["path"] = os.path.abspath(os.path.join(base, g["path"]))


# mesh files and sample spacings (in particle diameters 2r, r = 0.02) whose
# boundary samples are kept in meshes.npz
MESH_CASES = (("ramp", 0.5), ("ramp", 1.3), ("tetra_attrs", 1.0), ("tetra_attrs", 0.25))


def main(ref_tree="/root/reference"):
    if not oracle.reference_available():
        if not oracle.build_reference(ref_tree):
            raise SystemExit("reference tree not found; cannot generate fixtures")
    here = os.path.dirname(os.path.abspath(__file__))
    for name in SCENES:
        params, x, boxes, spheres = scene(name)
        v, bh_boxes, bh_spheres = scene_extra(name, x)
        dump = oracle.run_reference(params, x, v, boxes=boxes, spheres=spheres, steps=STEPS,
                                    dump_neighbors=params["method"] == 2, bh_boxes=bh_boxes, bh_spheres=bh_spheres)
        out = {"input.x": x}
        if v is not None:
            out["input.v"] = v
        for k, v in dump.items():
            tag, _, field = k.partition(".")
            if k in UNSET_AT_INIT:
                continue
            if k in ("b.x", "b.psi", "h", "mass") or k.startswith("init.") or field in KEEP:
                out[k] = v
        np.savez_compressed(os.path.join(here, f"{name}.npz"), **out)
        print(name, x.shape[0], "fluid,", len(dump.get("b.x", [])) // 3, "boundary")
    # emitter scenes: EMIT_STEPS steps, the state of every EMIT_DUMP_EVERY-th
    for name in EMIT_SCENES:
        params, x, boxes, spheres, emitters = emit_scene(name)
        dump = oracle.run_reference(params, x, None, boxes=boxes, spheres=spheres, steps=EMIT_STEPS,
                                    dump_every=EMIT_DUMP_EVERY, emitters=emitters)
        out = {"input.x": x}
        for k, v in dump.items():
            tag, _, field = k.partition(".")
            if k in UNSET_AT_INIT:
                continue
            if k in ("b.x", "b.psi", "h", "mass") or k.startswith("init.") or field in KEEP:
                out[k] = v
        np.savez_compressed(os.path.join(here, f"{name}.npz"), **out)
        print(name, x.shape[0], "fluid at start,", len(dump[f"s{EMIT_STEPS}.rho"]), "after", EMIT_STEPS, "steps")
    # scene files (scenes/*.json) through the reference's own loader
    # (Simulation::importScene) with frame output on: state every third of
    # SCENE_FILE_STEPS steps and every frame file SceneLoader::writeFluid wrote
    import json

    for fn in sorted(os.listdir(os.path.join(here, "scenes"))):
        if not fn.endswith(".json"):
            continue
        with open(os.path.join(here, "scenes", fn)) as f:
            sc = json.load(f)
        resolve_mesh_paths(sc, os.path.join(here, "scenes"))
        dump = oracle.run_reference_json(sc, steps=SCENE_FILE_STEPS, dump_every=3, save=True,
                                         dump_neighbors=sc["Configuration"]["simulationMethod"] == 2)
        out = {}
        for k, v in dump.items():
            tag, _, field = k.partition(".")
            if k in UNSET_AT_INIT:
                continue
            if k in ("b.x", "b.psi", "h", "mass") or k.startswith("init.") or k.startswith("frame") or field in KEEP:
                out[k] = v
        np.savez_compressed(os.path.join(here, "file_" + fn[:-5] + ".npz"), **out)
        print("file", fn, len(dump["init.rho"]), "fluid at init,", sum(1 for k in dump if k.endswith(".raw")), "frames")
    mesh_fixture(here)


def mesh_fixture(here):
    """AkinciBoundaryModel::addGeometry's samples of the test meshes, from
    the reference build (a box is added first, as a scene file would)."""
    x = oracle.fluid_block(0.02, (0.2, 0.5, 0.2), (0.3, 0.6, 0.3))
    nbox = oracle.sample_box(0.08, (0, 0, 0), (0.8, 0.8, 0.8)).shape[0]
    out = {}
    for mesh, sp in MESH_CASES:
        path = os.path.join(here, "meshes", mesh + ".obj")
        dump = oracle.run_reference(dict(method=2, boundary=2, radius=0.02), x, boxes=[((0, 0, 0), (0.8, 0.8, 0.8))],
                                    steps=1, geometries=[(path, sp)])
        out[f"{mesh}/{sp!r}"] = dump["b.x"].reshape(-1, 3)[nbox:]
    np.savez_compressed(os.path.join(here, "meshes.npz"), **out)
    print("meshes", {k: v.shape[0] for k, v in out.items()})


if __name__ == "__main__":
    main(*sys.argv[1:])
