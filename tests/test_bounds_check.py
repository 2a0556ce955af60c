"""The bounds-checked build (libsph_gb300_checked.so: the same sources with
-DSPH_BOUNDS_CHECK, sph_gb300/buildlib.py): every neighbour index read from
device data -- pair records of the DFSPH lists (one scene and pool), PCISPH
candidate-list entries -- is checked against its array's length, and an
out-of-range one would set SPH_STATUS_BOUNDS and be skipped (no trap, no
fault).  compute-sanitizer is closed on this machine; this build stands in for
its out-of-bounds check on the indices that come from device data.

Run on the same fixed workload (tests/bounds_workload.py) as the ordinary
build: no scene reports SPH_STATUS_BOUNDS, and every result is bit-identical
(the checks change no arithmetic)."""
import json
import os
import subprocess
import sys

import pytest

import sph_gb300
from sph_gb300 import buildlib

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def run_workload(library):
    env = dict(os.environ)
    if library:
        env["SPH_GB300_LIBRARY"] = library
    else:
        env.pop("SPH_GB300_LIBRARY", None)
    p = subprocess.run([sys.executable, os.path.join(HERE, "bounds_workload.py")], capture_output=True, text=True,
                       env=env, timeout=900)
    assert p.returncode == 0, p.stderr[-2000:]
    return json.loads(p.stdout.strip().splitlines()[-1])


def test_checked_build_finds_no_bad_index_and_changes_nothing(gpu_lib):
    checked = buildlib.build(variant="checked")
    plain = run_workload(None)
    chk = run_workload(checked)
    print(plain, chk)
    for name, st in chk["status"].items():
        assert st & sph_gb300.STATUS_BOUNDS == 0, name
        assert st == plain["status"][name], name
    assert chk["hash"] == plain["hash"]
