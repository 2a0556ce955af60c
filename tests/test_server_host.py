"""The request loop's host logic (sph_gb300/csrc/sph_serve.cpp, the C++
driver behind sph_server_*) on the CPU: the same source compiled with g++
against a fake of the pool's C ABI (tests/server_fake_pool.cpp), in which a
scene is a particle count against a capacity and a step advances step
counts, taking a fixed wall time as a GPU epoch would.

* every submitted scene completes, is reported once, keeps its result, and
  the work is counted exactly (particles x steps);
* admission respects capacity, scenes join while others are mid-run
  (continuous batching);
* the look-ahead admits a later small scene past one that does not fit;
* a bound on queued request bytes refuses submissions beyond it (counted as
  rejected) and the queued ones still complete.

The GPU test (test_server.py) runs the same loop on the real pool."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("server") / "server_fake")
    subprocess.run(["g++", "-std=c++17", "-O1", "-pthread", "-o", out, os.path.join(ROOT, "tests", "server_fake_pool.cpp"),
                    os.path.join(ROOT, "sph_gb300", "csrc", "sph_serve.cpp")], check=True, capture_output=True)
    return out


def run(exe, scenario):
    p = subprocess.run([exe, scenario], capture_output=True, text=True, timeout=120)
    assert p.returncode == 0, p.stderr
    return [json.loads(ln) for ln in p.stdout.splitlines() if ln.startswith("{")]


def test_every_request_completes_once_with_its_result(exe):
    extra, out = run(exe, "complete")
    assert extra == {"reported": 25, "bad": 0, "reported_again": 0}
    assert out["completed"] == out["submitted"] == 25 and out["queued"] == 0 and out["resident"] == 0
    assert out["particle_steps"] == 25 * 100 * 30
    assert 0 < out["p50"] <= out["p99"]
    assert out["max_used"] <= out["capacity"]


def test_admission_respects_capacity_and_batches_continuously(exe):
    (out,) = run(exe, "capacity")
    assert out["completed"] == 16
    assert out["max_resident"] == 3 and out["max_used"] <= out["capacity"] == 350
    assert out["particle_steps"] == 10 * 100 * 30 + 100 * (10 + 20 + 30 + 40 + 50 + 60)
    assert out["joined_mid_run"] == 1


def test_lookahead_admits_a_later_scene_past_one_that_does_not_fit(exe):
    (out,) = run(exe, "lookahead")
    assert out["completed"] == 3
    assert out["order"] == [50, 50, 900]


def test_queue_bound_rejects_submissions_beyond_it(exe):
    full, out = run(exe, "backpressure")
    assert full["submitted"] == 3 and full["rejected"] == 7 and full["queued"] == 3
    assert full["queued_bytes"] == 3 * 100 * 3 * 8
    assert out["completed"] == 3 and out["queued"] == 0 and out["queued_bytes"] == 0
