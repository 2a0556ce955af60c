"""bench.py's roofline arithmetic on the host: kernels merged by __global__
function as the ncu launch list names them, the largest share first, the
figures of the ncu summaries under profiles/, and the list build's FP32 work."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402

N, NB, PAIRS = 4_151_352, 4_127_798, 107_200_000
PROF = {"k_pool_build_lists": (10, 16.2), "k_pool_correct": (40, 13.3), "k_pool_errors_density": (30, 10.8),
        "k_pool_errors_div": (10, 3.6), "k_gather_fluid": (10, 1.1)}


def test_error_pass_instantiations_count_as_one_kernel():
    r = bench.roofline(PROF, N, NB, PAIRS, "batched_mix_256")
    names = [k["kernel"] for k in r["kernels"]]
    assert names == ["k_pool_build_lists", "k_pool_errors", "k_pool_correct"]
    err = r["kernels"][1]
    assert err["launches"] == 40 and err["avg_launch_ms"] == pytest.approx(14.4 / 40)
    # algorithmic bytes: the launch-weighted mean of 40 and 36 B per particle
    assert err["algorithmic_bytes_per_launch"] == pytest.approx(N * (30 * 40 + 10 * 36) / 40)
    total = sum(ms for _, ms in PROF.values())
    assert r["kernel"] == "k_pool_build_lists" and r["kernel_share"] == pytest.approx(16.2 / total)


def test_achieved_bandwidth_and_pair_stream():
    r = bench.roofline(PROF, N, NB, PAIRS, "batched_mix_256")
    b = r["kernels"][0]
    algo = N * bench.ALGO_BYTES["k_pool_build_lists"][0] + NB * 16
    assert b["algorithmic_bytes_per_launch"] == algo
    assert b["achieved"] == pytest.approx(algo / 1.62e-3 / 1e9)
    assert b["with_pair_lists"]["bytes_per_launch"] == algo + PAIRS * 16
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])


def test_profile_figures_attach_to_their_kernels():
    figs = bench.profile_figures("batched_mix_256")
    assert figs["k_pool_build_lists"]["dram_bytes_per_launch"] > 0
    assert "sm_issue_active_pct" in figs["k_pool_build_lists"]
    assert figs["k_pool_correct"]["dram_bytes_per_launch"] > 0
    assert figs["k_pool_errors"]["dram_bytes_per_launch"] > 0   # a line of the correction summary
    r = bench.roofline(PROF, N, NB, PAIRS, "batched_mix_256")
    assert r["traffic"] == figs["k_pool_build_lists"]["dram_bytes_per_launch"]
    assert r["issue"]["source"].startswith("profiles")


def test_build_fp32_work():
    w = dict(fluid_candidates=1000, fluid_pairs=200, boundary_candidates=300, boundary_pairs=50)
    assert bench.build_flops(w) == 8 * 1300 + 34 * 250 + 6 * 200
    r = bench.roofline(PROF, N, NB, PAIRS, "batched_mix_256", work=w, fp32_peak=70.0)
    f = r["fp32"]
    assert f["flops_per_launch"] == bench.build_flops(w)
    assert f["achieved"] == pytest.approx(bench.build_flops(w) / 1.62e-3 / 1e12)
    assert f["frac"] == pytest.approx(f["achieved"] / 70.0)
    assert "fp32" not in bench.roofline(PROF, N, NB, PAIRS, "batched_mix_256")
