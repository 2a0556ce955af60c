"""Benchmark of the per-step SPH particle loop on GB300.

Workload (default): the DFSPH dam break with Akinci boundaries -- a
50 x 50 x 50 = 125,000-particle fluid block at r = 0.005 m in the corner of a
1.5 x 0.8 x 0.8 m box whose walls are sampled as Akinci boundary particles
(60,802 points), CFL-adaptive dt in [1e-5, 5e-3] s, 0.1 % average density
error, 0.1 %/s divergence error, at most 100 iterations, 2000 steps.  (At
r = 0.01 m the 50^3 block would be 1 m tall and not fit the 0.8 m box;
r = 0.005 m keeps the particle count and the box.  The block starts 2r off
the walls: with its first layer at r from an Akinci wall the reference's DFSPH
ejects the wall-adjacent particles at hundreds of m/s in the first step.)  A "step" is one DFSPHSolver::step of that scene
(one time step: non-pressure forces, CFL, density solve, neighbour grid,
densities/alpha, divergence solve); the metric is particle-steps/s.

Arms:
  default            the CUDA path (FP32 bulk, FP64 reductions), whole steps as
                     CUDA graphs with device-side solver loops
  --impl reference   the reference's CPU algorithm on the host cores (the C
                     restatement in oracle/, OpenMP, every host thread), a
                     bounded number of steps of the same scene

Prints one JSON line (rank 0).  Multi-GPU (torchrun): every rank runs its own
replica of the scene (scenes are independent; no collective on the data
path); value = all ranks' particle-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DFSPH particle-steps/s @0.1% density err"
UNIT = "particle-steps/s"

WORKLOADS = {
    "dfsph_dam_break_125k": dict(
        params=dict(method=2, boundary=2, radius=0.005, eta=0.001, eta_v=0.001, cfl=1.0, max_it=100, dt=1e-4,
                    min_dt=1e-5, max_dt=5e-3, fps=60.0),
        block=((0.01, 0.01, 0.01), (0.51, 0.51, 0.51)),
        box=((0.0, 0.0, 0.0), (1.5, 0.8, 0.8)),
    ),
}

# Compulsory bytes of each kernel as implemented (FP32 form: float4 = 16 B,
# scalar = 4 B; each array read once and written once, neighbour re-reads not
# counted): (bytes per fluid particle, bytes per stored pair, touches the
# boundary particles at 16 B each).
ALGO_BYTES = {
    "k_cell_update": (64, 0, False),
    "k_scatter": (16, 0, False),
    "k_gather_fluid": (108, 0, False),
    "k_density": (32, 0, True),
    "k_dfsph_cfl": (32, 0, False),
    "k_dfsph_predict_v_warm": (108, 0, False),
    "k_dfsph_correct": (68, 0, True),
    "k_dfsph_predict_density": (64, 0, True),
    "k_dfsph_divergence": (64, 0, True),
    "k_npforce": (68, 0, True),
    "k_st_normals": (36, 0, False),
    "k_build_lists": (52, 16, True),
    "k_dfsph_correct_list": (72, 16, False),
    "k_dfsph_predict_density_list": (52, 16, False),
    "k_dfsph_divergence_list": (52, 16, False),
}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def dist_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def make_scene(wl, precision="f32", G=0, list_max=64):
    import sph_gb300

    w = WORKLOADS[wl]
    s = sph_gb300.Scene(precision=precision, threads_per_particle=G, neighbor_list_max=list_max, **w["params"])
    s.add_fluid_block(*w["block"])
    s.add_boundary_box(*w["box"])
    return s


def cpu_reference(wl, steps, warmup, threads, budget_s):
    """The reference's algorithm on the host (C restatement, OpenMP)."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle

    w = WORKLOADS[wl]
    r = w["params"]["radius"]
    x = oracle.fluid_block(r, *w["block"])
    o = oracle.OracleScene(w["params"], x, boxes=[w["box"]])
    for _ in range(max(0, warmup)):
        o.step(1)
    done, its, t0 = 0, 0, time.perf_counter()
    while done < max(1, steps):
        o.step(1)
        its += o.scalar("iterations")
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    el = time.perf_counter() - t0
    return o.n * done / el, done, its / done, o.n


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    warm = min(args.warmup, 1)
    v, done, mean_it, n = cpu_reference(args.workload, args.steps, warm, threads, args.ref_budget)
    sample = f"{done} DFSPH steps of the {n}-particle scene after {warm} warm-up step(s)"
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": done, "warmup": warm,
        "ms_per_step": 1000.0 * n / v, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": args.workload, "fluid_particles": n, "mean_iterations": mean_it,
                   "implementation": "reference algorithm restated in C (oracle/sph_oracle.c), OpenMP"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def flush_l2(buf):
    # write a buffer larger than L2 (126 MB) between timed steps
    buf.fill_(1.0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="dfsph_dam_break_125k", choices=list(WORKLOADS))
    ap.add_argument("--threads-per-particle", type=int, default=0)
    ap.add_argument("--list-max", type=int, default=64, help="pair-list slots per particle (0: cell walks)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=25.0, help="seconds of CPU baseline work")
    ap.add_argument("--ref-budget", type=float, default=90.0, help="seconds of reference-arm timed work")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import torch

    import sph_gb300

    sph_gb300.build()
    sph_gb300.select_device(local)
    torch.cuda.set_device(local)
    G = args.threads_per_particle

    # ---- device-resident timed region -------------------------------------
    s = make_scene(args.workload, G=G, list_max=args.list_max)
    s.init()
    s.set_graph(True)
    s.step(max(3, args.warmup))
    s.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    st0 = s.stats()
    l0 = s.launch_count()
    n = s.n
    step_ms = []
    dist_barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush_l2(flush)
            torch.cuda.synchronize()
            step_ms.append(s.step_timed(1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    st1 = s.stats()
    l1 = s.launch_count()
    total_ms = float(np.sum(step_ms))
    t_max = dist_max(total_ms, world)
    value = world * n * args.steps / (t_max / 1000.0)
    its = (st1["sum_iterations"] - st0["sum_iterations"]) / args.steps
    itsv = (st1["sum_iterations_v"] - st0["sum_iterations_v"]) / args.steps
    sim_s = st1["time"] - st0["time"]

    # ---- per-kernel event timing (same scene, host-driven steps) ----------
    s.set_graph(False)
    s.set_profiling(True)
    s.profile()
    prof_steps = min(args.steps, 20)
    for _ in range(prof_steps):
        flush_l2(flush)
        torch.cuda.synchronize()
        s.step(1)
    prof = s.profile()
    s.set_profiling(False)
    nb = s.nb
    kern = max(prof.items(), key=lambda kv: kv[1][1]) if prof else ("none", (1, 0.0))
    kname, (kcount, kms) = kern
    per_b, per_pair, touches_b = ALGO_BYTES.get(kname, (0, 0, False))
    pairs = s.stats()["list_pairs"]
    bytes_launch = n * per_b + pairs * per_pair + (nb * 16 if touches_b else 0)
    avg_ms = kms / max(kcount, 1)
    achieved = bytes_launch / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else 0.0
    peak, peak_kind = load_peaks()
    traffic = None
    tp = os.path.join(ROOT, "profiles", f"ncu_{kname}_{args.workload}.md")
    if os.path.exists(tp):
        for ln in open(tp):
            if ln.startswith("dram_bytes_per_launch:"):
                traffic = float(ln.split(":", 1)[1])
    total_prof_ms = sum(v[1] for v in prof.values())

    # ---- end to end through the C ABI with host buffers --------------------
    e2e = None
    if rank == 0 or world > 1:
        import ctypes

        w = WORKLOADS[args.workload]
        x_host = torch.from_numpy(sph_gb300.fluid_block(w["params"]["radius"], *w["block"])).pin_memory().numpy()
        v_host = torch.zeros_like(torch.from_numpy(x_host)).pin_memory().numpy()
        out_x = torch.empty(x_host.shape, dtype=torch.float64).pin_memory().numpy()
        out_v = torch.empty(x_host.shape, dtype=torch.float64).pin_memory().numpy()
        e_steps = args.steps
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e = sph_gb300.Scene(precision="f32", threads_per_particle=G, neighbor_list_max=args.list_max, **w["params"])
        e.set_fluid(x_host, v_host)
        e.add_boundary_box(*w["box"])
        e.init()
        e.set_graph(True)
        for _ in range(args.warmup + e_steps):
            e.step(1)
            e.stats()  # the step's result (dt, iterations, errors) read back every step
        out_x[:] = e.get("x")
        out_v[:] = e.get("v")
        e_wall = time.perf_counter() - t0
        e_n = e.n
        h2d = x_host.nbytes + v_host.nbytes + e.nb * 24
        d2h = out_x.nbytes + out_v.nbytes + (args.warmup + e_steps) * ctypes.sizeof(sph_gb300.Stats)
        tot_steps = args.warmup + e_steps
        e_wall_max = dist_max(e_wall, world)
        e2e = {"value": world * e_n * tot_steps / e_wall_max, "unit": UNIT,
               "h2d_bytes_per_step": h2d / tot_steps, "d2h_bytes_per_step": d2h / tot_steps,
               "scope": "create + upload from pinned host + init + steps (stats read back each step) + download x, v"}
        e.close()

    # ---- CPU baseline (rank 0, N = 1) ---------------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, done, mean_it, nn = cpu_reference(args.workload, 3, 1, threads, args.cpu_budget)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{done} DFSPH steps of the {nn}-particle scene after 1 warm-up step, "
                         f"reference algorithm restated in C (oracle/), OpenMP, mean {mean_it:.1f} iterations/step"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": args.workload, "fluid_particles": n, "boundary_particles": nb,
                       "parallelism": f"replicas x{world}", "l2": "flushed between timed steps (256 MB write)",
                       "step_timing": "CUDA events on the scene's stream around each graph-launched step",
                       "mean_density_iterations": its, "mean_divergence_iterations": itsv,
                       "simulated_seconds_per_second": sim_s / (total_ms / 1000.0),
                       "threads_per_particle": G or 1, "neighbor_list_max": args.list_max,
                       "list_pairs": st1["list_pairs"], "list_overflow": st1["list_overflow"], "wall_s": wall},
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": bytes_launch, "avg_launch_ms": avg_ms,
                         "kernel_share": kms / total_prof_ms if total_prof_ms else None,
                         "timing": f"CUDA events around each launch, {prof_steps} host-driven steps"},
            "clocks": clocks.summary(),
            "gpu_launches": l1 - l0,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "kernels": {k: {"launches": c, "ms": round(ms, 4)} for k, (c, ms) in sorted(prof.items(),
                                                                                      key=lambda kv: -kv[1][1])},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
