"""Benchmark of the per-step SPH particle loop on GB300: DFSPH particle-steps/s
at 0.1 % average density error, batched/served versus the plain one-scene GPU
solver, with p50/p99 scene latency.

Workloads (seeded, synthetic; sph_gb300/workloads.py):
  batched_mix_256  (headline) 256 independent DFSPH scenes, fluid counts
                   log-uniform in [2k, 64k] (seed 42; 4,151,352 fluid and
                   4,127,798 Akinci boundary particles in all), block aspect
                   ratios U(0.5, 2), 0-3 Akinci sphere obstacles of radius
                   0.05-0.2 m in a 1 m Akinci box, r = 0.01 m, CFL-adaptive
                   dt in [1e-5, 5e-3] s, 0.1 % density / 0.1 %/s divergence
                   error, FP32 bulk with FP64 reductions.  Every scene runs
                   the autotuner's measuring steps (24, ordinary steps that
                   pick the launch shapes), W warm-up and K timed steps
                   (about 500 at the defaults).
  dam_break_125k   one 50^3 = 125,000-particle dam break at r = 0.005 m in a
                   1.5 x 0.8 x 0.8 m Akinci box (60,802 boundary points).
                   (At r = 0.01 m the 50^3 block is 1 m tall and does not
                   fit the 0.8 m box; r = 0.005 m keeps count and box.)
  pcisph_drop_490k the PCISPH drop impact at r = 2.75 mm: a 9-layer pool and a
                   0.2 m-radius sphere 0.6 m above it in a 1 m Akinci box
                   (489,771 fluid, 198,746 boundary particles), standard
                   viscosity, Akinci surface tension and adhesion, dt 1e-4 s,
                   one scene in graph mode (candidate lists), 1,000 steps.

One "step" of the headline is one step of every scene of the mix: the pool
advances all resident scenes with one CUDA graph launch per step (segmented
grid, per-scene CFL, per-scene solver loops as device-side conditional
nodes).  value = sum over scenes of fluid particles x K / device time of the
K timed steps.  Beside it, on the same mix and the same steps:
  plain      each scene alone through the plain one-scene solver (the same
             kernels, one scene per graph);
  served     the request loop (continuous batching, admission by an 80 GB
             HBM budget) on a Poisson stream of mixed scenes at 200 scenes/s
             (saturating) and at a sub-saturation rate, with a 4M-particle
             dam break every 10 s: aggregate particle-steps/s, p50/p99 scene
             latency;
  dam_break_125k  the plain solver on the single large scene;
  pcisph_drop_490k  the PCISPH solver on the full-size drop;
  e2e        the mix through the pool's C ABI with host buffers: scenes
             uploaded from pinned host memory, per-step status read back,
             final positions and velocities downloaded, all timed;
  cpu_baseline  the reference's algorithm (the C restatement in oracle/,
             OpenMP on every host core) on a seeded 16-scene sample of the mix.

Arms:
  default            the CUDA path
  --impl reference   the reference's CPU algorithm on the host cores on the
                     16-scene sample of the mix, bounded in time

Prints one JSON line (rank 0).  Multi-GPU (torchrun): every rank runs its own
replica of the mix (scenes are independent; no collective on the data path);
value = all ranks' particle-steps / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DFSPH particle-steps/s @0.1% density err, served vs plain GPU; p50/p99 latency"
UNIT = "particle-steps/s"
WORKLOAD = "batched_mix_256"
CPU_SAMPLE_SCENES = 16
TUNE_STEPS = 25  # at most: the autotuner's 24 measuring steps + the admitting step

# Algorithmic bytes of each kernel: the compulsory field traffic per fluid
# particle of the reference's pass it implements (FP32 SoA: float4 = 16 B,
# scalar = 4 B; each array read once and written once, neighbour re-reads not
# counted; walks that touch the boundary add 16 B per boundary particle).
# (bytes per fluid particle, touches the boundary, pair-list bytes per stored
# pair that the kernel streams as implemented).
ALGO_BYTES = {
    "k_cell_update": (64, False, 0),
    "k_pool_cell_update": (64, False, 0),
    "k_scatter": (16, False, 0),
    "k_gather_fluid": (108, False, 0),
    "k_density": (28, True, 0),
    "k_build_lists": (28, True, 16),
    # fused with the divergence solve's first error pass: + v 16, div 4
    "k_pool_build_lists": (48, True, 16),
    "k_dfsph_cfl": (32, False, 0),
    "k_pool_cfl_accum": (32, False, 0),
    "k_dfsph_predict_v_warm": (76, False, 0),
    "k_pool_predict_v_warm": (76, False, 0),
    "k_dfsph_correct": (68, True, 0),
    "k_dfsph_correct_list": (68, False, 16),
    "k_pool_correct": (68, False, 16),
    "k_dfsph_predict_density": (40, True, 0),
    "k_dfsph_predict_density_list": (40, False, 16),
    "k_pool_errors_density": (40, False, 16),
    "k_dfsph_divergence": (36, True, 0),
    "k_dfsph_divergence_list": (36, False, 16),
    "k_pool_errors_div": (36, False, 16),
    "k_npforce": (68, True, 0),
    "k_pool_npforce": (68, True, 0),
    "k_st_normals": (36, False, 0),
    "k_pool_st_normals": (36, False, 0),
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


def mix(steps, geometry=None):
    from sph_gb300 import workloads

    return workloads.batched_mix(n_scenes=256, seed=42, steps=steps, r=0.01, geometry=geometry)


# ---- CPU: the reference's algorithm on a sample of the mix -----------------

def cpu_mix_sample(scenes, steps_each, threads, budget_s):
    """The first CPU_SAMPLE_SCENES scenes of the mix through the C restatement
    (OpenMP on `threads` host threads), one untimed warm-up step each, then up
    to `steps_each` timed steps each within budget_s / #scenes seconds."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle

    sample = scenes[:CPU_SAMPLE_SCENES]
    per = budget_s / len(sample)
    work, el, done_steps, its = 0, 0.0, 0, 0
    for x, b, params, _ in sample:
        p = {k: v for k, v in params.items() if k != "precision"}
        o = oracle.OracleScene(p, x, points=b)
        o.step(1)
        t0 = time.perf_counter()
        k = 0
        while k < steps_each:
            o.step(1)
            its += o.scalar("iterations")
            k += 1
            if time.perf_counter() - t0 > per:
                break
        el += time.perf_counter() - t0
        work += o.n * k
        done_steps += k
        del o
    desc = (f"first {len(sample)} scenes of the mix (seed 42; {sum(s[0].shape[0] for s in sample)} fluid particles), "
            f"1 untimed warm-up step each, then {done_steps} timed steps in all "
            f"(at most {steps_each} per scene, {per:.1f} s per scene); reference algorithm restated in C "
            f"(oracle/sph_oracle.c), FP64, OpenMP; mean {its / max(done_steps, 1):.1f} density iterations/step")
    return work / el, desc, done_steps


def run_reference_arm(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    import oracle

    # the same scenes, sampled by the oracle's own lattice and Akinci
    # samplers (equal point for point to the library's): this arm never
    # loads the CUDA library
    scenes = mix(args.warmup + args.steps, geometry=oracle)
    v, desc, done = cpu_mix_sample(scenes, max(1, args.steps), threads, args.ref_budget)
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "sample": desc,
                   "implementation": "reference algorithm restated in C (oracle/sph_oracle.c), OpenMP"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- GPU pieces --------------------------------------------------------------

def make_pool(scenes, kmax):
    import sph_gb300

    n = sum(s[0].shape[0] for s in scenes)
    nb = sum(s[1].shape[0] for s in scenes)
    return sph_gb300.Pool(max_particles=n, max_boundary=nb, max_keys=16 * n, max_scenes=len(scenes) + 1,
                          neighbor_list_max=kmax)


def scene_stats(pool, ids):
    out = []
    for sid in ids:
        st, done = pool.query(sid)
        out.append((st["sum_iterations"], st["sum_iterations_v"], st["time"], st["steps"], done))
    return out


def run_batched(scenes, args, world, local):
    """Headline: the mix resident in one pool, K graph-launched steps timed
    with CUDA events on the pool's stream, then a host-driven profiled pass."""
    import torch

    W, K, P = args.warmup, args.steps, args.profile_steps
    pool = make_pool(scenes, args.list_max)
    if args.tuning:
        b, bo, q, sb, so, w = (int(t) for t in args.tuning.split(","))
        pool.set_tuning(build_block=b, build_occupancy=bo, queue_depth=q, solver_block=sb, solver_occupancy=so,
                        scan_width=w)
    else:
        pool.set_autotune(2)  # measure launch shapes on this mix (cached afterwards)
    ids = [pool.add_scene(x, boundary_points=b, steps=TUNE_STEPS + W + K + P, **params) for x, b, params, _ in scenes]
    n = sum(s[0].shape[0] for s in scenes)
    nb = sum(s[1].shape[0] for s in scenes)
    pool.set_graph(True)
    tune_steps = pool.tune()
    tuning = dict(pool.tuning(), steps=tune_steps, log=pool.tuning_log().strip().splitlines())
    pool.step(W)
    pool.synchronize()
    s0 = scene_stats(pool, ids)
    l0 = pool.launch_count()
    dist_barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        ms = pool.step_timed(K)
    torch.cuda.synchronize()
    l1 = pool.launch_count()
    s1 = scene_stats(pool, ids)
    finished_early = sum(1 for q in s1 if q[4])
    its = sum(b[0] - a[0] for a, b in zip(s0, s1)) / (len(ids) * K)
    itsv = sum(b[1] - a[1] for a, b in zip(s0, s1)) / (len(ids) * K)
    sim = sum(b[2] - a[2] for a, b in zip(s0, s1)) / len(ids)
    pairs, overflow = pool.list_pairs()
    work = pool.count_work()  # the list build's candidates and pairs (not timed)

    # per-kernel CUDA-event timing over P host-driven steps of the same pool
    pool.set_graph(False)
    pool.set_profiling(True)
    pool.profile()
    pool.step(P)
    prof = pool.profile()
    pool.set_profiling(False)
    pool.close()
    return dict(ms=ms, n=n, nb=nb, launches=l1 - l0, clocks=clocks.summary(), its=its, itsv=itsv,
                sim_s_per_scene=sim, pairs=pairs, overflow=overflow, prof=prof, finished_early=finished_early,
                tuning=tuning, work=work)


def run_plain(scenes, args):
    """The same mix, each scene alone through the plain one-scene solver
    (graph mode), W untimed then K_plain timed steps per scene."""
    import sph_gb300

    W = args.warmup
    Kp = args.plain_steps if args.plain_steps > 0 else args.steps
    work, ms_total, its, steps_total = 0, 0.0, 0, 0
    for x, b, params, _ in scenes:
        s = sph_gb300.Scene(neighbor_list_max=args.list_max, **params)
        s.set_fluid(x)
        s.add_boundary_points(b)
        s.init()
        s.set_graph(True)
        s.step(W)
        s.synchronize()
        st0 = s.stats()
        ms_total += s.step_timed(Kp)
        st1 = s.stats()
        its += st1["sum_iterations"] - st0["sum_iterations"]
        work += s.n * Kp
        steps_total += Kp
        s.close()
    return dict(value=work / (ms_total / 1000.0), ms=ms_total, steps_per_scene=Kp, mean_iterations=its / steps_total)


def run_dam_break(args):
    """The 125k dam break alone, plain solver, L2 flushed between steps."""
    import torch

    import sph_gb300
    from sph_gb300 import workloads

    x, b, params, _ = workloads.dam_break()
    s = sph_gb300.Scene(neighbor_list_max=args.list_max, **params)
    s.set_fluid(x)
    s.add_boundary_points(b)
    s.init()
    s.set_graph(True)
    s.step(max(3, args.warmup))
    s.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    st0 = s.stats()
    ms = 0.0
    K = args.dam_steps
    for _ in range(K):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ms += s.step_timed(1)
    st1 = s.stats()
    out = dict(value=s.n * K / (ms / 1000.0), ms_per_step=ms / K, steps=K, fluid_particles=s.n,
               boundary_particles=s.nb,
               mean_density_iterations=(st1["sum_iterations"] - st0["sum_iterations"]) / K,
               mean_divergence_iterations=(st1["sum_iterations_v"] - st0["sum_iterations_v"]) / K,
               l2="flushed between timed steps (256 MB write)")
    s.close()
    return out


def run_drop(args, r=0.00275):
    """The PCISPH drop at r = 2.75 mm (489,771 fluid particles: a 9-layer
    pool and an R = 0.2 m sphere 0.6 m above it; 198,746 Akinci points),
    plain solver in graph mode, standard viscosity, Akinci surface tension
    and adhesion; L2 flushed between timed steps."""
    import torch

    import sph_gb300
    from sph_gb300 import workloads

    x, b, params, _ = workloads.pcisph_drop(r)
    s = sph_gb300.Scene(neighbor_list_max=args.list_max, **dict(params, precision="f32"))
    s.set_fluid(x)
    s.add_boundary_points(b)
    s.init()
    s.set_graph(True)
    s.step(max(3, args.warmup))
    s.synchronize()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    st0 = s.stats()
    ms = 0.0
    K = args.drop_steps
    for _ in range(K):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        ms += s.step_timed(1)
    st1 = s.stats()
    out = dict(value=s.n * K / (ms / 1000.0), unit="particle-steps/s", ms_per_step=ms / K, steps=K,
               fluid_particles=s.n, boundary_particles=s.nb, radius=r, dt=params["dt"],
               mean_pressure_iterations=(st1["sum_iterations"] - st0["sum_iterations"]) / K,
               status=st1["status"], l2="flushed between timed steps (256 MB write)")
    s.close()
    return out


def run_e2e(scenes, args):
    """The mix through the pool's C ABI with host buffers, all of it timed:
    pool creation, upload of every scene from pinned host memory, W + K steps
    with each step's per-scene completion flags read back, and the download of
    every scene's final positions and velocities into pinned host memory."""
    import torch

    import sph_gb300

    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t, t.numpy()

    hold, xs, bs, outs = [], [], [], []
    for x, b, _, _ in scenes:
        tx, ax = pinned(x)
        tb, ab = pinned(b)
        to, ao = pinned(np.empty_like(x))
        tv, av = pinned(np.empty_like(x))
        hold += [tx, tb, to, tv]
        xs.append(ax)
        bs.append(ab)
        outs.append((ao, av))
    T = args.warmup + args.steps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pool = make_pool(scenes, args.list_max)
    t_create = time.perf_counter() - t0
    ids = [pool.add_scene(x, boundary_points=b, steps=T, **params) for x, b, (_, _, params, _) in zip(xs, bs, scenes)]
    t_add = time.perf_counter() - t0 - t_create
    pool.set_graph(True)
    pool.step(0)   # admission: upload, sort, densities and lists of every scene
    pool.synchronize()
    t_setup = time.perf_counter() - t0
    polled = 0
    for _ in range(T):
        pool.step(1)
        polled += len(pool.poll())
    t_steps = time.perf_counter() - t0 - t_setup
    for sid, (ox, ov) in zip(ids, outs):
        pool.get(sid, "x", out=ox)
        pool.get(sid, "v", out=ov)
    wall = time.perf_counter() - t0
    pool.close()
    n = sum(x.shape[0] for x in xs)
    h2d = sum(x.nbytes + b.nbytes for x, b in zip(xs, bs))
    d2h = sum(ox.nbytes + ov.nbytes for ox, ov in outs) + T * len(ids) * 4
    return {"value": n * T / wall, "unit": UNIT, "h2d_bytes_per_step": h2d / T, "d2h_bytes_per_step": d2h / T,
            "wall_s": wall, "setup_s": t_setup, "create_s": t_create, "add_s": t_add, "steps_s": t_steps,
            "download_s": wall - t_setup - t_steps, "scenes_completed": polled,
            "scope": "pool create + upload from pinned host + W+K steps (completion flags read back each step) "
                     "+ download x, v of every scene into pinned host memory"}


def stream_mean_work(r=0.01):
    """E[N * steps] of the stream's regular scenes (N log-uniform in [1k, 200k],
    steps uniform in {200..2000})."""
    en = (200000 - 1000) / math.log(200000 / 1000)
    return en * 1100.0


def flat_served(plain, served, dam, drop=None):
    """The metric's served half and the plain-GPU comparison as scalar config
    keys (a record that keeps only flat keys still carries them)."""
    out = {}
    if plain:
        out["plain_gpu_pss"] = plain["value"]
    if served:
        sat = served["saturated"]
        out.update(served_pss_saturated=sat["particle_steps_per_s"], served_p50_s=sat["p50_latency_s"],
                   served_p99_s=sat["p99_latency_s"], served_completed=sat["completed"],
                   served_rejected=sat.get("rejected"), served_seconds=sat.get("duration_s"))
        sub = served.get("sub_saturation")
        if sub:
            out.update(served_pss_sub=sub["particle_steps_per_s"], served_p50_sub_s=sub["p50_latency_s"],
                       served_p99_sub_s=sub["p99_latency_s"], served_completed_sub=sub["completed"],
                       served_rate_sub_per_s=sub["rate_per_s"])
    if dam:
        out["dam_break_125k_pss"] = dam["value"]
        out["dam_break_125k_ms_per_step"] = dam["ms_per_step"]
    if drop:
        out["pcisph_drop_490k_pss"] = drop["value"]
        out["pcisph_drop_490k_ms_per_step"] = drop["ms_per_step"]
    return out


def run_served(args, rate, seconds, big_every):
    import sph_gb300
    from sph_gb300 import serve, workloads

    pool = sph_gb300.Pool(budget_bytes=int(args.serve_budget_gb * 1e9), neighbor_list_max=args.list_max)
    pool.set_graph(True)
    reqs = workloads.request_stream(rate=rate, duration=seconds, seed=7, big_every=big_every)
    out = serve.serve(pool, reqs, seconds, epoch_steps=args.epoch_steps,
                      max_queued_bytes=int(args.serve_queue_gb * 1e9))
    out.pop("request_ids", None)
    out["rate_per_s"] = rate
    out["duration_s"] = seconds
    out["budget_gb"] = args.serve_budget_gb
    out["max_queued_gb"] = args.serve_queue_gb
    out["big_dam_break_every_s"] = big_every
    pool.close()
    return out


# Instantiations of one __global__ function are one kernel, as the ncu launch
# list names them: the profile times the error passes under two names.
KERNEL_OF = {"k_pool_errors_density": "k_pool_errors", "k_pool_errors_div": "k_pool_errors"}


def profile_figures(workload):
    """Per kernel, the ncu figures the summaries under profiles/ record:
    `dram_bytes_per_launch: V` for the file's own kernel (the name between
    `ncu_` and the workload), `dram_bytes_per_launch.<kernel>: V` for another
    kernel of the same capture, and the issue utilisations."""
    out = {}
    d = os.path.join(ROOT, "profiles")
    suffix = f"_{workload}.md"
    for fn in sorted(os.listdir(d)) if os.path.isdir(d) else []:
        if not (fn.startswith("ncu_") and fn.endswith(suffix)):
            continue
        own = fn[len("ncu_"):-len(suffix)]
        for ln in open(os.path.join(d, fn)):
            key, _, val = ln.partition(":")
            key, _, other = key.strip().partition(".")
            if key not in ("dram_bytes_per_launch", "sm_issue_active_pct", "l1_lsu_wavefronts_pct", "fp32_pipe_pct"):
                continue
            try:
                v = float(val)
            except ValueError:
                continue
            k = other or own
            out.setdefault(k, {"source": os.path.join("profiles", fn)})[key] = v
    return out


def fp32_peak_tflops():
    """FP32 (non-tensor) throughput of this GPU, measured: an 8192^3 FP32
    matrix product with TF32 off (cuBLAS SGEMM on the FMA pipe), best of 5,
    CUDA events."""
    import torch

    prev = torch.get_float32_matmul_precision()
    torch.set_float32_matmul_precision("highest")
    try:
        n = 8192
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        c = torch.empty_like(a)
        for _ in range(2):
            torch.matmul(a, b, out=c)
        best = float("inf")
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b, c
        return 2.0 * n ** 3 / (best / 1000.0) / 1e12
    finally:
        torch.set_float32_matmul_precision(prev)


# FP32 work of one list-build launch: 8 flop per candidate for the distance
# test (3 subtractions, r^2 by 3 multiply-adds, the compare), 12 for W plus 22
# for grad W and the accumulations per pair within h (fluid and boundary), and
# 6 for the fused divergence term per fluid pair (3 subtractions, 3 multiply-adds).
def build_flops(work):
    return (8 * (work["fluid_candidates"] + work["boundary_candidates"])
            + 34 * (work["fluid_pairs"] + work["boundary_pairs"]) + 6 * work["fluid_pairs"])


def roofline(prof, n, nb, pairs, workload, work=None, fp32_peak=None):
    """HBM roofline of the kernel with the largest share of the profiled
    steps (`kernel`), and the same figures for the three largest in
    `kernels`.  Algorithmic bytes: compulsory field bytes per particle
    (ALGO_BYTES) x particles, plus 16 B per boundary particle for walks that
    touch the boundary; `with_pair_lists` adds the 16-byte pair records a
    list kernel writes or reads."""
    peak, peak_kind = load_peaks()
    figs = profile_figures(workload)
    groups = {}
    for name, (count, ms) in prof.items():
        groups.setdefault(KERNEL_OF.get(name, name), []).append((name, count, ms))
    total = sum(ms for _, ms in prof.values())

    def one(kname, entries):
        count = sum(c for _, c, _ in entries)
        ms = sum(m for _, _, m in entries)
        algo = sum(c * (n * ALGO_BYTES.get(e, (0, False, 0))[0] + (nb * 16 if ALGO_BYTES.get(e, (0, False, 0))[1] else 0))
                   for e, c, _ in entries)
        stream = algo + sum(c * pairs * ALGO_BYTES.get(e, (0, False, 0))[2] for e, c, _ in entries)
        avg_ms = ms / max(count, 1)
        bytes_launch = algo / max(count, 1)
        stream_launch = stream / max(count, 1)
        achieved = bytes_launch / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else 0.0
        streamed = stream_launch / (avg_ms / 1000.0) / 1e9 if avg_ms > 0 else 0.0
        f = figs.get(kname, {})
        r = {"kernel": kname, "achieved": achieved, "frac": achieved / peak, "traffic": f.get("dram_bytes_per_launch"),
             "algorithmic_bytes_per_launch": bytes_launch, "avg_launch_ms": avg_ms, "launches": count,
             "kernel_share": ms / total if total else None,
             "with_pair_lists": {"bytes_per_launch": stream_launch, "achieved": streamed, "frac": streamed / peak,
                                 "note": "field bytes plus the 16-byte pair records the kernel writes or reads"}}
        issue = {k: v for k, v in f.items() if k in ("sm_issue_active_pct", "l1_lsu_wavefronts_pct", "fp32_pipe_pct")}
        if issue:
            # a neighbour walk is bound by instruction issue and the L1 load
            # pipe, not by DRAM: the utilisations ncu measured for this kernel
            r["issue"] = dict(issue, source=f["source"])
        if f.get("source"):
            r["profile"] = f["source"]
        if kname == "k_pool_build_lists" and work and fp32_peak and avg_ms > 0:
            # the neighbour walks' second bound: FP32 issue
            flops = build_flops(work)
            tf = flops / (avg_ms / 1000.0) / 1e12
            r["fp32"] = {"achieved": tf, "peak": fp32_peak, "unit": "TFLOP/s", "frac": tf / fp32_peak,
                         "peak_kind": "of measured (FP32 SGEMM, TF32 off)", "flops_per_launch": flops,
                         "candidates_per_particle": (work["fluid_candidates"] + work["boundary_candidates"]) / max(n, 1),
                         "pairs_per_particle": (work["fluid_pairs"] + work["boundary_pairs"]) / max(n, 1),
                         "formula": "8 per candidate + 34 per pair within h + 6 per fluid pair (fused divergence)"}
        return r

    ranked = sorted(groups.items(), key=lambda kv: -sum(m for _, _, m in kv[1]))
    if not ranked:
        return {"bound": "hbm", "kernel": "none", "achieved": 0.0, "peak": peak, "unit": "GB/s", "frac": 0.0,
                "peak_kind": f"of {peak_kind}", "traffic": None}
    top = one(*ranked[0])
    out = {"bound": "hbm", "kernel": top.pop("kernel"), "achieved": top.pop("achieved"), "peak": peak, "unit": "GB/s",
           "frac": top.pop("frac"), "peak_kind": f"of {peak_kind}", "traffic": top.pop("traffic")}
    out.update(top)
    out["kernels"] = [one(k, e) for k, e in ranked[:3]]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=495)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--list-max", type=int, default=64, help="pair-list slots per particle")
    ap.add_argument("--tuning", default="", help="fixed launch shapes: build block,build occupancy,queue,solver block,"
                                                 "solver occupancy,scan width (skips the autotuner)")
    ap.add_argument("--scenes", type=int, default=256, help="first N scenes of the mix (256: the full workload)")
    ap.add_argument("--profile-steps", type=int, default=10, help="host-driven steps timed per kernel")
    ap.add_argument("--plain-steps", type=int, default=0, help="timed steps per scene for the plain arm (0: --steps)")
    ap.add_argument("--dam-steps", type=int, default=500)
    ap.add_argument("--drop-steps", type=int, default=1000, help="timed steps of the 490k PCISPH drop")
    ap.add_argument("--serve-seconds", type=float, default=30.0)
    ap.add_argument("--serve-budget-gb", type=float, default=80.0)
    ap.add_argument("--serve-queue-gb", type=float, default=16.0,
                    help="host bytes of queued requests beyond which submissions are refused")
    ap.add_argument("--epoch-steps", type=int, default=10)
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-sub-saturation", action="store_true", help="served: only the 200 scenes/s stream")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="arrival rate of the first served stream (scenes/s)")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-dam", action="store_true")
    ap.add_argument("--no-drop", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=25.0, help="seconds of CPU baseline work")
    ap.add_argument("--ref-budget", type=float, default=90.0, help="seconds of reference-arm timed work")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
        return

    import torch

    import sph_gb300

    sph_gb300.build()
    sph_gb300.select_device(local)
    torch.cuda.set_device(local)
    wall0 = time.perf_counter()

    scenes = mix(args.warmup + args.steps)[: args.scenes]
    workload = WORKLOAD if args.scenes == 256 else f"batched_mix_{args.scenes}"
    B = run_batched(scenes, args, world, local)
    t_max = dist_max(B["ms"], world)
    value = world * B["n"] * args.steps / (t_max / 1000.0)
    try:
        fp32 = fp32_peak_tflops()
    except RuntimeError as e:  # e.g. no room for the three 256 MB matrices: no FP32 view
        print(f"FP32 peak not measured: {e}", file=sys.stderr)
        fp32 = None
    roof = roofline(B["prof"], B["n"], B["nb"], B["pairs"], workload, work=B.get("work"), fp32_peak=fp32)
    roof["timing"] = f"CUDA events around each launch, {args.profile_steps} host-driven pool steps"

    plain = None if args.no_plain else run_plain(scenes, args)
    dam = None if args.no_dam else run_dam_break(args)
    drop = None if args.no_drop else run_drop(args)
    e2e = None if args.no_e2e else run_e2e(scenes, args)
    if e2e is not None:
        e2e["value"] = world * e2e["value"] * e2e["wall_s"] / dist_max(e2e["wall_s"], world)

    served = None
    if not args.no_served and world == 1:
        big_load = 4_000_000 * 200 / 10.0
        sub_rate = max(0.5, (0.5 * value - big_load) / stream_mean_work())
        served = {"saturated": run_served(args, args.serve_rate, args.serve_seconds, 10.0)}
        if not args.no_sub_saturation:
            served["sub_saturation"] = run_served(args, round(sub_rate, 2), args.serve_seconds, 10.0)
            served["sub_saturation_rate_rule"] = "offered load = half the batched value, 4M dam break included"

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, desc, _ = cpu_mix_sample(scenes, 50, threads, args.cpu_budget)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scenes)",
            "config": {"workload": workload, "scenes": len(scenes), "fluid_particles": B["n"],
                       "boundary_particles": B["nb"],
                       "steps_per_scene": f"{B['tuning']['steps']} autotuning + {args.warmup} warm-up + {args.steps} "
                                          f"timed + {args.profile_steps} profiled",
                       "autotuner": B["tuning"],
                       "parallelism": f"replicas x{world}",
                       "l2": "not flushed: the resident working set (pair lists ~4 GB) is far larger than L2",
                       "step_timing": "CUDA events on the pool's stream around the K graph-launched steps",
                       "mean_density_iterations": B["its"], "mean_divergence_iterations": B["itsv"],
                       "simulated_seconds_per_scene": B["sim_s_per_scene"],
                       "neighbor_list_max": args.list_max, "list_pairs": B["pairs"],
                       "list_overflow": B["overflow"], "scenes_finished_early": B["finished_early"],
                       "plain_gpu": plain,
                       "batched_over_plain": value / plain["value"] if plain else None,
                       "served": served, "dam_break_125k": dam, "pcisph_drop_490k": drop,
                       **flat_served(plain, served, dam, drop),
                       "wall_s": time.perf_counter() - wall0},
            "roofline": roof,
            "clocks": B["clocks"],
            "gpu_launches": B["launches"],
            "e2e": e2e,
            "cpu_baseline": cpu,
            "kernels": {k: {"launches": c, "ms": round(ms, 4)} for k, (c, ms) in sorted(B["prof"].items(),
                                                                                      key=lambda kv: -kv[1][1])},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
