"""Generate tests/golden/longrun_stats.npz: long-run statistics of the two
full-size single-scene workloads, from the oracle (the C restatement pinned
bit for bit to the reference build), so that the GPU test compares against a
committed fixture and runs for seconds.

Cases (both on lattices jittered by U(-0.01 r, 0.01 r), so that no pair sits
at exactly q = 1, where the last bit of a coordinate decides membership):
  * dam_break_125k: DFSPH dam break, 50^3 = 125,000 particles at r = 5 mm in a
    1.5 x 0.8 x 0.8 m Akinci box, CFL-adaptive dt in [1e-5, 5e-3] s, density
    and divergence tolerance 0.1 %; checkpoints at the simulated times the
    oracle reaches after 500, 1000 and 2000 steps;
  * pcisph_drop_81k: PCISPH drop (5-layer pool + R = 0.2 m sphere 0.6 m above
    it, 81,421 particles at r = 5 mm), standard viscosity 0.01, Akinci surface
    tension 0.5 and adhesion 0.1, fixed dt 1e-4 s; checkpoints after 1000,
    2500 and 3500 steps (the sphere meets the pool at about 0.29 s, so the
    last checkpoint is 60 ms into the splash).

Statistics per checkpoint (STATS): kinetic energy per unit mass
0.5 <|v|^2>, centre of mass (3), the mean, 99.9th and 99.99th percentile and
maximum of the relative density deviation (rho - rho0)/rho0, and the
simulated time.  Besides the base run, three perturbed oracle runs give the
statistics' sensitivity to rounding-sized changes: the initial positions
perturbed once by U(-1e-6 r, 1e-6 r) (two seeds), and the positions
perturbed after every step by U(-2e-7 r, 2e-7 r) (about the rounding of an
FP32 cell-relative coordinate).  "spread" is the largest absolute difference
of a perturbed run from the base run (kinetic energy relative to the base).
Every run stops at the same step counts; "time_mismatch" is the largest
relative difference of a perturbed run's time there from the base's (0 when,
as here, the perturbed runs take the same time steps).

    Eight processes of one OpenMP thread, all runs at once.
    python tests/golden/make_longrun_stats.py
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "longrun_stats.npz")

PERTURB = (("once", 1e-6, 11), ("once", 1e-6, 12), ("every", 2e-7, 13))


def case_inputs(name):
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from scenes import jitter
    from sph_gb300 import workloads

    if name == "dam_break_125k":
        x, b, p, _ = workloads.dam_break()
        x = jitter(x, p["radius"], 17)
        marks = ("steps", (500, 1000, 2000))
    else:
        x, b, p, _ = workloads.pcisph_drop()
        x = jitter(x, p["radius"], 31)
        marks = ("steps", (1000, 2500, 3500))
    return x, b, {k: v for k, v in p.items() if k != "precision"}, marks


STATS = ("ke", "com_x", "com_y", "com_z", "mean_dev", "p999_dev", "p9999_dev", "max_dev", "time")


def stats(o, rho0=1000.0):
    x, v, rho = o.get("x"), o.get("v"), o.get("rho")
    com = x.mean(0)
    dev = (rho - rho0) / rho0
    q = np.quantile(dev, [0.999, 0.9999])
    return np.array([0.5 * float(np.mean((v * v).sum(1))), com[0], com[1], com[2], float(np.mean(dev)), float(q[0]),
                     float(q[1]), float(np.max(dev)), o.scalar("time")])


def run(job):
    """One oracle run to the case's step marks."""
    name, perturb, threads = job
    os.environ["OMP_NUM_THREADS"] = str(threads)
    sys.path.insert(0, ROOT)
    import oracle

    x, b, p, (_, marks) = case_inputs(name)
    o = oracle.OracleScene(p, x, points=b)
    kind, amp, seed = perturb if perturb else (None, 0.0, 0)
    if kind == "once":
        o.perturb(amp * p["radius"], 0.0, seed)
    rows, steps = [], []
    t0 = time.time()
    for k, m in enumerate(marks):
        while o.scalar("steps") < m:
            o.step(1)
            if kind == "every":
                o.perturb(amp * p["radius"], 0.0, seed * 100000 + int(o.scalar("steps")))
        rows.append(stats(o))
        steps.append(int(o.scalar("steps")))
        print(f"{name} {perturb}: mark {m} at step {steps[-1]}, t {rows[-1][-1]:.5f} ({time.time() - t0:.0f} s)",
              flush=True)
    return name, perturb, np.array(rows), np.array(steps)


def main():
    ctx = mp.get_context("spawn")
    cases = ("dam_break_125k", "pcisph_drop_81k")
    out = {"stats": np.array(STATS)}
    # a fresh process per run, so that each reads its own OMP_NUM_THREADS
    jobs = [(nm, pt, 1) for nm in cases for pt in (None,) + PERTURB]
    with ctx.Pool(len(jobs), maxtasksperchild=1) as pool:
        res = pool.map(run, jobs, chunksize=1)
    ns = len(STATS) - 1
    for nm in cases:
        b = next(rows for rn, pt, rows, _ in res if rn == nm and pt is None)
        d = np.zeros((b.shape[0], ns))
        tm = 0.0
        for rn, pt, rows, _ in res:
            if rn != nm or pt is None:
                continue
            diff = np.abs(rows[:, :ns] - b[:, :ns])
            diff[:, 0] /= np.abs(b[:, 0])
            d = np.maximum(d, diff)
            tm = max(tm, float(np.max(np.abs(rows[:, ns] - b[:, ns]) / b[:, ns])))
        _, _, _, (_, marks) = case_inputs(nm)
        out[f"{nm}.marks"] = np.array(marks)
        out[f"{nm}.base"] = b
        out[f"{nm}.spread"] = d
        out[f"{nm}.time_mismatch"] = np.array([tm])
        print(nm, "base", b, "spread", d, "time mismatch", tm, sep="\n")
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
