"""Request loop serving DFSPH scenes from one device-resident pool.

Scenes arrive over time; the loop admits waiting scenes whenever they fit the
pool's device-memory budget (first come first served, with a short look-ahead
so one large scene does not block smaller ones behind it), advances every
resident scene together in epochs of pool steps (continuous batching: new
scenes join between steps while others are mid-run), and retires each scene
when its step count completes.  Reported: completed scenes, per-scene
latency (arrival to completion) percentiles, and aggregate particle-steps/s.
"""
from __future__ import annotations

import collections
import time

import numpy as np

from . import Pool, PoolFull


def serve(pool: Pool, requests, duration, epoch_steps=10, lookahead=8, keep_results=False):
    """Run the request stream [(arrival_s, builder)] for at most `duration`
    seconds of wall time.  Returns a summary dict."""
    t0 = time.perf_counter()
    waiting = collections.deque()
    resident = {}          # scene id -> (arrival, n, steps)
    latencies, done_ps, results = [], 0, {}
    ri = 0
    admitted = 0
    while True:
        now = time.perf_counter() - t0
        while ri < len(requests) and requests[ri][0] <= now:
            waiting.append(tuple(requests[ri]))
            ri += 1
        # admission by the pool's capacity (device-memory budget)
        k = 0
        while waiting and k < min(lookahead, len(waiting)):
            req = waiting[k]
            if len(req) == 2:  # build the scene once, on first consideration
                req = waiting[k] = (req[0], req[1](), 0)
            arrival, (x, b, params, steps), _ = req
            try:
                sid = pool.add_scene(x, boundary_points=b, steps=steps, **params)
            except PoolFull:
                k += 1
                continue
            del waiting[k]
            resident[sid] = (arrival, x.shape[0], steps)
            admitted += 1
        if not resident:
            if ri >= len(requests) and not waiting:
                break
            if now >= duration:
                break
            nxt = requests[ri][0] if ri < len(requests) else now + 0.01
            time.sleep(max(0.0, min(nxt - now, 0.01)))
            continue
        pool.step(epoch_steps)
        pool.synchronize()
        tnow = time.perf_counter() - t0
        for sid in pool.poll():
            arrival, n, steps = resident.pop(sid)
            latencies.append(tnow - arrival)
            done_ps += n * steps
            if keep_results:
                results[sid] = pool.get(sid, "x")
            pool.remove(sid)
        if tnow >= duration:
            break
    wall = time.perf_counter() - t0
    partial = 0
    for sid, (arrival, n, steps) in resident.items():
        st, _ = pool.query(sid)
        partial += n * st["steps"]
    lat = np.asarray(latencies) if latencies else np.zeros(1)
    return dict(
        wall_s=wall, arrived=ri, admitted=admitted, completed=len(latencies), waiting=len(waiting),
        resident=len(resident), particle_steps=done_ps + partial,
        particle_steps_per_s=(done_ps + partial) / wall if wall > 0 else 0.0,
        p50_latency_s=float(np.percentile(lat, 50)) if latencies else None,
        p99_latency_s=float(np.percentile(lat, 99)) if latencies else None,
        results=results,
    )
