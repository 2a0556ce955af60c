"""Serving a stream of DFSPH scene requests from one device-resident pool.

The request loop itself is the library's (``sph_server_*``, C++): a driver
thread steps the pool in epochs, admits waiting scenes as the pool's
device-memory budget frees up (first come first served, with a look-ahead
so one large scene does not block smaller ones behind it), overlaps that
host work with the epoch running on the device, and retires each scene
when its step count completes (continuous batching).  This module is the
client side of a benchmark: it submits each request of a stream at its
arrival time, building the scene just then, and reports completed scenes,
latency percentiles (submission to completion) and aggregate
particle-steps/s.
"""
from __future__ import annotations

import time

from . import Server


def serve(pool, requests, duration, epoch_steps=10, lookahead=8, keep_results=False, max_queued_bytes=0):
    """Submit the stream [(arrival_s, builder)] (builder() -> (x, boundary
    points, params, steps)) at its arrival times for `duration` seconds of
    wall time, then stop the server.  Requests refused because the queue
    holds max_queued_bytes (0: no bound) are counted as rejected.  Returns a
    summary dict (with the server when keep_results is set, so completed
    results can be fetched)."""
    srv = Server(pool, epoch_steps=epoch_steps, lookahead=lookahead, keep_results=keep_results,
                 max_queued_bytes=max_queued_bytes)
    t0 = time.perf_counter()
    arrived = 0
    late = 0.0
    ids = []
    for arrival, builder in requests:
        if arrival > duration:
            break
        now = time.perf_counter() - t0
        if arrival > now:
            time.sleep(arrival - now)
        else:
            late = max(late, now - arrival)
        x, b, params, steps = builder()
        rid = srv.submit(x, boundary_points=b, steps=steps, **params)
        if rid is not None:
            ids.append(rid)
        arrived += 1
    rest = duration - (time.perf_counter() - t0)
    if rest > 0:
        time.sleep(rest)
    st = srv.stats()
    out = dict(
        wall_s=st["wall_s"], arrived=arrived, admitted=st["admitted"], completed=st["completed"],
        waiting=st["queued"], resident=st["resident"], failed=st["failed"], epochs=st["epochs"],
        rejected=st["rejected"], queued_bytes=st["queued_bytes"],
        particle_steps=st["particle_steps"], particle_steps_per_s=st["particle_steps_per_s"],
        p50_latency_s=st["p50_latency_s"] if st["completed"] else None,
        p99_latency_s=st["p99_latency_s"] if st["completed"] else None,
        mean_latency_s=st["mean_latency_s"] if st["completed"] else None,
        max_submit_lag_s=late, request_ids=ids,
    )
    if keep_results:
        out["server"] = srv
    else:
        srv.close()
    return out
