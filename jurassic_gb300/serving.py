"""Retrieval serving on one device: a request loop over the continuous-
batching engine (``jgb_engine_*``).

Requests (a-priori atmosphere + measurement of one observation) arrive as a
Poisson stream; each arrival is submitted at once, the engine admits it as
soon as a slot and working-set memory are free, and every engine step moves
all admitted requests one Levenberg-Marquardt iteration forward.  The loop
records, per request, the time from arrival to its results being back on the
host; it reports retrievals/s and latency percentiles.

This replaces the reference's retrieval driver, which runs one
optimal_estimation per process over a list of directories
(retrieval.c:148-245).
"""
from __future__ import annotations

import time
from typing import Sequence

import numpy as np

from . import synth


def serve(engine, ctl, requests: Sequence, rate_hz: float, seed: int = 0,
          clock=time.perf_counter) -> dict:
    """Run ``requests`` (list of (Atm, Obs)) through ``engine`` with Poisson
    arrivals at ``rate_hz`` (``inf``: all arrive at t=0, closed loop).
    Returns throughput, latency percentiles and per-request results."""
    n = len(requests)
    rng = np.random.default_rng(seed)
    if np.isfinite(rate_hz):
        arrivals = np.cumsum(rng.exponential(1.0 / rate_hz, n))
        arrivals -= arrivals[0]
    else:
        arrivals = np.zeros(n)
    owner, arrival_of = {}, {}
    latency = np.full(n, np.nan)
    results = [None] * n
    nxt, done, steps = 0, 0, 0
    t0 = clock()
    while done < n:
        now = clock() - t0
        k = nxt
        while k < n and arrivals[k] <= now:
            k += 1
        if k > nxt:
            ids = engine.submit(synth.pack(ctl, [requests[j] for j in range(nxt, k)]))
            for j, rid in zip(range(nxt, k), ids):
                owner[rid] = j
                arrival_of[rid] = arrivals[j]
            nxt = k
        st = engine.stats()
        if st["active"] or st["queued"]:
            engine.step()
            steps += 1
        elif nxt < n:
            time.sleep(max(0.0, arrivals[nxt] - (clock() - t0)))
        for rid in engine.finished():
            j = owner.pop(rid)
            results[j] = engine.result(rid)
            latency[j] = (clock() - t0) - arrival_of.pop(rid)
            done += 1
    wall = clock() - t0
    est = engine.stats()
    lat_ms = latency * 1e3
    return dict(n=n, wall_s=wall, retrievals_per_s=n / wall,
                p50_ms=float(np.percentile(lat_ms, 50)), p99_ms=float(np.percentile(lat_ms, 99)),
                mean_ms=float(np.mean(lat_ms)), rate_hz=float(rate_hz), steps=steps,
                iters_mean=float(np.mean([r["iters"] for r in results])),
                failed=int(sum(1 for r in results if r["status"])),
                engine={k: est[k] for k in ("steps", "rebuilds", "forward_calls", "lm_trials",
                                            "jacobians", "step_ms", "rebuild_ms", "init_ms",
                                            "jacobian_ms", "normal_ms", "trial_ms",
                                            "finish_ms", "trial_fwd_ms", "trial_trace_ms",
                                            "trial_path_ms")},
                results=results)


def stream_workload(seed=5):
    """Retrieval serving stream: a 300-channel context (650-2400 cm^-1,
    CO2 + H2O + O3); T retrieved on 0-60 km and H2O on 0-20 km; diagonal S_a
    (2 K, 30 %, 3 km vertical correlation length without a horizontal one,
    so no correlation, retrieval.c:901), up to 10 LM iterations, kernel
    recomputed every iteration, covariance and averaging-kernel analysis on.
    Returns (ctl, ret, tables, filters)."""
    from .model import Ctl, Ret
    ctl = Ctl(emitter=["CO2", "H2O", "O3"], nu=np.linspace(650.0, 2400.0, 300))
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 60.0
    ctl.retq_zmin = np.array([-999.0, 0.0, -999.0])
    ctl.retq_zmax = np.array([-999.0, 20.0, -999.0])
    ret = Ret(kernel_recomp=1, conv_itmax=10, conv_dmin=0.1, err_ana=1,
              err_noise=np.full(ctl.nd, 1e-4), err_formod=np.full(ctl.nd, 0.5),
              err_temp=2.0, err_temp_cz=3.0, err_temp_ch=-999.0,
              err_q=np.array([0.0, 30.0, 0.0]), err_q_cz=np.array([-999.0, 3.0, -999.0]),
              err_q_ch=np.array([-999.0, -999.0, -999.0]))
    return ctl, ret, synth.make_tables(ctl, seed + 100), synth.make_filters(ctl)


def stream_requests(ctl, forward, n, seed=55):
    """n requests of the serving stream: 50-300 measured channels (seeded),
    41-101 levels on 0-100 km, nadir (1 ray) and limb (5 rays) alternating;
    ``forward`` computes the measurements of the truth batch."""
    rng = np.random.default_rng(seed)
    nch = rng.integers(50, 301, n)
    return synth.retrieval_requests(ctl, forward, n, seed, nlev=(41, 101), ztop=100.0, nch=nch,
                                    limb_rays=5)


def main(argv=None):
    """Closed-loop run of the serving stream: ``python -m
    jurassic_gb300.serving --requests N [--precision mixed|fp64]
    [--marker]``.  Serves N requests after a 4-request warm-up and prints
    one JSON line (wall time, steps, retrievals/s, engine phase times).
    --marker launches a short measurement kernel (jgb_measure_l2_read)
    just before the timed run, so that a profiler's launch list can be cut
    there."""
    import argparse
    import ctypes
    import json

    from . import native
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--marker", action="store_true")
    a = ap.parse_args(argv)
    prec = native.MIXED if a.precision == "mixed" else native.FP64
    ctl, ret, tables, filters = stream_workload()
    ctx = native.Context(ctl, tables, filters)
    reqs = stream_requests(ctl, lambda b: ctx.formod_batch(b.fresh_outputs(), native.FP64),
                           a.requests)
    serve(ctx.engine(ret, prec), ctl, reqs[:4], np.inf)   # warm-up (autotuner, allocations)
    eng = ctx.engine(ret, prec)
    if a.marker:
        g = ctypes.c_double(0.0)
        native.load().jgb_measure_l2_read(1 << 20, 1, ctypes.byref(g))
    r = serve(eng, ctl, reqs, np.inf)
    print(json.dumps({k: v for k, v in r.items() if k != "results"}), flush=True)
    eng.close()
    ctx.close()


if __name__ == "__main__":
    main()
