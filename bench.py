#!/usr/bin/env python3
"""Benchmark: ray-channel radiances/s of the batched forward model on one GB300.

Workload (default): batched nadir forward model, 1e5 observations from
705 km, 101 levels on 0-100 km, 100 channels on 650-2400 cm^-1, 5 emitters
(CO2, H2O, O3, CH4, N2O), EGA, seeded synthetic atmospheres and tables
(~1.6 GB of float32 emissivity tables).  One step = one forward-model call
over the whole batch (ray tracing + path loop + epilogue).

Reported line (one JSON object, rank 0):
  value        mixed-precision path, inputs resident in GPU memory
  e2e          same through jgb_formod_batch with page-locked host buffers,
               host->device and device->host copies inside the timed region
  fp64         the plain FP64 GPU form (rounding-level agreement with the
               reference) on the same batch
  roofline     path kernel: warp-instruction issue rate against the SMs'
               issue peak at the sampled clock (the bound ncu shows), with
               the compulsory-byte HBM fraction beside it
  cpu_baseline the CPU oracle (restatement of the reference) on a bounded,
               stratified sample of the same workload with all host threads
  accuracy     |BT_mixed - BT_oracle| and FP64 relative error on that sample
  limb_cga     the uneven limb CGA batch (2e4 observations, 32 channels,
               3 emitters, 50-400 LOS points per ray): mixed and FP64
               radiances/s, accuracy against the oracle
  jacobian     the batched FD Jacobian (2048 nadir profiles x 405 state
               elements, 150 channels) and its 3xTF32 normal equations
  serving      retrieval stream: retrievals/s, p50/p99 latency, mixed/FP64

--impl reference times the reference's CPU implementation instead (the
reference build when present, else the CPU restatement) on a bounded sample.
Multi-GPU (torchrun): independent replicas, weak scaling, max time over ranks.
"""
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

METRIC = "ray-channel radiances/s"
UNIT = "ray-channel radiances/s"


def dist_setup(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as td
        td.init_process_group("gloo")
        pg = td
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ncu counters of k_path_mixed per LOS point of the nadir workload (all 100
# channels, 5 emitters), from one capture of the 4000-observation launch
# with the same channels, emitters and tables (the nadir observations are
# alike, so the counters scale with the LOS points):
#   JGB_PATH_VARIANT=14 ncu --set full --clock-control none -k regex:k_path_mixed \
#       -s 1 -c 1 -o path python bench.py --nobs 4000 --steps 2 --warmup 1 \
#       --fp64-steps 0 --no-cpu --serve-requests 0 --no-extra
#   (variant 14: the one the autotuner picks on the 1e5-observation launch)
#   smsp__inst_executed.sum 3.2978e10, dram__bytes_read.sum + write.sum 862.5 MB,
#   4,004,179 LOS points in the launch.
PATH_NCU_NADIR = {"warp_inst_per_los_point": 32978257734 / 4004179,
                  "dram_bytes_per_los_point": 862.547456e6 / 4004179}


def sm_count(device=0):
    """Multiprocessors of the device (CUDA runtime attribute 16)."""
    import ctypes
    rt = ctypes.CDLL("libcudart.so.13")
    v = ctypes.c_int(0)
    if rt.cudaDeviceGetAttribute(ctypes.byref(v), 16, device) != 0:
        return None
    return v.value


def path_fields(ctl):
    """Float fields per LOS point of the path kernel's tile planes: p, t, ds,
    q_H2O, cloud factor, extinction per window, and per emitter its column
    (plus the CG pressure, temperature and column in CGA), the p-T cell's
    rows and the pressure and two temperature interpolation weights."""
    return 5 + ctl.nw + ctl.ng * (8 if ctl.formod == 0 else 5)


def compulsory_bytes(ctl, tables, los_points, nray):
    """Bytes the path kernel cannot avoid moving: its LOS inputs once (FP32
    fields per point), every table entry once ({u, eps} float pairs and the
    row records), the source-function table, and the FP64 radiance and
    transmittance of every ray-channel."""
    tp, tt, tu = tables.u.shape[2:]
    rows = ctl.nd * ctl.ng * tp * tt
    rec = 32 if ctl.formod == 1 else 16
    return (float(los_points) * path_fields(ctl) * 4 + rows * (tu * 8 + rec)
            + ctl.nd * 1200 * 4 + float(nray) * ctl.nd * 16)


def issue_roofline(los_points, path_ms, sm_mhz, sms, ctl, tables, nray, hbm, hbm_kind):
    """Binding roofline of k_path_mixed: warp instructions issued per second
    (ncu instructions per LOS point x the launch's LOS points / CUDA-event
    time) against the issue peak of the SMs (4 schedulers x SMs x the SM
    clock sampled during the timed region); the compulsory-byte HBM
    fraction beside it."""
    inst = PATH_NCU_NADIR["warp_inst_per_los_point"] * los_points
    t = path_ms / 1e3
    achieved = inst / t / 1e9
    peak = 4.0 * sms * sm_mhz * 1e6 / 1e9 if sm_mhz and sms else None
    comp = compulsory_bytes(ctl, tables, los_points, nray)
    return {"bound": "issue", "kernel": "k_path_mixed", "achieved": achieved,
            "peak": peak, "unit": "G warp-instructions/s",
            "frac": achieved / peak if peak else None,
            "traffic": PATH_NCU_NADIR["dram_bytes_per_los_point"] * los_points,
            "traffic_note": "ncu dram__bytes_read+write per LOS point (4000-observation capture) "
                            "x LOS points of this launch",
            "warp_instructions_per_launch": inst,
            "peak_note": "4 warp schedulers x %d SMs x %.0f MHz (median SM clock sampled in "
                         "the timed region)" % (sms or 0, sm_mhz or 0),
            "hbm": {"bound": "hbm", "achieved": comp / t / 1e9, "peak": hbm, "unit": "GB/s",
                    "frac": comp / t / 1e9 / hbm, "peak_kind": hbm_kind,
                    "bytes_per_launch": comp,
                    "bytes_note": "compulsory: LOS inputs once (%d FP32 fields per point), every "
                                  "table entry and row record once, source function, FP64 "
                                  "rad+tau per ray-channel" % path_fields(ctl)}}


def build_workload(args):
    from jurassic_gb300 import synth
    if args.workload == "nadir":
        return synth.config_nadir(args.nobs)
    if args.workload == "limb_cga":
        return synth.config_limb_cga(args.nobs)
    raise SystemExit("unknown workload " + args.workload)


SAMPLE_SEED = 11


def stratified_indices(nobs, n, seed=SAMPLE_SEED):
    """One observation drawn uniformly from each of n equal strata of the
    batch (numpy default_rng(seed)), ascending."""
    n = max(1, min(n, nobs))
    rng = np.random.default_rng(seed)
    edges = (np.arange(n + 1, dtype=np.int64) * nobs) // n
    return edges[:-1] + (rng.random(n) * (edges[1:] - edges[:-1])).astype(np.int64)


def sample_batch(w, idx):
    from jurassic_gb300 import synth
    b = w.batch
    return synth.pack(w.ctl, [b.item(w.ctl, int(i)) for i in idx])


def sample_rays(b, idx):
    """Ray indices of the sampled observations, in sample order."""
    return np.concatenate([np.arange(b.ray_off[i], b.ray_off[i + 1]) for i in idx])


def sample_record(idx, nobs):
    import hashlib
    idx = np.asarray(idx, dtype=np.int64)
    return {"rule": "stratified: one observation uniform in each of %d equal strata of the "
                    "%d observations, numpy default_rng(%d)" % (len(idx), nobs, SAMPLE_SEED),
            "observations": int(len(idx)), "indices_head": idx[:12].tolist(),
            "indices_tail": idx[-4:].tolist(),
            "indices_sha256": hashlib.sha256(idx.tobytes()).hexdigest()[:16]}


def time_cpu(w, ora, target_s, threads, n0=8):
    """Time the oracle on a growing stratified sample until ~target_s of work.
    Returns (indices, sample batch, oracle output, seconds)."""
    n = n0
    while True:
        idx = stratified_indices(w.batch.nobs, n)
        s = sample_batch(w, idx)
        t0 = time.perf_counter()
        out = ora.formod_batch(s.fresh_outputs(), nthreads=threads)
        dt = time.perf_counter() - t0
        if dt >= target_s or n >= w.batch.nobs:
            return idx, s, out, dt
        n = min(w.batch.nobs, max(n * 2, int(n * target_s / max(dt, 1e-3) * 1.05)))


def run_reference(args, rank):
    if rank != 0:
        return
    from oracle import oracle
    w = build_workload(args)
    threads = os.cpu_count() or 1
    kind = "port"
    ora = oracle.Oracle(w.ctl, w.tables, w.filters)
    per_step = []
    sample_n = None
    for step in range(args.warmup + args.steps):
        idx, s, out, dt = time_cpu(w, ora, args.cpu_seconds / max(args.steps, 1), threads)
        sample_n = s.nobs
        if step >= args.warmup:
            per_step.append(dt)
    units = s.nray * w.ctl.nd
    value = units / statistics.mean(per_step)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * statistics.mean(per_step), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w.name, "sample_observations": sample_n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": "%d of %d observations (stratified over the batch) x %d "
                                       "channels per step" % (sample_n, w.batch.nobs, w.ctl.nd)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def jacobian_measure(local, nobs, steps, warmup, fp64_nobs, pg=None, world=1):
    """Batched FD Jacobian + normal equations (kernel(), jurassic.c:4004-4099,
    and K^T Se^-1 K, retrieval.c:403-444) of the Jacobian workload, Se
    diagonal from a 0.2 K noise-equivalent brightness temperature at 250 K.
    The mixed form runs on all nobs profiles through jgb_kernel_batch (host
    buffers, copies inside the timed call); the FP64 form, which is ~20x
    slower, on the first fp64_nobs profiles, with the mixed form timed on the
    same profiles for the ratio and the mixed-vs-FP64 Jacobian error."""
    import ctypes as C
    from jurassic_gb300 import model, native, synth
    w = synth.config_jacobian(nobs)
    ctl = w.ctl
    ctx = native.Context(ctl, w.tables, w.filters, device=local)
    L = native.load()
    m, n = ctx.kernel_sizes(w.batch)
    units = int(np.sum(m.astype(np.int64) * (n + 1)))
    small = synth.pack(ctl, [w.batch.item(ctl, i) for i in range(min(8, nobs))])
    for _ in range(warmup):
        ctx.kernel_batch(small, native.MIXED)
    barrier(pg)
    ms = []
    with ClockSampler(local) as clk:
        for _ in range(steps):
            t0 = time.perf_counter()
            Ks, _ = ctx.kernel_batch(w.batch, native.MIXED)
            ms.append(1e3 * (time.perf_counter() - t0))
    barrier(pg)
    ms_step = allmax(pg, statistics.mean(ms))
    value = units * world / (ms_step / 1e3)
    stats = ctx.stats()
    # FP64 against mixed on a subset of the profiles
    fp64 = None
    if fp64_nobs > 0:
        k = min(fp64_nobs, nobs)
        sub = synth.pack(ctl, [w.batch.item(ctl, i) for i in range(k)])
        sunits = int(np.sum(m[:k].astype(np.int64) * (n[:k] + 1)))
        ctx.kernel_batch(small, native.FP64)
        t0 = time.perf_counter()
        K64, fm64 = ctx.kernel_batch(sub, native.FP64)
        t64 = time.perf_counter() - t0
        t0 = time.perf_counter()
        K32, _ = ctx.kernel_batch(sub, native.MIXED)
        t32 = time.perf_counter() - t0
        # error of the finite-difference radiance changes K_ij h_j relative
        # to the radiance y_i (columns of upper levels are rounding noise
        # relative to their own size in any finite difference)
        fd = 0.0
        for i in range(k):
            atm, _ = sub.item(ctl, i)
            x, kind = model.atm2x(ctl, atm)
            h = model.fd_steps(ctl, x, kind)
            y = model.obs2y(fm64.rad[:, sub.ray_off[i]:sub.ray_off[i + 1]])
            fd = max(fd, float(np.max(np.abs(K32[i] - K64[i]) * h[None, :] / np.abs(y)[:, None])))
        fp64 = {"profiles": k, "value": sunits / t64, "unit": UNIT,
                "mixed_same_profiles": sunits / t32,
                "speedup_mixed_over_fp64": t64 / t32,
                "mixed_vs_fp64_max_fd_radiance_change_rel": fd}
    # normal equations on the device
    nu = np.asarray(ctl.nu)
    x = 1.43877506 * nu / 250.0
    dbdt = 1.19104259e-8 * nu ** 3 * x * np.exp(x) / (250.0 * np.expm1(x) ** 2)
    sig = 0.2 * dbdt
    rng = np.random.default_rng(5)
    Kc = np.ascontiguousarray(np.concatenate([k_.ravel() for k_ in Ks]))
    wv = np.concatenate([1.0 / sig[:mi] for mi in m])
    dy = rng.standard_normal(wv.size) / wv
    nA, nb = int(np.sum(n.astype(np.int64) ** 2)), int(np.sum(n))
    dev = {}
    for key, a in (("K", Kc), ("w", wv), ("dy", dy)):
        dev[key] = L.jgb_dev_alloc(a.nbytes)
        L.jgb_memcpy_h2d(dev[key], a.ctypes.data, a.nbytes)
    dev["A"] = L.jgb_dev_alloc(8 * nA)
    dev["b"] = L.jgb_dev_alloc(8 * nb)
    mi = np.ascontiguousarray(m, np.int32)
    ni = np.ascontiguousarray(n, np.int32)
    flops = float(np.sum(2.0 * m * (n + 1.0) ** 2))
    ne, A = {}, {}
    for name, prec in (("mixed_3xtf32", native.MIXED), ("fp64", native.FP64)):
        kms = C.c_float(0)
        ctx._check(L.jgb_normal_equations_dev(ctx.h, nobs, mi.ctypes.data_as(C.POINTER(C.c_int)),
                                              ni.ctypes.data_as(C.POINTER(C.c_int)), dev["K"],
                                              dev["w"], dev["dy"], dev["A"], dev["b"], prec,
                                              C.byref(kms)))
        a = np.zeros(nA)
        L.jgb_memcpy_d2h(a.ctypes.data, dev["A"], a.nbytes)
        A[name] = a
        ne[name] = {"kernel_ms": kms.value, "tflops": flops / (kms.value / 1e3) / 1e12}
    for ptr in dev.values():
        L.jgb_dev_free(ptr)
    rel = float(np.max(np.abs(A["mixed_3xtf32"] - A["fp64"])) / np.max(np.abs(A["fp64"])))
    try:
        bf16 = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"]
        kind = "measured"
    except (OSError, KeyError, ValueError):
        bf16, kind = 1900.0, "fallback"
    peak = bf16 / 2 / 3     # dense TF32 = half the bf16 rate; 3xTF32 = three products
    ctx.close()
    return {"value": value, "unit": UNIT, "ms_per_step": ms_step, "steps": steps,
            "workload": "fd_jacobian_nadir_%dobs_81lev_150ch_4gas_n405" % nobs,
            "observations": nobs, "state_elements": int(n[0]), "radiances_per_step": units,
            "resume_skip": stats.get("resume_skip"),
            "h2d_bytes_per_step": int(w.batch.nlev * 8 * (6 + ctl.ng + ctl.nw)),
            "d2h_bytes_per_step": int(8 * Kc.size), "fp64": fp64,
            "normal_equations": dict(ne, flops=flops, problems=nobs, m=int(m[0]),
                                     n=int(n[0]), mixed_vs_fp64_max_rel=rel,
                                     roofline={"bound": "tensor", "peak": peak,
                                               "unit": "TFLOP/s", "peak_kind": kind,
                                               "peak_note": "bf16 dense / 2 (TF32) / 3 (3xTF32)",
                                               "frac": ne["mixed_3xtf32"]["tflops"] / peak}),
            "clocks": clk.summary()}


def run_jacobian(args, rank, world, local, pg):
    nobs = args.nobs if args.nobs != 100000 else 2048
    r = jacobian_measure(local, nobs, args.steps, args.warmup, args.c4_fp64_nobs, pg, world)
    if rank == 0:
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 path loop, f64 perturbation bookkeeping", "data": "synthetic (seeded)",
                "config": {"workload": r["workload"], "observations": nobs,
                           "state_elements": r["state_elements"],
                           "radiances_per_step": r["radiances_per_step"],
                           "l2_policy": "inputs larger than L2 (129 MB); no flush"},
                "e2e": {"value": r["value"], "unit": UNIT,
                        "h2d_bytes_per_step": r["h2d_bytes_per_step"],
                        "d2h_bytes_per_step": r["d2h_bytes_per_step"]},
                "fp64": r["fp64"], "normal_equations": r["normal_equations"],
                "clocks": r["clocks"]}
        print(json.dumps(line), flush=True)


def invert_measure(ctx, L, nmat, n, steps, warmup):
    """FP64 inverse of nmat symmetric positive-definite n x n matrices
    (matrix_invert, retrieval.c:373-399: Cholesky factor and inverse) through
    jgb_matrix_invert_dev: a-priori covariances with exponential
    correlation (seeded heights, sigmas and correlation lengths) like the
    retrieval's S_a.  Algorithmic flops n^3 per matrix (factor n^3/3,
    inverse from the factor 2 n^3/3); the FP64 peak is GB300's nominal
    1.25 TFLOP/s (no FP64 figure is measured for the pool)."""
    import ctypes as C
    rng = np.random.default_rng(12)
    z = np.sort(rng.uniform(0, 60, (nmat, n)), axis=1)
    sig = rng.uniform(1, 3, (nmat, n))
    cz = rng.uniform(1, 5, (nmat, 1, 1))
    mats = np.ascontiguousarray(sig[:, :, None] * sig[:, None, :] *
                                np.exp(-np.abs(z[:, :, None] - z[:, None, :]) / cz))
    dA = L.jgb_dev_alloc(mats.nbytes)
    ni = np.full(nmat, n, np.int32)
    st = np.zeros(nmat, np.int32)
    times = []
    for _ in range(warmup + steps):
        L.jgb_memcpy_h2d(dA, mats.ctypes.data, mats.nbytes)
        kms = C.c_float(0)
        ctx._check(L.jgb_matrix_invert_dev(ctx.h, nmat, ni.ctypes.data_as(C.POINTER(C.c_int)), dA,
                                           st.ctypes.data_as(C.POINTER(C.c_int)), C.byref(kms)))
        times.append(kms.value)
    out = np.zeros_like(mats)
    L.jgb_memcpy_d2h(out.ctypes.data, dA, out.nbytes)
    L.jgb_dev_free(dA)
    t = statistics.mean(times[warmup:])
    flops = float(n) ** 3 * nmat
    dev = max(float(np.max(np.abs(out[k] - np.linalg.inv(mats[k]))) /
                    np.max(np.abs(np.linalg.inv(mats[k])))) for k in range(4))
    peak = 1250.0
    return {"matrices": nmat, "n": n, "kernel_ms": t, "gflops": flops / (t / 1e3) / 1e9,
            "flops_per_matrix": float(n) ** 3, "not_positive_definite": int(np.sum(st)),
            "max_rel_vs_numpy_first4": dev,
            "roofline": {"bound": "fp64", "achieved": flops / (t / 1e3) / 1e9, "peak": peak,
                         "unit": "GFLOP/s", "frac": flops / (t / 1e3) / 1e9 / peak,
                         "peak_kind": "nominal"}}


def run_normal(args, rank, world, local, pg):
    """Normal-equation products alone (matrix_product, retrieval.c:403-444):
    nobs problems with m = 150 measurements and n = 405 state elements
    (the shapes of the Jacobian workload), seeded K with the magnitudes of
    radiance Jacobians; 3xTF32 (tcgen05 tensor cores, TMEM accumulators)
    and FP64."""
    import ctypes as C
    from jurassic_gb300 import native, synth
    from jurassic_gb300.model import Ctl
    nobs = args.nobs if args.nobs != 100000 else 2048
    m_, n_ = 150, 405
    ctl = Ctl(emitter=["CO2"], nu=[700.0])
    ctx = native.Context(ctl, device=local)
    L = native.load()
    rng = np.random.default_rng(6)
    K = (rng.standard_normal((nobs, m_, n_)) * np.exp(rng.uniform(-6, 0, (nobs, 1, n_))) * 1e-4)
    w = 1.0 / (2e-6 * (1 + rng.uniform(0, 1, (nobs, m_))))
    dy = rng.standard_normal((nobs, m_)) / w
    dev = {}
    for k, a in (("K", K), ("w", w), ("dy", dy)):
        a = np.ascontiguousarray(a)
        dev[k] = L.jgb_dev_alloc(a.nbytes)
        L.jgb_memcpy_h2d(dev[k], a.ctypes.data, a.nbytes)
    dev["A"] = L.jgb_dev_alloc(8 * nobs * n_ * n_)
    dev["b"] = L.jgb_dev_alloc(8 * nobs * n_)
    mi = np.full(nobs, m_, np.int32)
    ni = np.full(nobs, n_, np.int32)
    flops = 2.0 * m_ * (n_ + 1) ** 2 * nobs
    res, A = {}, {}
    for name, prec in (("mixed_3xtf32", native.MIXED), ("fp64", native.FP64)):
        times = []
        for _ in range(args.warmup + args.steps):
            kms = C.c_float(0)
            ctx._check(L.jgb_normal_equations_dev(ctx.h, nobs, mi.ctypes.data_as(C.POINTER(C.c_int)),
                                                  ni.ctypes.data_as(C.POINTER(C.c_int)), dev["K"],
                                                  dev["w"], dev["dy"], dev["A"], dev["b"], prec,
                                                  C.byref(kms)))
            times.append(kms.value)
        t = statistics.mean(times[args.warmup:])
        a = np.zeros(nobs * n_ * n_)
        L.jgb_memcpy_d2h(a.ctypes.data, dev["A"], a.nbytes)
        A[name] = a
        res[name] = {"kernel_ms": t, "tflops": flops / (t / 1e3) / 1e12}
    for p in dev.values():
        L.jgb_dev_free(p)
    try:
        bf16 = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["bf16_tflops"]
        kind = "measured"
    except (OSError, KeyError, ValueError):
        bf16, kind = 1900.0, "fallback"
    peak = bf16 / 2 / 3
    rel = float(np.max(np.abs(A["mixed_3xtf32"] - A["fp64"])) / np.max(np.abs(A["fp64"])))
    inv = invert_measure(ctx, L, min(nobs, 512), n_, args.steps, args.warmup)
    if rank == 0:
        v = res["mixed_3xtf32"]["tflops"]
        print(json.dumps({
            "metric": "normal-equation TFLOP/s", "value": v, "unit": "TFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["mixed_3xtf32"]["kernel_ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "3xTF32 (fp32 accumulate)",
            "data": "synthetic (seeded)",
            "config": {"workload": "normal_equations_%dx(150x405)" % nobs,
                       "l2_policy": "K (%.0f MB) larger than L2; no flush" % (K.nbytes / 1e6)},
            "fp64": res["fp64"], "mixed_vs_fp64_max_rel": rel, "flops_per_step": flops,
            "matrix_invert": inv,
            "roofline": {"bound": "tensor", "achieved": v, "peak": peak, "unit": "TFLOP/s",
                         "frac": v / peak, "traffic": None, "peak_kind": kind,
                         "peak_note": "bf16 dense / 2 (TF32) / 3 (3xTF32)"}}), flush=True)
    ctx.close()


def run_serving(args, device):
    """Closed-loop capacity and Poisson-arrival latency of the retrieval
    engine, mixed precision and FP64, on the serving stream."""
    from jurassic_gb300 import native, serving
    ctl, ret, tables, filters = serving.stream_workload()
    ctx = native.Context(ctl, tables, filters, device=device)
    n, m = args.serve_requests, args.serve_fp64_requests
    reqs = serving.stream_requests(ctl, lambda b: ctx.formod_batch(b.fresh_outputs(), native.FP64), n)
    out = {"workload": "retrieval stream: %d requests, 50-300 of 300 channels, 41-101 levels, "
                       "nadir/limb(5 rays) alternating, CO2+H2O+O3, T+H2O retrieved" % n}

    def engine(prec):
        return ctx.engine(ret, prec, mem_budget=int(args.serve_budget_gb * 2**30))

    def strip(r):
        return {k: v for k, v in r.items() if k != "results"}

    # warm-up (autotune, allocations) on two requests
    serving.serve(engine(native.MIXED), ctl, reqs[:2], np.inf)
    serving.serve(engine(native.FP64), ctl, reqs[:2], np.inf)
    closed = serving.serve(engine(native.MIXED), ctl, reqs, np.inf)
    rate = args.serve_load * closed["retrievals_per_s"]
    pois = serving.serve(engine(native.MIXED), ctl, reqs, rate, seed=7)
    # latency against offered load (the same requests, the same arrival seed)
    sweep = []
    for load in sorted({float(v) for v in args.serve_sweep.split(",") if v.strip()} | {args.serve_load}):
        r = pois if load == args.serve_load else serving.serve(
            engine(native.MIXED), ctl, reqs, load * closed["retrievals_per_s"], seed=7)
        sweep.append({"load": load, "rate_hz": r["rate_hz"], "retrievals_per_s": r["retrievals_per_s"],
                      "p50_ms": r["p50_ms"], "p99_ms": r["p99_ms"], "mean_ms": r["mean_ms"],
                      "steps": r["steps"]})
    m = min(m, n)
    sub_mixed = closed if m == n else serving.serve(engine(native.MIXED), ctl, reqs[:m], np.inf)
    sub_fp64 = serving.serve(engine(native.FP64), ctl, reqs[:m], np.inf)
    dev = []
    for a, b in zip(sub_fp64["results"], sub_mixed["results"]):
        if a["err_total"] is not None:
            dev.append(float(np.max(np.abs(a["x"] - b["x"]) / a["err_total"])))
    out.update({
        "mixed_closed_loop": strip(closed),
        "mixed_poisson": dict(strip(pois), load=args.serve_load),
        "mixed_poisson_sweep": sweep,
        "fp64_closed_loop": dict(strip(sub_fp64), requests=m),
        "mixed_closed_loop_same_requests": dict(strip(sub_mixed), requests=m),
        "retrievals_per_s_mixed_over_fp64": sub_mixed["retrievals_per_s"] / sub_fp64["retrievals_per_s"],
        "mixed_vs_fp64_max_dx_over_sigma": max(dev) if dev else None,
        "mem_budget_gb": args.serve_budget_gb})
    ctx.close()
    return out


class DeviceBatch:
    """A synthetic batch copied once into device memory (the inputs of the
    device-resident "value" path) and, on request, into page-locked host
    buffers (the e2e path)."""

    def __init__(self, L, ctl, b):
        self.L, self.b = L, b
        self.fields = {k: np.ascontiguousarray(getattr(b, k), dtype=np.float64)
                       for k in ("time", "z", "lon", "lat", "p", "t", "q", "k", "scal", "geo")}
        self.fields["rad"] = np.zeros((ctl.nd, b.nray))
        self.fields["tau"] = np.zeros((ctl.nd, b.nray))
        self.fields["tp"] = np.zeros((3, b.nray))
        self.ints = {"lev_off": np.ascontiguousarray(b.lev_off, np.int32),
                     "ray_off": np.ascontiguousarray(b.ray_off, np.int32)}
        self.dptr, self.hb = {}, {}
        for k, a in self.items():
            p = L.jgb_dev_alloc(max(a.nbytes, 8))
            assert p, "device allocation failed"
            L.jgb_memcpy_h2d(p, a.ctypes.data, a.nbytes)
            self.dptr[k] = p

    def items(self):
        return list(self.fields.items()) + list(self.ints.items())

    def step(self, ctx, prec):
        """One forward model of the device-resident batch (fresh mask)."""
        f = self.fields["rad"]
        self.L.jgb_memcpy_h2d(self.dptr["rad"], f.ctypes.data, f.nbytes)
        ctx.formod_batch_ptrs(self.dptr, self.b.nobs, prec, device=True)
        return ctx.stats()

    def rad(self):
        out = np.zeros_like(self.fields["rad"])
        self.L.jgb_memcpy_d2h(out.ctypes.data, self.dptr["rad"], out.nbytes)
        return out

    def host(self):
        import ctypes as C
        for k, a in self.items():
            p = self.L.jgb_host_alloc(max(a.nbytes, 8))
            C.memmove(p, a.ctypes.data, a.nbytes)
            self.hb[k] = p
        h2d = sum(self.fields[k].nbytes for k in ("time", "z", "lon", "lat", "p", "t", "q", "k",
                                                    "scal", "geo", "rad")) + 2 * self.ints["lev_off"].nbytes
        d2h = sum(self.fields[k].nbytes for k in ("rad", "tau", "tp"))
        return self.hb, h2d, d2h

    def free(self):
        for p in self.dptr.values():
            self.L.jgb_dev_free(p)
        for p in self.hb.values():
            self.L.jgb_host_free(p)


def accuracy_block(ctl, rad_mixed, rad_fp64, b, idx, ref):
    """Mixed |dBT| and FP64 relative radiance error against the oracle on
    the sampled observations (ref = oracle output of the sample batch)."""
    from jurassic_gb300.model import brightness
    rays = sample_rays(b, idx)
    nu = np.asarray(ctl.nu)[:, None]
    fin = np.isfinite(ref.rad)
    bt_ref = brightness(ref.rad, nu)
    dbt = np.abs(brightness(rad_mixed[:, rays], nu) - bt_ref)[fin]
    rel32 = (np.abs(rad_mixed[:, rays] - ref.rad) / np.abs(ref.rad))[fin]
    out = {"sample": sample_record(idx, b.nobs), "sample_rays": int(len(rays)),
           "mixed_max_abs_dBT_mK": 1e3 * float(np.max(dbt)),
           "mixed_p99_abs_dBT_mK": 1e3 * float(np.percentile(dbt, 99)),
           "mixed_max_rel_rad": float(np.max(rel32)), "gate_mK": 10.0,
           "mixed_within_gate": bool(np.max(dbt) <= 0.010)}
    if rad_fp64 is not None:
        out["fp64_max_rel_rad"] = float(np.max((np.abs(rad_fp64[:, rays] - ref.rad) /
                                                np.abs(ref.rad))[fin]))
    return out


def limb_cga_measure(local, nobs, steps, warmup, fp64_steps, cpu_seconds):
    """The uneven limb CGA batch: nobs single-ray observations with tangent
    heights uniform on 5-60 km (50-400 LOS points per ray at RAYDZ 0.5 km),
    32 channels, 3 emitters.  Mixed and FP64 device-resident radiances/s,
    the LOS point spread, the compulsory-byte HBM fraction of the path
    kernel and the accuracy of both forms against the oracle on a stratified
    sample."""
    from jurassic_gb300 import native, synth
    from oracle import oracle
    w = synth.config_limb_cga(nobs)
    ctl, b = w.ctl, w.batch
    ctx = native.Context(ctl, w.tables, w.filters, device=local)
    L = native.load()
    db = DeviceBatch(L, ctl, b)
    units = b.nray * ctl.nd
    for _ in range(warmup):
        db.step(ctx, native.MIXED)
    ms, path = [], []
    for _ in range(steps):
        st = db.step(ctx, native.MIXED)
        ms.append(st["total_ms"])
        path.append(st["path_ms"])
    rad32 = db.rad()
    los = st["los_points"]
    rad64, ms64 = None, []
    if fp64_steps > 0:
        db.step(ctx, native.FP64)
        for _ in range(fp64_steps):
            ms64.append(db.step(ctx, native.FP64)["total_ms"])
        rad64 = db.rad()
    hbm, kind = peaks()
    comp = compulsory_bytes(ctl, w.tables, los, b.nray)
    t_path = statistics.mean(path) / 1e3
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    idx, sb, ref, dt = time_cpu(w, ora, cpu_seconds, os.cpu_count() or 1, n0=64)
    # LOS points per ray of the sample, from the oracle's ray tracing
    pts = [len(ora.raytrace(*sb.item(ctl, i), 0)[0]) for i in range(sb.nobs)]
    ora.close()
    out = {"workload": w.name, "observations": nobs, "rays": b.nray, "channels": ctl.nd,
           "emitters": ctl.ng, "method": "CGA", "raydz_km": ctl.raydz, "los_points": los,
           "value": units / (statistics.mean(ms) / 1e3), "unit": UNIT,
           "ms_per_step": statistics.mean(ms), "steps": steps,
           "stage_ms": {k: st[k] for k in ("trace_ms", "pack_ms", "path_ms")},
           "fp64": None if not ms64 else {
               "value": units / (statistics.mean(ms64) / 1e3), "unit": UNIT,
               "ms_per_step": statistics.mean(ms64),
               "speedup_mixed_over_fp64": statistics.mean(ms64) / statistics.mean(ms)},
           "hbm_compulsory": {"achieved": comp / t_path / 1e9, "peak": hbm, "unit": "GB/s",
                              "frac": comp / t_path / 1e9 / hbm, "peak_kind": kind,
                              "bytes_per_launch": comp},
           "cpu_baseline": {"value": sb.nray * ctl.nd / dt, "unit": UNIT,
                            "cores": os.cpu_count() or 1, "kind": "port"},
           "accuracy": accuracy_block(ctl, rad32, rad64, b, idx, ref),
           "los_points_per_ray_sample": {"min": int(min(pts)), "max": int(max(pts)),
                                         "mean": float(np.mean(pts))}}
    db.free()
    ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="nadir",
                    choices=["nadir", "limb_cga", "jacobian", "normal"])
    ap.add_argument("--nobs", type=int, default=100000)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the limb CGA and FD Jacobian configurations of the default run")
    ap.add_argument("--c3-nobs", type=int, default=20000,
                    help="observations of the limb CGA configuration")
    ap.add_argument("--c4-nobs", type=int, default=2048,
                    help="profiles of the FD Jacobian configuration")
    ap.add_argument("--c4-fp64-nobs", type=int, default=128,
                    help="profiles of the FD Jacobian timed in FP64 (and mixed) for the ratio")
    ap.add_argument("--serve-requests", type=int, default=512)
    ap.add_argument("--serve-fp64-requests", type=int, default=48,
                    help="first requests of the stream also run through the FP64 engine for "
                         "the mixed/FP64 retrievals/s ratio and the accuracy")
    ap.add_argument("--serve-load", type=float, default=0.7,
                    help="Poisson arrival rate as a fraction of the closed-loop capacity")
    ap.add_argument("--serve-sweep", default="0.3,0.5",
                    help="further Poisson loads (fractions of the closed-loop capacity) for the "
                         "latency-load curve; empty: none")
    ap.add_argument("--serve-budget-gb", type=float, default=64.0)
    args = ap.parse_args()

    rank, world, local, pg = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank)
        return

    from jurassic_gb300 import native
    native.load()
    if args.workload in ("jacobian", "normal"):
        (run_jacobian if args.workload == "jacobian" else run_normal)(args, rank, world, local, pg)
        if pg is not None:
            pg.destroy_process_group()
        return
    w = build_workload(args)
    ctl, b = w.ctl, w.batch
    ctx = native.Context(ctl, w.tables, w.filters, device=local)
    L = native.load()
    units = b.nray * ctl.nd
    db = DeviceBatch(L, ctl, b)

    # ---- mixed precision, device-resident (value) ----
    for _ in range(args.warmup):
        db.step(ctx, native.MIXED)
    barrier(pg)
    ms, path_ms, stats = [], [], None
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            stats = db.step(ctx, native.MIXED)
            ms.append(stats["total_ms"])
            path_ms.append(stats["path_ms"])
        wall = time.perf_counter() - t0
    barrier(pg)
    ms_step = allmax(pg, statistics.mean(ms))
    value = units * world / (ms_step / 1e3)
    rad_mixed = db.rad()

    # ---- e2e through the public C ABI with page-locked host buffers ----
    hb, h2d, d2h = db.host()
    for _ in range(max(1, args.warmup - 1)):
        ctx.formod_batch_ptrs(hb, b.nobs, native.MIXED, device=False)
    e2e_ms, e2e_st = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ctx.formod_batch_ptrs(hb, b.nobs, native.MIXED, device=False)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
        e2e_st.append(ctx.stats())
    e2e_value = units * world / (allmax(pg, statistics.mean(e2e_ms)) / 1e3)

    # ---- plain FP64 GPU form ----
    fp64_ms, fp64_value, rad_fp64 = [], None, None
    if args.fp64_steps > 0:
        db.step(ctx, native.FP64)
        for _ in range(args.fp64_steps):
            fp64_ms.append(db.step(ctx, native.FP64)["total_ms"])
        fp64_value = units * world / (allmax(pg, statistics.mean(fp64_ms)) / 1e3)
        rad_fp64 = db.rad()

    line = None
    if rank == 0:
        hbm, peak_kind = peaks()
        clocks = clk.summary()
        roof = issue_roofline(stats["los_points"], statistics.mean(path_ms), clocks["sm_mhz"],
                              sm_count(local), ctl, w.tables, b.nray, hbm, peak_kind)
        if args.workload != "nadir":   # the instruction counts are the nadir launch's
            roof.update(achieved=None, frac=None, traffic=None, warp_instructions_per_launch=None)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 path loop (compensated), f64 ray tracing",
                "data": "synthetic (seeded)",
                "config": {"workload": w.name, "observations": b.nobs, "rays": b.nray,
                           "channels": ctl.nd, "emitters": ctl.ng,
                           "levels_per_profile": int(b.lev_off[1] - b.lev_off[0]),
                           "method": "EGA" if ctl.formod == 1 else "CGA",
                           "los_points": stats["los_points"],
                           "l2_policy": "inputs and tables larger than L2 (129 MB); no flush",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "stage_ms": {k: stats[k] for k in ("hydro_ms", "trace_ms", "pack_ms", "path_ms")},
                "trace_passes": stats["trace_passes"],
                "autotune": {"path_variant": stats["path_variant"], "variant_ms": stats["tune_ms"][:16],
                             "caps": ["no register cap", "5 blocks/SM (<=102 regs)",
                                      "6 blocks/SM (<=85 regs)", "4 blocks/SM (<=128 regs)",
                                      "8 blocks/SM (<=64 regs)", "10 blocks/SM (<=51 regs)",
                                      "12 blocks/SM (<=42 regs)"],
                             "note": "variant v < 14: register cap v % 7; block = 4 channels x 1 "
                                     "tile (v < 7) or 1 channel x 4 tiles (7 <= v < 14); v = 14, "
                                     "15: block = 1 channel x 8 tiles (256 threads), <= 64 or "
                                     "<= 51 registers"},
                "wall_s_timed": wall,
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h), "ms_per_step": statistics.mean(e2e_ms),
                        "stage_ms": {k: statistics.mean(st[k] for st in e2e_st)
                                     for k in ("h2d_ms", "d2h_ms", "path_ms", "total_ms")}},
                "fp64": None if fp64_value is None else {
                    "value": fp64_value, "unit": UNIT, "ms_per_step": statistics.mean(fp64_ms),
                    "speedup_mixed_over_fp64": value / fp64_value},
                "gpu_launches": int(stats["path_launches"]) * args.steps,
                "roofline": roof,
                "clocks": clocks}

    # ---- CPU baseline + accuracy on a bounded, stratified sample ----
    if rank == 0 and not args.no_cpu:
        from oracle import oracle
        ora = oracle.Oracle(ctl, w.tables, w.filters)
        threads = os.cpu_count() or 1
        idx, s, ref, dt = time_cpu(w, ora, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": s.nray * ctl.nd / dt, "unit": UNIT, "cores": threads,
                                "kind": "port",
                                "sample": "%d of %d observations, stratified over the batch, x %d "
                                          "channels" % (s.nobs, b.nobs, ctl.nd)}
        line["accuracy"] = accuracy_block(ctl, rad_mixed, rad_fp64, b, idx, ref)
        ora.close()
    db.free()
    ctx.close()
    if rank == 0 and not args.no_extra and args.workload == "nadir":
        line["limb_cga"] = limb_cga_measure(local, args.c3_nobs, max(3, min(args.steps, 10)),
                                            3, 1 if args.fp64_steps > 0 else 0,
                                            0.0 if args.no_cpu else 3.0)
        line["jacobian"] = jacobian_measure(local, args.c4_nobs, 2, 1, args.c4_fp64_nobs)
    if rank == 0 and args.serve_requests > 0:
        line["serving"] = run_serving(args, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
