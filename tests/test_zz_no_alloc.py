"""The allocation-free entry point (jgb_formod_batch_dev_noalloc) against the
regular device-batch entry point (jgb_formod_batch_dev, FP64).

The allocation-free variant exists for callers that cannot allocate GPU
memory while they run (a fixed memory budget, an allocator owned by another
runtime); its scratch is a fixed 64 MiB device array shared by all calls,
loaded onto the device by jgb_create.  Two calls in a row must each
reproduce the regular entry point (the second call finds the first call's
leftovers in the array), the device's free memory must not change across
the calls -- also on a fresh context in a fresh process, where the calls are
the first forward models of the process -- and a batch that does not fit
must be rejected with JGB_ERR_ARG instead of running.  The cases cover the
hydrostatic pre-step and the surface-reflection scratch.

This file is named so that pytest collects it last.
"""
import ctypes as C
import copy
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from jurassic_gb300 import native, synth

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9  # same tolerance as the FP64 parity tests
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def device_free_bytes():
    """cudaMemGetInfo of the current device, through the CUDA runtime the
    library itself is linked with."""
    rt = C.CDLL("libcudart.so.13")
    free, total = C.c_size_t(0), C.c_size_t(0)
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    return free.value


def workload(case):
    """Small workloads of the four cases: nadir, limb, nadir with the
    hydrostatic pre-step (pressures rewritten on the device) and nadir with
    a reflecting surface and the solar term (reflection scratch)."""
    if case == "limb":
        return synth.config_limb_ega(n_rays=6)
    w = synth.config_nadir(12, nd=6, nlev=51, ztop=50.0)
    if case == "hydrostatic":
        w.ctl = copy.deepcopy(w.ctl)
        w.ctl.hydz = 10.0
    elif case == "reflection":
        ctl = copy.deepcopy(w.ctl)
        ctl.sfnu = np.array([600.0, 1500.0, 2500.0])
        ctl.sftype = 3
        ctl.sfsza = -999.0
        b = w.batch
        # scal per observation: clz cldz sfz sfp sft sfeps[3]
        b.scal = np.zeros((b.nobs, 5 + ctl.ncl + ctl.nsf))
        b.scal[:, 4] = 290.0 + np.arange(b.nobs)
        b.scal[:, 5:] = [0.98, 0.9, 0.95]
        w.ctl = ctl
    return w


class DeviceBatch:
    """A synth.Batch copied to device memory with the library's allocator."""

    FIELDS = ("time", "z", "lon", "lat", "p", "t", "q", "k", "scal", "geo", "rad", "tau", "tp")

    def __init__(self, L, b):
        self.L = L
        self.b = b
        self.ptr = {}
        for k in self.FIELDS:
            self._put(k, np.ascontiguousarray(getattr(b, k), dtype=np.float64))
        for k in ("lev_off", "ray_off"):
            self._put(k, np.ascontiguousarray(getattr(b, k), dtype=np.int32))

    def _put(self, k, a):
        p = self.L.jgb_dev_alloc(max(a.nbytes, 8))
        assert p
        assert self.L.jgb_memcpy_h2d(p, a.ctypes.data, a.nbytes) == 0
        self.ptr[k] = p

    def reset_outputs(self):
        # the pressures too: the hydrostatic pre-step rewrites them in place
        p = np.ascontiguousarray(self.b.p, dtype=np.float64)
        assert self.L.jgb_memcpy_h2d(self.ptr["p"], p.ctypes.data, p.nbytes) == 0
        for k in ("rad", "tau", "tp"):
            a = np.ascontiguousarray(getattr(self.b, k), dtype=np.float64)
            if k != "rad":
                a = np.full_like(a, -1.0)  # garbage that must be overwritten
            assert self.L.jgb_memcpy_h2d(self.ptr[k], a.ctypes.data, a.nbytes) == 0

    def struct(self):
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        return native._Batch(nobs=self.b.nobs, **{
            k: C.cast(C.c_void_p(v), ip if k in ("lev_off", "ray_off") else dp)
            for k, v in self.ptr.items()})

    def outputs(self):
        out = {}
        for k, shape in (("rad", self.b.rad.shape), ("tau", self.b.tau.shape),
                         ("tp", self.b.tp.shape), ("p", self.b.p.shape)):
            a = np.zeros(shape)
            assert self.L.jgb_memcpy_d2h(a.ctypes.data, self.ptr[k], a.nbytes) == 0
            out[k] = a
        return out

    def free(self):
        for p in self.ptr.values():
            self.L.jgb_dev_free(p)


def _compare(a, b):
    for k in ("rad", "tau"):
        fa, fb = np.isfinite(a[k]), np.isfinite(b[k])
        assert np.array_equal(fa, fb)
        rel = np.max(np.abs(a[k][fa] - b[k][fa]) / np.maximum(np.abs(b[k][fa]), 1e-300))
        assert rel <= FP64_RTOL, (k, rel)
    assert np.max(np.abs(a["tp"] - b["tp"])) <= 1e-9
    assert np.max(np.abs(a["p"] - b["p"]) / b["p"]) <= FP64_RTOL


@pytest.mark.parametrize("case", ["nadir", "limb", "hydrostatic", "reflection"])
def test_noalloc_matches_regular_entry_point_twice(built_lib, case):
    L = native.load()
    w = workload(case)
    ctx = native.Context(w.ctl, w.tables, w.filters)
    db = DeviceBatch(L, w.batch.fresh_outputs())
    try:
        db.reset_outputs()
        s = db.struct()
        assert L.jgb_formod_batch_dev(ctx.h, C.byref(s), native.FP64) == 0
        expected = db.outputs()
        if case == "hydrostatic":
            assert np.max(np.abs(expected["p"] - w.batch.p) / w.batch.p) > 1e-6
        if case == "reflection":
            assert np.all(np.isfinite(expected["rad"]))
        free = []
        for _ in range(2):
            db.reset_outputs()
            free.append(device_free_bytes())
            rc = L.jgb_formod_batch_dev_noalloc(ctx.h, C.byref(s))
            assert rc == 0, L.jgb_last_error(ctx.h).decode()
            free.append(device_free_bytes())
            _compare(db.outputs(), expected)
            st = ctx.stats()
            assert st["los_points"] > 0 and st["total_ms"] > 0
        assert len(set(free)) == 1, "device memory changed across the calls: %s" % free
    finally:
        db.free()
        ctx.close()


FRESH = textwrap.dedent("""
    import ctypes as C, sys
    sys.path.insert(0, {root!r}); sys.path.insert(0, {tests!r})
    import numpy as np
    from jurassic_gb300 import native
    from test_zz_no_alloc import DeviceBatch, device_free_bytes, workload
    L = native.load()
    w = workload("reflection")
    ctx = native.Context(w.ctl, w.tables, w.filters)
    db = DeviceBatch(L, w.batch.fresh_outputs())
    db.reset_outputs()
    s = db.struct()
    free = [device_free_bytes()]
    for _ in range(2):
        assert L.jgb_formod_batch_dev_noalloc(ctx.h, C.byref(s)) == 0
        free.append(device_free_bytes())
    first = db.outputs()
    db.reset_outputs()
    assert L.jgb_formod_batch_dev(ctx.h, C.byref(s), native.FP64) == 0
    regular = db.outputs()
    rel = np.max(np.abs(first["rad"] - regular["rad"]) / np.abs(regular["rad"]))
    print("FREE", *free, "REL", rel)
""")


def test_noalloc_fresh_process_allocates_nothing(built_lib):
    """In a fresh process the allocation-free calls are the first forward
    models of the context: jgb_create has loaded the scratch array and the
    kernels, so the calls leave the device's free memory unchanged."""
    code = FRESH.format(root=ROOT, tests=os.path.join(ROOT, "tests"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    line = [ln for ln in r.stdout.splitlines() if ln.startswith("FREE")][-1].split()
    free = [int(v) for v in line[1:4]]
    assert len(set(free)) == 1, "device memory changed across the first calls: %s" % free
    assert float(line[5]) <= FP64_RTOL


def test_noalloc_rejects_batch_beyond_scratch(built_lib):
    L = native.load()
    # 6000 nadir rays of ~500 LOS points need far more than 64 MiB of LOS
    w = synth.config_nadir(6000, nd=2, nlev=51, ztop=50.0)
    ctx = native.Context(w.ctl, w.tables, w.filters)
    db = DeviceBatch(L, w.batch.fresh_outputs())
    try:
        rc = L.jgb_formod_batch_dev_noalloc(ctx.h, C.byref(db.struct()))
        assert rc == 1  # JGB_ERR_ARG
        assert "bytes of scratch" in L.jgb_last_error(ctx.h).decode()
    finally:
        db.free()
        ctx.close()
