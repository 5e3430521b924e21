"""The allocation-free entry point (jgb_formod_batch_dev_noalloc) against the
regular device-batch entry point (jgb_formod_batch_dev, FP64).

The allocation-free variant exists for callers that cannot allocate GPU
memory while they run; its scratch is a fixed 64 MiB device array shared by
all calls.  Two calls in a row must each reproduce the regular entry point
(the second call finds the first call's leftovers in the array), and a batch
that does not fit must be rejected with JGB_ERR_ARG instead of running.

This file is named so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from jurassic_gb300 import native, synth

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9  # same tolerance as the FP64 parity tests


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
                         ("tp", self.b.tp.shape)):
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


@pytest.mark.parametrize("case", ["nadir", "limb"])
def test_noalloc_matches_regular_entry_point_twice(built_lib, case):
    L = native.load()
    if case == "nadir":
        w = synth.config_nadir(12, nd=6, nlev=51, ztop=50.0)
    else:
        w = synth.config_limb_ega(n_rays=6)
    ctx = native.Context(w.ctl, w.tables, w.filters)
    db = DeviceBatch(L, w.batch.fresh_outputs())
    try:
        db.reset_outputs()
        s = db.struct()
        assert L.jgb_formod_batch_dev(ctx.h, C.byref(s), native.FP64) == 0
        expected = db.outputs()
        for _ in range(2):
            db.reset_outputs()
            rc = L.jgb_formod_batch_dev_noalloc(ctx.h, C.byref(s))
            assert rc == 0, L.jgb_last_error(ctx.h).decode()
            _compare(db.outputs(), expected)
    finally:
        db.free()
        ctx.close()


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
