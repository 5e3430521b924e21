"""Host-memory batches (jgb_formod_batch) on the GPU.

A host batch of more than 64 MB of inputs runs as two chunks of whole
observations whose copies overlap the other chunk's compute.  Its results
(radiances, transmittances, tangent points and, with HYDZ, the hydrostatic
pressures written back) equal those of the same batch resident on the device
(jgb_formod_batch_dev, one launch over all observations) bit for bit, in both
precisions.
"""
import copy

import numpy as np
import pytest

from jurassic_gb300 import native, synth

pytestmark = pytest.mark.gpu

FIELDS = ("time", "z", "lon", "lat", "p", "t", "q", "k", "scal", "geo", "rad", "tau", "tp")


def _device_run(ctx, batch, precision):
    L = native.load()
    arrs = {k: np.ascontiguousarray(getattr(batch, k), dtype=np.float64) for k in FIELDS}
    arrs["lev_off"] = np.ascontiguousarray(batch.lev_off, np.int32)
    arrs["ray_off"] = np.ascontiguousarray(batch.ray_off, np.int32)
    dptr = {}
    try:
        for k, a in arrs.items():
            p = L.jgb_dev_alloc(max(a.nbytes, 8))
            assert p
            dptr[k] = p
            assert L.jgb_memcpy_h2d(p, a.ctypes.data, a.nbytes) == 0
        ctx.formod_batch_ptrs(dptr, batch.nobs, precision, device=True)
        out = {}
        for k in ("rad", "tau", "tp", "p"):
            o = np.empty_like(arrs[k])
            assert L.jgb_memcpy_d2h(o.ctypes.data, dptr[k], o.nbytes) == 0
            out[k] = o
        return out
    finally:
        for p in dptr.values():
            L.jgb_dev_free(p)


@pytest.mark.parametrize("hydz", [-999.0, 0.0])
def test_chunked_host_batch_equals_device_batch(built_lib, hydz):
    w = synth.config_nadir(20000, nd=6, nlev=101, ztop=60.0, emitters=("CO2", "H2O"))
    ctl = copy.deepcopy(w.ctl)
    ctl.hydz = hydz
    ctx = native.Context(ctl, w.tables, w.filters)
    for prec in (native.MIXED, native.FP64):
        host = ctx.formod_batch(w.batch.fresh_outputs(), prec)
        st = ctx.stats()
        assert st["los_points"] > 0
        dev = _device_run(ctx, w.batch.fresh_outputs(), prec)
        assert ctx.stats()["los_points"] == st["los_points"]
        for k in ("rad", "tau", "tp", "p"):
            assert np.array_equal(getattr(host, k), dev[k], equal_nan=True), (prec, k)
        if hydz >= 0:
            assert not np.array_equal(dev["p"], w.batch.p)
