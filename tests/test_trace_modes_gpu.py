"""Ray-tracing modes of the mixed-precision forward model on the GPU.

A batch of more than 2^23 / NLOS rays is traced in one pass into per-ray
capacities from a geometric bound of the LOS points (raytrace's step rule,
jurassic.c:4278-4287); smaller batches into fixed NLOS slabs; a ray that
outgrows its bound makes the batch count its rays first.  The LOS of a ray
does not depend on the mode, so every mode gives bit-identical results:
checked against the same rays run as smaller batches (fixed slabs), with the
bound scaled down until rays overflow it (count after the failed pass) and
turned off (count first).
"""
import numpy as np
import pytest

from jurassic_gb300 import native, synth

pytestmark = pytest.mark.gpu

NRAY = 2304          # > 2^23 / 4096 rays: capacity-bound mode


def _split(ctl, batch, parts):
    n = batch.nobs
    cuts = np.linspace(0, n, parts + 1).astype(int)
    return [synth.pack(ctl, [batch.item(ctl, i) for i in range(a, b)])
            for a, b in zip(cuts[:-1], cuts[1:])]


def _same_as_parts(ctx, ctl, batch, out):
    r0 = 0
    for part in _split(ctl, batch, 2):
        o = ctx.formod_batch(part.fresh_outputs(), native.MIXED)
        assert ctx.stats()["trace_passes"] == 1          # fixed slabs
        r1 = r0 + part.nray
        assert np.array_equal(o.rad, out.rad[:, r0:r1], equal_nan=True)
        assert np.array_equal(o.tau, out.tau[:, r0:r1], equal_nan=True)
        assert np.array_equal(o.tp, out.tp[:, r0:r1], equal_nan=True)
        r0 = r1


@pytest.mark.parametrize("kind", ["nadir", "limb"])
def test_bound_mode_matches_slabs_and_counts(built_lib, kind):
    if kind == "nadir":
        w = synth.config_nadir(NRAY, nd=4, nlev=51, ztop=60.0, emitters=("CO2", "H2O"))
    else:   # tangent heights 5-60 km, RAYDZ 0.1 km, refraction on
        w = synth.config_limb_cga(NRAY, nd=4, emitters=("CO2", "H2O"), raydz=0.1)
    ctl, batch = w.ctl, w.batch
    ctx = native.Context(ctl, w.tables, w.filters)
    out = ctx.formod_batch(batch.fresh_outputs(), native.MIXED)
    st = ctx.stats()
    assert st["trace_passes"] == 1                       # the bound held for every ray
    assert np.all(np.isfinite(out.rad)) and np.all(out.rad > 0)
    _same_as_parts(ctx, ctl, batch, out)
    # bound too small for most rays: one failed pass, then counts
    ctx.set_los_bound_scale(0.3)
    o = ctx.formod_batch(batch.fresh_outputs(), native.MIXED)
    assert ctx.stats()["trace_passes"] == 3
    assert ctx.stats()["los_points"] == st["los_points"]
    assert np.array_equal(o.rad, out.rad) and np.array_equal(o.tau, out.tau)
    # bound off: count first
    ctx.set_los_bound_scale(0.0)
    o = ctx.formod_batch(batch.fresh_outputs(), native.MIXED)
    assert ctx.stats()["trace_passes"] == 2
    assert np.array_equal(o.rad, out.rad) and np.array_equal(o.tp, out.tp)
    with pytest.raises(Exception, match="LOS bound"):
        ctx.set_los_bound_scale(-1.0)


def test_bound_mode_los_overflow_is_an_error(built_lib):
    # 0-60 km nadir needs ~600 LOS points per ray; NLOS = 300 (bound clamped
    # to NLOS): the reference's "Too many LOS points!" in every mode
    w = synth.config_nadir(2 ** 23 // 300 + 64, nd=2, nlev=31, ztop=60.0, emitters=("CO2",))
    ctx = native.Context(w.ctl, w.tables, w.filters, nlos_max=300)
    for scale in (1.0, 0.0):
        ctx.set_los_bound_scale(scale)
        with pytest.raises(Exception, match="Too many LOS points"):
            ctx.formod_batch(w.batch.fresh_outputs(), native.MIXED)
    ok = synth.config_nadir(4, nd=2, nlev=31, ztop=20.0, emitters=("CO2",))
    ctx2 = native.Context(ok.ctl, ok.tables, ok.filters, nlos_max=300)
    out = ctx2.formod_batch(ok.batch.fresh_outputs(), native.MIXED)
    assert np.all(np.isfinite(out.rad))
