"""Edge cases of the device forward model and retrieval, in both precisions.

* The reference's fatal errors come back as status codes and leave the
  context usable: "Too many LOS points!" (jurassic.c:4335) and "Observer
  below surface!" (jurassic.c:4238).
* A ray whose view point lies above the atmosphere gets no LOS (raytrace
  returns no points): its results equal the oracle's; an observation with
  every channel masked returns NaN everywhere; both mixed into a batch with
  ordinary observations that stay correct.
* Results per observation do not depend on the order of the batch.
* The batch retrieval rejects more than 65535 observations before any work.
"""
import copy

import numpy as np
import pytest

from jurassic_gb300 import native, synth
from jurassic_gb300.model import JurassicError, Ret, brightness

pytestmark = pytest.mark.gpu

PRECISIONS = (native.FP64, native.MIXED)


def test_los_overflow_is_an_error_and_context_recovers(built_lib):
    # 0-4 km nadir atmosphere: ~41 LOS points (RAYDZ = 0.1 km), within a
    # 50-point limit; a limb ray through the layer with RAYDS = 0.5 km needs
    # hundreds
    w = synth.config_nadir(3, nd=4, nlev=9, ztop=4.0, emitters=("CO2", "H2O"))
    ctl = copy.deepcopy(w.ctl)
    ctl.rayds = 0.5
    ctx = native.Context(ctl, w.tables, w.filters, nlos_max=50)
    atm, _ = w.batch.item(ctl, 0)
    obs = synth.limb_obs(ctl.nd, [1.0])
    for prec in PRECISIONS:
        with pytest.raises(JurassicError, match="Too many LOS points"):
            ctx.formod(atm.copy(), obs, prec)
        out = ctx.formod_batch(w.batch.fresh_outputs(), prec)   # the context still works
        assert np.all(np.isfinite(out.rad)) and np.all(out.rad > 0)


def test_observer_below_surface_is_an_error(built_lib):
    w = synth.config_nadir(2, nd=4, nlev=31, ztop=60.0, emitters=("CO2", "H2O"))
    ctx = native.Context(w.ctl, w.tables, w.filters)
    atm, obs = w.batch.item(w.ctl, 0)
    obs.obsz = np.full_like(obs.obsz, -1.0)
    for prec in PRECISIONS:
        with pytest.raises(JurassicError, match="Observer below surface"):
            ctx.formod(atm.copy(), obs, prec)
        out = ctx.formod_batch(w.batch.fresh_outputs(), prec)
        assert np.all(np.isfinite(out.rad))


def test_ray_above_atmosphere_and_fully_masked_observation(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_limb_ega(n_rays=4)
    ctl = w.ctl
    atm, obs = w.batch.item(ctl, 0)
    high = synth.limb_obs(ctl.nd, [20.0, 95.0])     # second view point above the 80 km top
    masked = obs.copy()
    masked.rad = np.full_like(masked.rad, np.nan)
    items = [(atm, obs), (atm.copy(), high), (atm.copy(), masked)]
    batch = synth.pack(ctl, items)
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    ref = ora.formod_batch(batch.fresh_outputs())
    ctx = native.Context(ctl, w.tables, w.filters)
    nu = np.asarray(ctl.nu)[:, None]
    r0, r1 = batch.ray_off[2], batch.ray_off[3]
    for prec in PRECISIONS:
        out = ctx.formod_batch(batch.fresh_outputs(), prec)
        assert np.all(np.isnan(out.rad[:, r0:r1]))
        fin = np.isfinite(ref.rad)
        assert np.array_equal(fin, np.isfinite(out.rad))
        pos = fin & (ref.rad > 0)
        if prec == native.FP64:
            assert np.max(np.abs(out.rad[pos] - ref.rad[pos]) / ref.rad[pos]) <= 1e-9
        else:
            dbt = np.abs(brightness(out.rad, nu) - brightness(ref.rad, nu))[pos]
            assert np.max(dbt) <= 0.010
        # no LOS: nothing emits, nothing absorbs; tangent point = view point
        hr = batch.ray_off[1] + 1
        assert np.all(out.rad[:, hr] == ref.rad[:, hr])
        assert np.all(out.tau[:, hr] == ref.tau[:, hr])
        assert out.tp[0, hr] == batch.geo[4, hr]


def test_results_do_not_depend_on_batch_order(built_lib):
    w = synth.config_nadir(300, nd=8, nlev=51, ztop=50.0, emitters=("CO2", "H2O", "O3"))
    ctl = w.ctl
    ctx = native.Context(ctl, w.tables, w.filters)
    order = np.random.default_rng(3).permutation(w.batch.nobs)
    shuffled = synth.pack(ctl, [w.batch.item(ctl, int(i)) for i in order])
    for prec in PRECISIONS:
        a = ctx.formod_batch(w.batch.fresh_outputs(), prec)
        b = ctx.formod_batch(shuffled.fresh_outputs(), prec)
        for k, i in enumerate(order):
            ra = a.rad[:, a.ray_off[i]:a.ray_off[i + 1]]
            rb = b.rad[:, b.ray_off[k]:b.ray_off[k + 1]]
            assert np.array_equal(ra, rb), (prec, int(i))


def test_retrieval_batch_limit(built_lib):
    w = synth.config_nadir(65536, nd=2, nlev=3, ztop=10.0, emitters=("CO2",))
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 10.0
    ctx = native.Context(ctl, w.tables, w.filters)
    ret = Ret(kernel_recomp=1, conv_itmax=1, err_noise=np.full(2, 1e-4),
              err_formod=np.full(2, 1.0), err_temp=1.0)
    with pytest.raises(JurassicError, match="65535"):
        ctx.retrieve_batch(ret, w.batch, native.FP64)
