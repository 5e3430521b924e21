"""Mixed path loop split over the emitters (latency-bound batches) on the GPU.

The emitters' path states are independent along a line of sight
(intpol_tbl_ega / intpol_tbl_cga keep one tau_path per emitter); only their
per-point combination couples them.  The split form runs one warp per (tile,
channel, emitter) for the states and the unchanged combination and radiance
code per (tile, channel).  Its results equal the fused form's bit for bit:
EGA and CGA, limb and nadir, clouds, extinction windows, surface reflection
with the sun, hydrostatic pressures, FOV, and a whole retrieval.
"""
import copy

import numpy as np
import pytest

from jurassic_gb300 import native, synth
from jurassic_gb300.model import Ret

pytestmark = pytest.mark.gpu


def _both(ctx, batch):
    outs = []
    for mode in (1, 0):
        ctx.set_path_split(mode)
        outs.append(ctx.formod_batch(batch.fresh_outputs(), native.MIXED))
    ctx.set_path_split(-1)
    return outs


def _same(a, b):
    for k in ("rad", "tau", "tp"):
        assert np.array_equal(getattr(a, k), getattr(b, k), equal_nan=True), k


def _limb_cloud():
    w = synth.config_limb_ega(n_rays=8)
    ctl = copy.deepcopy(w.ctl)
    ctl.clnu = np.array([600.0, 900.0])
    ctl.hydz = 10.0
    items = []
    for i in range(3):
        atm, obs = w.batch.item(w.ctl, 0)
        atm.clz, atm.cldz = 12.0 + i, 2.0
        atm.clk = np.array([1e-3, 3e-3])
        items.append((atm, obs))
    return ctl, w, synth.pack(ctl, items)


def test_split_limb_clouds_hydrostatic(built_lib):
    ctl, w, batch = _limb_cloud()
    ctx = native.Context(ctl, w.tables, w.filters)
    a, b = _both(ctx, batch)
    assert ctx.stats()["path_launches"] > 0
    _same(a, b)
    assert np.all(np.isfinite(a.rad))


def test_split_nadir_surface_sun(built_lib):
    w = synth.config_nadir(40, nd=6, nlev=61, ztop=60.0, numin=700, numax=2300)
    ctl = copy.deepcopy(w.ctl)
    ctl.sfnu = np.array([600.0, 1500.0, 2500.0])
    ctl.sftype = 3
    ctl.sfsza = -999.0
    items = []
    for i in range(w.batch.nobs):
        atm, obs = w.batch.item(w.ctl, i)
        atm.sfz, atm.sfp, atm.sft = 0.0, 0.0, 285.0 + i
        atm.sfeps = np.array([0.95, 0.8, 0.9])
        items.append((atm, obs))
    batch = synth.pack(ctl, items)
    ctx = native.Context(ctl, w.tables, w.filters)
    a, b = _both(ctx, batch)
    _same(a, b)


def test_split_cga_and_fov(built_lib):
    w = synth.config_limb_cga(64, nd=8, emitters=("CO2", "H2O", "O3"))
    ctx = native.Context(w.ctl, w.tables, w.filters)
    _same(*_both(ctx, w.batch))
    w2 = synth.config_limb_ega(n_rays=10)
    dz = np.linspace(-2.0, 2.0, 21)
    ctx2 = native.Context(w2.ctl, w2.tables, w2.filters, fov=(dz, np.exp(-dz ** 2)))
    _same(*_both(ctx2, w2.batch))


def test_split_retrieval_identical(built_lib, built_oracle):
    w = synth.config_nadir(1, nd=8, nlev=31, ztop=60.0, emitters=("CO2", "H2O"),
                           numin=660.0, numax=1600.0)
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 40.0
    ctl.retq_zmin = np.array([-999.0, 0.0])
    ctl.retq_zmax = np.array([-999.0, 14.0])
    from oracle import oracle
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    items = synth.retrieval_requests(ctl, lambda b: ora.formod_batch(b.fresh_outputs()), 3, 9,
                                     nlev=(21, 31))
    ret = Ret(kernel_recomp=1, conv_itmax=4, conv_dmin=0.01, err_ana=1,
              err_noise=np.full(ctl.nd, 1e-4), err_formod=np.full(ctl.nd, 0.5),
              err_temp=2.0, err_temp_cz=3.0, err_temp_ch=500.0,
              err_q=np.array([0.0, 30.0]), err_q_cz=np.array([-999.0, 3.0]),
              err_q_ch=np.array([-999.0, 500.0]))
    ctx = native.Context(ctl, w.tables, w.filters)
    res = []
    for mode in (1, 0):
        ctx.set_path_split(mode)
        res.append(ctx.engine(ret, native.MIXED).run(synth.pack(ctl, items)))
    for a, b in zip(*res):
        for k in ("x", "costs", "rad", "cov", "avk"):
            assert np.array_equal(np.asarray(a[k]), np.asarray(b[k]), equal_nan=True), k
        assert a["iters"] == b["iters"] and a["status"] == b["status"] == 0
    with pytest.raises(Exception, match="split"):
        ctx.set_path_split(2)
