"""Resumed finite-difference perturbations (mixed-precision kernel()) on the
GPU.

A perturbation of a level value changes the atmosphere only on the two
intervals next to the level, so the perturbed ray's LOS points and path
state equal its unperturbed base's until the ray comes near those levels;
the perturbed path restarts there from the base's saved state.  A
perturbation of one emitter's mixing ratio also leaves the other emitters'
states equal to the base's all along the path, so their segment
emissivities can be taken from the base's walk.  The Jacobians (and a whole
retrieval) are bit-identical in every mode -- resumed with emitters always
shared (mode 3), resumed (2, sharing where it pays), plain (0), automatic
(1): nadir with masked channels, refracted limb EGA, limb CGA, limb EGA with
window extinctions and pressures.  In EGA the perturbed rays' tracing is
resumed too: a perturbed mixing ratio or extinction takes the base ray's
geometry, a perturbed temperature walks on from the base's walk.
"""
import copy

import numpy as np
import pytest

from jurassic_gb300 import native, synth
from jurassic_gb300.model import Ret

pytestmark = pytest.mark.gpu


def _both(ctx, batch):
    """Jacobians resumed (forced) and plain; the resumed call must have
    skipped LOS points."""
    out = []
    for mode in (3, 2, 0, 1):
        ctx.set_fd_resume(mode)
        Ks, fm = ctx.kernel_batch(batch.fresh_outputs(), native.MIXED)
        out.append(Ks)
        if mode == 2:
            skip = ctx.stats()["resume_skip"]
    ctx.set_fd_resume(1)
    return out, skip


def _same(res):
    (Kd, Ka, Kb, Kc), skip = res
    assert skip > 0.05
    assert len(Ka) == len(Kb) == len(Kc) == len(Kd)
    for a, b, c, d in zip(Ka, Kb, Kc, Kd):
        assert a.shape == b.shape
        assert np.array_equal(a, b) and np.array_equal(a, c) and np.array_equal(a, d)
        assert np.all(np.isfinite(a))


def test_resume_nadir_masked(built_lib):
    w = synth.config_nadir(5, nd=6, nlev=41, ztop=40.0, emitters=("CO2", "H2O", "O3"))
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 30.0
    ctl.retq_zmin = np.array([-999.0, 0.0, 15.0])
    ctl.retq_zmax = np.array([-999.0, 12.0, 35.0])
    b = w.batch.fresh_outputs()
    b.rad[2, 3] = np.nan
    b.rad[3:, 1] = np.nan
    ctx = native.Context(ctl, w.tables, w.filters)
    _same(_both(ctx, b))


@pytest.mark.parametrize("formod", [1, 0])
def test_resume_limb(built_lib, formod):
    w = synth.config_limb_ega(n_rays=8, formod=formod)
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 5.0, 45.0
    ctl.retq_zmin = np.array([-999.0, 5.0])
    ctl.retq_zmax = np.array([-999.0, 30.0])
    items = [w.batch.item(w.ctl, 0) for _ in range(3)]
    for i, (atm, obs) in enumerate(items):
        atm.t = atm.t + i                       # three different atmospheres
    ctx = native.Context(ctl, w.tables, w.filters)
    _same(_both(ctx, synth.pack(ctl, items)))


def test_resume_limb_extinction_pressure(built_lib):
    """Window extinctions (whose perturbed rays take their base's geometry)
    and pressures (which walk from the start) next to temperatures and a
    mixing ratio, on refracted limb rays that cross the perturbed levels and
    rays that stay above them."""
    w = synth.config_limb_ega(n_rays=8, formod=1)
    ctl = copy.deepcopy(w.ctl)
    ctl.window = np.array([0, 0, 0], dtype=np.int32)
    ctl.rett_zmin, ctl.rett_zmax = 5.0, 45.0
    ctl.retp_zmin, ctl.retp_zmax = 18.0, 26.0
    ctl.retq_zmin = np.array([-999.0, 8.0])
    ctl.retq_zmax = np.array([-999.0, 20.0])
    ctl.retk_zmin = np.array([12.0])
    ctl.retk_zmax = np.array([36.0])
    items = [w.batch.item(w.ctl, 0) for _ in range(2)]
    for i, (atm, obs) in enumerate(items):
        atm.t = atm.t - 2 * i
        atm.k = np.where((atm.z >= 10) & (atm.z <= 40), 1e-3 * (1 + i), 0.0)[None, :]
    ctx = native.Context(ctl, w.tables, w.filters)
    _same(_both(ctx, synth.pack(ctl, items)))


def test_resume_retrieval_identical(built_lib, built_oracle):
    w = synth.config_nadir(1, nd=8, nlev=31, ztop=60.0, emitters=("CO2", "H2O"),
                           numin=660.0, numax=1600.0)
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 40.0
    ctl.retq_zmin = np.array([-999.0, 0.0])
    ctl.retq_zmax = np.array([-999.0, 14.0])
    from oracle import oracle
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    items = synth.retrieval_requests(ctl, lambda b: ora.formod_batch(b.fresh_outputs()), 4, 11,
                                     nlev=(21, 31))
    ret = Ret(kernel_recomp=1, conv_itmax=4, conv_dmin=0.01, err_ana=1,
              err_noise=np.full(ctl.nd, 1e-4), err_formod=np.full(ctl.nd, 0.5),
              err_temp=2.0, err_temp_cz=3.0, err_temp_ch=500.0,
              err_q=np.array([0.0, 30.0]), err_q_cz=np.array([-999.0, 3.0]),
              err_q_ch=np.array([-999.0, 500.0]))
    ctx = native.Context(ctl, w.tables, w.filters)
    res = []
    for mode in (3, 2, 0):
        ctx.set_fd_resume(mode)
        res.append(ctx.engine(ret, native.MIXED).run(synth.pack(ctl, items)))
    for a, b, c in zip(*res):
        for k in ("x", "costs", "rad", "tau", "cov", "avk"):
            assert np.array_equal(np.asarray(a[k]), np.asarray(b[k]), equal_nan=True), k
            assert np.array_equal(np.asarray(a[k]), np.asarray(c[k]), equal_nan=True), k
        assert a["iters"] == b["iters"] == c["iters"] and a["status"] == b["status"] == 0
