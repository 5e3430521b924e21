"""Field-of-view convolution (formod_fov, jurassic.c:3121-3192) on the GPU.

Against the reference's own output (golden fixture made by running the
reference with a FOV file) and against the CPU oracle on a batch with two
observations and rays of different times: FP64 within 1e-9 relative, mixed
within 10 mK; the FP64 Jacobian with FOV within 1e-7 per column of the
oracle's kernel().
"""
import copy

import numpy as np
import pytest

import golden_io as G
from jurassic_gb300 import native, synth
from jurassic_gb300.model import brightness

pytestmark = pytest.mark.gpu


def _fov():
    dz = np.linspace(-2.0, 2.0, 21)
    return dz, np.exp(-dz ** 2)


@pytest.mark.parametrize("case", ["ega", "bbt"])
def test_fov_golden(built_lib, case):
    f = G.load("ref_formod_fov.npz")
    ctl = G.ctl_from(f[case + "_ctl"])
    ctx = native.Context(ctl, G.tables_from(f), G.filters_from(f, ctl.nd),
                         fov=(f["fov_dz"], f["fov_w"]))
    atm = G.atm_from(f, "atm_", ctl)
    obs = G.obs_from(f, "obs_", ctl.nd)
    ref = f[case + "_rad"]
    fin = np.isfinite(ref)
    nu = np.asarray(ctl.nu)[:, None]
    for prec in (native.FP64, native.MIXED):
        out = ctx.formod(atm.copy(), obs, prec)
        assert np.array_equal(np.isfinite(out.rad), fin)
        if prec == native.FP64:
            assert np.max(np.abs(out.rad[fin] - ref[fin]) / np.abs(ref[fin])) <= 1e-9
            assert np.max(np.abs(out.tau - f[case + "_tau"])) <= 1e-10
        else:
            bt = out.rad if ctl.write_bbt else brightness(out.rad, nu)
            bt_ref = ref if ctl.write_bbt else brightness(ref, nu)
            assert np.max(np.abs(bt[fin] - bt_ref[fin])) <= 0.010


def _batch_two_times():
    w = synth.config_limb_ega(n_rays=8)
    ctl = w.ctl
    atm, obs = w.batch.item(ctl, 0)
    obs2 = obs.copy()
    obs2.time = obs2.time.copy()
    obs2.time[4:] += 60.0        # second scan in the same observation
    return w, ctl, [(atm, obs), (atm.copy(), obs2)]


def test_fov_batch_vs_oracle(built_lib, built_oracle):
    from oracle import oracle
    w, ctl, items = _batch_two_times()
    ora = oracle.Oracle(ctl, w.tables, w.filters, fov=_fov())
    ctx = native.Context(ctl, w.tables, w.filters, fov=_fov())
    batch = synth.pack(ctl, items)
    ref = ora.formod_batch(batch.fresh_outputs())
    nu = np.asarray(ctl.nu)[:, None]
    out64 = ctx.formod_batch(batch.fresh_outputs(), native.FP64)
    assert np.max(np.abs(out64.rad - ref.rad) / np.abs(ref.rad)) <= 1e-9
    out32 = ctx.formod_batch(batch.fresh_outputs(), native.MIXED)
    assert np.max(np.abs(brightness(out32.rad, nu) - brightness(ref.rad, nu))) <= 0.010
    # FOV off again: pencil beams only
    ctx.set_fov([], [])
    ora2 = oracle.Oracle(ctl, w.tables, w.filters)
    ref2 = ora2.formod_batch(batch.fresh_outputs())
    out = ctx.formod_batch(batch.fresh_outputs(), native.FP64)
    assert np.max(np.abs(out.rad - ref2.rad) / np.abs(ref2.rad)) <= 1e-9
    assert np.max(np.abs(ref2.rad - ref.rad)) > 0


def test_fov_jacobian_fp64_vs_oracle(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_limb_ega(n_rays=6)
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 5.0, 45.0
    atm, obs = w.batch.item(w.ctl, 0)
    ora = oracle.Oracle(ctl, w.tables, w.filters, fov=_fov())
    K_ref = ora.kernel(atm.copy(), obs)
    ctx = native.Context(ctl, w.tables, w.filters, fov=_fov())
    K = ctx.kernel(atm.copy(), obs, native.FP64)
    assert K.shape == K_ref.shape
    scale = np.maximum(np.max(np.abs(K_ref), axis=0), 1e-300)
    assert np.max(np.abs(K - K_ref) / scale) <= 1e-7


def test_fov_too_few_rays_is_an_error(built_lib, built_oracle):
    w = synth.config_limb_ega(n_rays=1)
    ctx = native.Context(w.ctl, w.tables, w.filters, fov=_fov())
    atm, obs = w.batch.item(w.ctl, 0)
    with pytest.raises(Exception, match="FOV"):
        ctx.formod(atm, obs, native.FP64)
