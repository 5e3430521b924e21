"""Parity of the CUDA forward model against the CPU oracle (restatement of
the reference formod, pinned bit-exact to the reference build).

FP64 path: relative radiance error <= 1e-9 (rounding-level; CUDA's libm and
           the host libm differ in the last bits).
Mixed path: |BT_gpu - BT_oracle| <= 10 mK per (ray, channel), BT from the
           reference's BRIGHT formula in FP64; tangent point within 2 m and
           1e-4 degrees (mixed ray tracing).
"""
import copy

import numpy as np
import pytest

from jurassic_gb300 import native, synth
from jurassic_gb300.model import brightness

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9
BT_TOL_K = 0.010


def _bt(ctl, rad):
    return brightness(rad, np.asarray(ctl.nu)[:, None])


def _check(ctl, ref, out, precision, what=""):
    rad_ref, tau_ref, tp_ref = ref
    fin = np.isfinite(rad_ref)
    assert np.array_equal(fin, np.isfinite(out.rad)), "mask differs " + what
    if precision == native.FP64:
        rel = np.max(np.abs(out.rad[fin] - rad_ref[fin]) / np.maximum(np.abs(rad_ref[fin]), 1e-300))
        assert rel <= FP64_RTOL, "%s FP64 rad rel %.3e" % (what, rel)
        assert np.max(np.abs(out.tau - tau_ref)) <= 1e-10, what
    else:
        if ctl.write_bbt:
            dbt = np.max(np.abs(out.rad[fin] - rad_ref[fin]))
        else:
            dbt = np.max(np.abs(_bt(ctl, out.rad)[fin] - _bt(ctl, rad_ref)[fin]))
        assert dbt <= BT_TOL_K, "%s mixed |dBT| %.4f K" % (what, dbt)
        assert np.max(np.abs(out.tau - tau_ref)) <= 2e-4, what
    tp = np.stack([out.tpz, out.tplon, out.tplat])
    if precision == native.FP64:
        assert np.max(np.abs(tp - tp_ref)) <= 1e-8, what
    else:
        # mixed ray tracing: FP32 altitude increments and atmosphere, FP64
        # position; tangent altitude within 2 m, longitude/latitude 1e-4 deg
        assert np.max(np.abs(tp[0] - tp_ref[0])) <= 2e-3, what
        assert np.max(np.abs(tp[1:] - tp_ref[1:])) <= 1e-4, what


def _run_single(w, ctl=None, precisions=(native.FP64, native.MIXED), atm_mod=None, obs_mod=None):
    from oracle import oracle
    ctl = ctl or w.ctl
    atm, obs = w.batch.item(w.ctl, 0)
    if atm_mod:
        atm_mod(atm)
    if obs_mod:
        obs_mod(obs)
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    rad, tau, tp, p = ora.formod(atm.copy(), obs)
    ctx = native.Context(ctl, w.tables, w.filters)
    for prec in precisions:
        a2 = atm.copy()
        out = ctx.formod(a2, obs, prec)
        _check(ctl, (rad, tau, tp), out, prec, "prec=%d" % prec)
        if ctl.hydz >= 0:
            assert np.allclose(a2.p, p, rtol=1e-12, atol=0)
    ctx.close()
    ora.close()


def test_srcfunc_matches_oracle(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_limb_ega()
    ora = oracle.Oracle(w.ctl, w.tables, w.filters)
    ctx = native.Context(w.ctl, w.tables, w.filters)
    st0, sr0 = ora.srcfunc()
    st1, sr1 = ctx.srcfunc()
    assert np.array_equal(st0, st1)
    assert np.max(np.abs(sr1 - sr0) / sr0) < 1e-13


def test_limb_ega(built_lib, built_oracle):
    _run_single(synth.config_limb_ega())


def test_limb_cga(built_lib, built_oracle):
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.formod = 0
    _run_single(w, ctl)


def test_limb_bt_and_mask(built_lib, built_oracle):
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.write_bbt = 1

    def mask(obs):
        obs.rad[1, 2] = np.nan
        obs.rad[0, 5] = np.nan
    _run_single(w, ctl, obs_mod=mask)


def test_no_continua_no_refraction(built_lib, built_oracle):
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.ctm_co2 = ctl.ctm_h2o = ctl.ctm_n2 = ctl.ctm_o2 = 0
    ctl.refrac = 0
    _run_single(w, ctl)


def test_nadir_surface_reflection_solar(built_lib, built_oracle):
    w = synth.config_nadir(1, nd=6, nlev=61, ztop=60.0, numin=700, numax=2300)
    for sftype in (1, 2, 3):
        ctl = copy.deepcopy(w.ctl)
        ctl.sfnu = np.array([600.0, 1500.0, 2500.0])
        ctl.sftype = sftype
        ctl.sfsza = -999.0 if sftype == 3 else 30.0

        def surf(atm):
            atm.sfz, atm.sfp, atm.sft = 0.0, 0.0, 290.0
            atm.sfeps = np.array([0.95, 0.8, 0.9])
        _run_single(w, ctl, atm_mod=surf)


def test_clouds_and_extinction(built_lib, built_oracle):
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.clnu = np.array([600.0, 900.0])

    def cloud(atm):
        atm.clz, atm.cldz = 12.0, 2.0
        atm.clk = np.array([1e-3, 3e-3])
        atm.k[0] = 1e-4 * np.exp(-atm.z / 10.0)
    _run_single(w, ctl, atm_mod=cloud)


def test_hydrostatic(built_lib, built_oracle):
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.hydz = 10.0
    _run_single(w, ctl)


def test_missing_and_short_tables(built_lib, built_oracle):
    w = synth.config_limb_ega()
    tbl = copy.deepcopy(w.tables)
    tbl.np_[1, 1] = -1          # missing file
    tbl.np_[2, 0] = 20          # fewer than 30 pressure levels -> eps = 0
    w2 = synth.Workload(w.name, w.ctl, tbl, w.filters, w.batch)
    _run_single(w2)


def test_batch_equals_single(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_nadir(24, nd=8, nlev=51, ztop=50.0)
    ctl = w.ctl
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    ref = ora.formod_batch(w.batch.fresh_outputs())
    ctx = native.Context(ctl, w.tables, w.filters)
    for prec in (native.FP64, native.MIXED):
        out = ctx.formod_batch(w.batch.fresh_outputs(), prec)
        if prec == native.FP64:
            rel = np.max(np.abs(out.rad - ref.rad) / np.abs(ref.rad))
            assert rel <= FP64_RTOL, rel
        else:
            dbt = np.max(np.abs(_bt(ctl, out.rad) - _bt(ctl, ref.rad)))
            assert dbt <= BT_TOL_K, dbt
        for i in (0, 7, 23):
            atm, obs = w.batch.item(ctl, i)
            one = ctx.formod(atm, obs, prec)
            sl = slice(w.batch.ray_off[i], w.batch.ray_off[i + 1])
            assert np.array_equal(one.rad, out.rad[:, sl])


def test_limb_cga_batch_uneven(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_limb_cga(64, nd=6)
    ctl = w.ctl
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    ref = ora.formod_batch(w.batch.fresh_outputs())
    ctx = native.Context(ctl, w.tables, w.filters)
    out = ctx.formod_batch(w.batch.fresh_outputs(), native.FP64)
    rel = np.max(np.abs(out.rad - ref.rad) / np.abs(ref.rad))
    assert rel <= FP64_RTOL, rel
    out = ctx.formod_batch(w.batch.fresh_outputs(), native.MIXED)
    dbt = np.max(np.abs(_bt(ctl, out.rad) - _bt(ctl, ref.rad)))
    assert dbt <= BT_TOL_K, dbt


def test_contributions_task_c(built_lib, built_oracle):
    """TASK c (formod.c:200-249): per-emitter and extinction-only forward
    models with the continua off, against the oracle run on the same
    modified atmospheres."""
    from oracle import oracle
    w = synth.config_limb_ega()
    ctl = w.ctl
    atm, obs = w.batch.item(ctl, 0)
    atm.k = np.where(atm.z < 20.0, 1e-3, 0.0)[None, :] * np.ones((ctl.nw, 1))
    batch = synth.pack(ctl, [(atm, obs)])
    ctl_off = copy.deepcopy(ctl)
    ctl_off.ctm_co2 = ctl_off.ctm_h2o = ctl_off.ctm_n2 = ctl_off.ctm_o2 = 0
    ora = oracle.Oracle(ctl_off, w.tables, w.filters)
    refs = []
    for v in range(ctl.ng + 1):
        a2 = atm.copy()
        a2.k = np.zeros_like(a2.k) if v < ctl.ng else a2.k
        a2.q = np.array([a2.q[g] if g == v else np.zeros_like(a2.q[g]) for g in range(ctl.ng)])
        refs.append(ora.formod(a2, obs))
    ctx = native.Context(ctl, w.tables, w.filters)
    for prec in (native.FP64, native.MIXED):
        rad, tau = ctx.contributions(batch, prec)
        for v in range(ctl.ng + 1):
            r_ref, t_ref = refs[v][0], refs[v][1]
            pos = r_ref > 0            # rays above the extinction layer see nothing (EXTINCT)
            assert np.all(np.abs(rad[v][~pos]) <= 1e-15), v
            if prec == native.FP64:
                assert np.max(np.abs(rad[v][pos] - r_ref[pos]) / r_ref[pos]) <= FP64_RTOL, v
                assert np.max(np.abs(tau[v] - t_ref)) <= 1e-10, v
            else:
                dbt = np.abs(_bt(ctl, rad[v])[pos] - _bt(ctl, r_ref)[pos])
                assert np.max(dbt) <= BT_TOL_K, v
        # the context's own continua are back on afterwards
        out = ctx.formod(atm.copy(), obs, native.FP64)
        assert np.allclose(out.rad, ctx.formod(atm.copy(), obs, native.FP64).rad)
