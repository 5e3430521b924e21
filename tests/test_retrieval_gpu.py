"""Optimal-estimation retrieval on the GPU (jgb_retrieve_batch) against the
CPU oracle (restatement of optimal_estimation, retrieval.c:448-749, pinned to
the reference build) and the reference's own golden retrieval.

FP64: final state within 1e-6 relative of the oracle, costs within 1e-6,
      covariance within 1e-6 of its largest entry (forward models agree to
      ~1e-13; the LM decisions are identical).
Mixed (FP32 forward model and Jacobian, 3xTF32 normal equations, FP64
      Cholesky/LM): final state within 0.05 posterior standard deviations of
      the FP64 retrieval.
"""
import copy

import numpy as np
import pytest

import golden_io as G
from jurassic_gb300 import native, synth
from jurassic_gb300.model import Ret

pytestmark = pytest.mark.gpu


def _golden():
    f = G.load("ref_retrieval.npz")
    ctl = G.ctl_from(f["ctl"])
    ret = G.ret_from(f["ret"])
    tbl, filt = G.tables_from(f), G.filters_from(f, ctl.nd)
    apr = G.atm_from(f, "atm_", ctl)
    meas = G.obs_from(f, "obs_", ctl.nd)
    return f, ctl, ret, tbl, filt, apr, meas


def test_retrieval_golden_fp64(built_lib, built_oracle):
    f, ctl, ret, tbl, filt, apr, meas = _golden()
    ctx = native.Context(ctl, tbl, filt)
    out = ctx.retrieve_batch(ret, synth.pack(ctl, [(apr, meas)]), native.FP64)
    x = out["x"][0]
    assert len(x) == len(f["x"])
    assert np.max(np.abs(x - f["x"]) / np.maximum(np.abs(f["x"]), 1e-300)) <= 1e-6
    assert np.allclose(out["costs"][0], f["costs"], rtol=1e-5)   # reference prints %g
    cov = out["cov"][0]
    assert np.max(np.abs(cov - f["cov"])) <= 1e-6 * np.max(np.abs(f["cov"]))


def test_error_analysis_golden_fp64(built_lib, built_oracle):
    """Gain, averaging kernel, noise/formod/total error and analyze_avk
    outputs of the engine against the reference's own files
    (matrix_gain.tab, matrix_avk.tab, atm_err_*.tab, atm_cont.tab,
    atm_res.tab, retrieval.c:668-726), within 1e-6 of each output's largest
    entry."""
    f, ctl, ret, tbl, filt, apr, meas = _golden()
    ctx = native.Context(ctl, tbl, filt)
    r = ctx.engine(ret, native.FP64, keep_gain=True).run(synth.pack(ctl, [(apr, meas)]))[0]
    assert r["status"] == 0
    for k in ("gain", "avk", "err_total", "err_noise", "err_formod", "cont", "res"):
        assert r[k].shape == f[k].shape, k
        assert np.max(np.abs(r[k] - f[k])) <= 1e-6 * np.max(np.abs(f[k])), k


def _nadir_retrievals(nobs=3):
    w = synth.config_nadir(nobs, nd=8, nlev=31, ztop=60.0, emitters=("CO2", "H2O"),
                           numin=660.0, numax=1600.0)
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 40.0
    ctl.retq_zmin = np.array([-999.0, 0.0])
    ctl.retq_zmax = np.array([-999.0, 14.0])
    from oracle import oracle
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    truth = ora.formod_batch(w.batch.fresh_outputs())
    meas = w.batch.fresh_outputs()
    rng = np.random.default_rng(9)
    meas.rad = truth.rad * (1 + 2e-3 * rng.standard_normal(truth.rad.shape))
    # a priori: the unperturbed standard atmosphere
    apr_items = []
    for i in range(nobs):
        a, o = meas.item(w.ctl, i)
        a0 = synth.profile(ctl.emitter, a.z, time=a.time[0], lon=a.lon[0], lat=a.lat[0])
        apr_items.append((a0, o))
    ret = Ret(kernel_recomp=1, conv_itmax=5, conv_dmin=0.01, err_ana=1,
              err_noise=np.full(ctl.nd, 1e-4), err_formod=np.full(ctl.nd, 0.5),
              err_temp=2.0, err_temp_cz=3.0, err_temp_ch=500.0,
              err_q=np.array([0.0, 30.0]), err_q_cz=np.array([-999.0, 3.0]),
              err_q_ch=np.array([-999.0, 500.0]))
    return ctl, w, ret, synth.pack(ctl, apr_items), ora


def test_retrieval_batch_fp64_vs_oracle(built_lib, built_oracle):
    ctl, w, ret, apr_batch, ora = _nadir_retrievals()
    ctx = native.Context(ctl, w.tables, w.filters)
    out = ctx.retrieve_batch(ret, apr_batch, native.FP64)
    for i in range(apr_batch.nobs):
        a, o = apr_batch.item(w.ctl, i)
        r = ora.retrieval(ret, a, o)
        assert np.max(np.abs(out["x"][i] - r["x"]) / np.maximum(np.abs(r["x"]), 1e-300)) <= 1e-6, i
        assert out["iters"][i] == r["iters"], i
        assert np.allclose(out["costs"][i], r["costs"], rtol=1e-6), i
        assert np.max(np.abs(out["cov"][i] - r["cov"])) <= 1e-6 * np.max(np.abs(r["cov"])), i


def test_retrieval_batch_mixed_vs_fp64(built_lib, built_oracle):
    ctl, w, ret, apr_batch, ora = _nadir_retrievals()
    ctx = native.Context(ctl, w.tables, w.filters)
    r64 = ctx.retrieve_batch(ret, apr_batch, native.FP64)
    r32 = ctx.retrieve_batch(ret, apr_batch, native.MIXED)
    for i in range(apr_batch.nobs):
        sig = np.sqrt(np.diag(r64["cov"][i]))
        assert np.max(np.abs(r32["x"][i] - r64["x"][i]) / sig) <= 0.05, i
