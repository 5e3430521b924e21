"""Finite-difference Jacobian on the GPU (jgb_kernel_batch) against the CPU
oracle's kernel() (restatement of jurassic.c:4004-4099).

FP64: every entry within 1e-7 of the largest |K| of its column (forward
      differences amplify the last-bit differences of the two forward models).
Mixed: the finite-difference radiance changes K_ij h_j agree with the FP64
      ones to 2e-5 of the radiance y_i (FP32 radiances carry ~1e-7 relative
      rounding noise, which the finite difference divides by the step; small
      columns are noise-dominated relative to their own size but not
      relative to the measurement).
"""
import copy

import numpy as np
import pytest

import golden_io as G
from jurassic_gb300 import native, synth

pytestmark = pytest.mark.gpu


def _fd_noise(K, Kr, h, y):
    """max |K - Kr| h_j / |y_i|: error of the finite-difference radiance change
    relative to the radiance."""
    return np.max(np.abs(K - Kr) * h[None, :] / np.abs(y)[:, None])


def _steps(ora, atm):
    """Perturbation steps of kernel() (jurassic.c:4046-4068) from atm2x."""
    x, iqa, _ = ora.atm2x(atm)
    ng = ora.ctl.ng
    h = np.ones_like(x)
    h[iqa == 0] = np.maximum(np.abs(0.01 * x[iqa == 0]), 1e-7)
    q = (iqa >= 2) & (iqa < 2 + ng)
    h[q] = np.maximum(np.abs(0.01 * x[q]), 1e-15)
    h[(iqa >= 2 + ng) & (iqa < 2 + ng + ora.ctl.nw)] = 1e-4
    return h


def _yvec(rad):
    """obs2y order: ray-major, finite channels only."""
    return np.array([v for col in rad.T for v in col if np.isfinite(v)])


def _colrel(K, Kr):
    scale = np.maximum(np.max(np.abs(Kr), axis=0, keepdims=True), 1e-300)
    return np.max(np.abs(K - Kr) / scale)


def test_kernel_golden_case(built_lib, built_oracle):
    from oracle import oracle
    f = G.load("ref_kernel.npz")
    ctl = G.ctl_from(f["ctl"])
    tbl, filt = G.tables_from(f), G.filters_from(f, ctl.nd)
    atm = G.atm_from(f, "atm_", ctl)
    obs = G.obs_from(f, "obs_", ctl.nd)
    ctx = native.Context(ctl, tbl, filt)
    K64 = ctx.kernel(atm, obs, native.FP64)
    assert K64.shape == f["K"].shape
    assert _colrel(K64, f["K"]) <= 1e-7
    K32 = ctx.kernel(atm, obs, native.MIXED)
    ora = oracle.Oracle(ctl, tbl, filt)
    rad, _, _, _ = ora.formod(atm.copy(), obs)
    assert _fd_noise(K32, f["K"], _steps(ora, atm), _yvec(rad)) <= 2e-5


def test_kernel_batch_nadir_vs_oracle(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_nadir(5, nd=6, nlev=41, ztop=40.0, emitters=("CO2", "H2O", "O3"))
    ctl = copy.deepcopy(w.ctl)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 30.0
    ctl.retq_zmin = np.array([-999.0, 0.0, 15.0])
    ctl.retq_zmax = np.array([-999.0, 12.0, 35.0])
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    ctx = native.Context(ctl, w.tables, w.filters)
    b = w.batch.fresh_outputs()
    b.rad[2, 3] = np.nan  # one masked channel
    b.rad[3:, 1] = np.nan  # observation 1 measures channels 0-2 only: the
    # perturbed forward models skip its other channels
    Ks, out = ctx.kernel_batch(b, native.FP64)
    for i in range(b.nobs):
        atm, obs = b.item(w.ctl, i)
        Kr = ora.kernel(atm, obs)
        assert Ks[i].shape == Kr.shape
        assert _colrel(Ks[i], Kr) <= 1e-7, i
    ref = ora.formod_batch(b)
    fin = np.isfinite(ref.rad)
    assert np.array_equal(fin, np.isfinite(out.rad))
    assert np.max(np.abs(out.rad[fin] - ref.rad[fin]) / np.abs(ref.rad[fin])) <= 1e-9
    Km, _ = ctx.kernel_batch(b, native.MIXED)
    for i in range(b.nobs):
        atm, obs = b.item(w.ctl, i)
        y = _yvec(ref.rad[:, b.ray_off[i]:b.ray_off[i + 1]])
        assert _fd_noise(Km[i], Ks[i], _steps(ora, atm), y) <= 2e-5, i
