"""Parity at the benchmark configurations' own shapes (not reduced ones),
each against the CPU oracle (restatement of the reference, pinned to the
reference build) on seeded inputs of that shape.

* Nadir forward model (formod, jurassic.c:3026-3071; EGA, intpol_tbl_ega
  3799-3891): 100 channels on 650-2400 cm^-1, 5 emitters, 101 levels on
  0-100 km, tables of 41 pressures x 30 temperatures x 320 columns per
  (channel, emitter), 192 observations.  FP64 <= 1e-9 relative, mixed
  <= 10 mK brightness temperature.
* Limb CGA forward model (intpol_tbl_cga, 3710-3795): 32 channels, 3
  emitters, tangent heights uniform on 5-60 km at RAYDZ 0.5 km (paths of
  uneven length, batched together), 512 observations.  Same bounds.
* FD Jacobian (kernel, 4004-4099) at the Jacobian configuration: 150
  channels, 81 levels, T and 4 gases on all levels up to 80 km (n = 405), 2
  profiles.  The error of each finite-difference radiance change K_ij h_j
  relative to the radiance y_i: FP64 within 1e-11 (the two forward models
  agree to ~2e-13 of the radiance), mixed within 2e-5 (FP32 radiances carry
  ~1e-7 relative rounding noise); and FP64 within 1e-7 of each column's
  largest entry for the columns whose largest change is at least 1e-5 of
  the radiance.  Perturbations of the upper levels move the nadir
  radiances by only 1e-10 to 1e-6 of themselves (91 of the 405 columns of
  the first profile, 29-80 km), so a last-bit difference of the two FP64
  forward models is a large part of those columns; they are held by the
  first bound.  And the 3xTF32 normal equations K^T W K of those Jacobians
  within 1e-5 of the FP64 product (relative to its largest entry).
"""
import numpy as np
import pytest

from jurassic_gb300 import model, native, synth
from jurassic_gb300.model import brightness

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9
BT_TOL_K = 0.010


def _forward_vs_oracle(w, nthreads=0):
    from oracle import oracle
    ctl = w.ctl
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    ref = ora.formod_batch(w.batch.fresh_outputs(), nthreads=nthreads)
    ora.close()
    ctx = native.Context(ctl, w.tables, w.filters)
    out64 = ctx.formod_batch(w.batch.fresh_outputs(), native.FP64)
    out32 = ctx.formod_batch(w.batch.fresh_outputs(), native.MIXED)
    los = ctx.stats()["los_points"]
    ctx.close()
    fin = np.isfinite(ref.rad)
    assert fin.all()
    rel64 = np.max(np.abs(out64.rad - ref.rad) / np.abs(ref.rad))
    assert rel64 <= FP64_RTOL, rel64
    assert np.max(np.abs(out64.tau - ref.tau)) <= 1e-9
    nu = np.asarray(ctl.nu)[:, None]
    dbt = np.max(np.abs(brightness(out32.rad, nu) - brightness(ref.rad, nu)))
    assert dbt <= BT_TOL_K, dbt
    assert np.max(np.abs(out32.tau - ref.tau)) <= 1e-5
    return ref, out32, los


def test_nadir_100ch_5gas_101lev_full_tables(built_lib, built_oracle):
    w = synth.config_nadir(192)
    assert w.tables.u.shape == (100, 5, 41, 30, 320)
    assert w.batch.lev_off[1] - w.batch.lev_off[0] == 101
    ref, out32, los = _forward_vs_oracle(w)
    # nadir rays from 705 km through 0-100 km at RAYDZ 0.1: ~1000 points each
    assert los >= 900 * w.batch.nray


def test_limb_cga_32ch_uneven_paths(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_limb_cga(512)
    assert w.ctl.formod == 0 and w.ctl.nd == 32 and w.ctl.ng == 3
    ref, out32, los = _forward_vs_oracle(w)
    # the batch mixes short and long paths (tangent heights 5-60 km)
    ora = oracle.Oracle(w.ctl, w.tables, w.filters)
    pts = [len(ora.raytrace(*w.batch.item(w.ctl, i), 0)[0]) for i in range(0, 512, 8)]
    ora.close()
    assert min(pts) < 150 and max(pts) > 300, (min(pts), max(pts))
    assert abs(los - np.mean(pts) * 512) < 0.1 * los
    # tangent points: mixed ray tracing within 2 m of the FP64 oracle
    assert np.max(np.abs(out32.tp[0] - ref.tp[0])) <= 2e-3


def test_jacobian_150ch_n405_and_normal_equations(built_lib, built_oracle):
    from oracle import oracle
    w = synth.config_jacobian(2)
    ctl = w.ctl
    ctx = native.Context(ctl, w.tables, w.filters)
    m, n = ctx.kernel_sizes(w.batch)
    assert list(n) == [405, 405] and list(m) == [150, 150]
    K64, fm = ctx.kernel_batch(w.batch.fresh_outputs(), native.FP64)
    K32, _ = ctx.kernel_batch(w.batch.fresh_outputs(), native.MIXED)
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    for i in range(w.batch.nobs):
        atm, obs = w.batch.item(ctl, i)
        Kr = ora.kernel(atm, obs)
        assert Kr.shape == (150, 405)
        x, kind = model.atm2x(ctl, atm)
        h = model.fd_steps(ctl, x, kind)
        y = model.obs2y(fm.rad[:, w.batch.ray_off[i]:w.batch.ray_off[i + 1]])
        rel = lambda K: np.abs(K) * h[None, :] / np.abs(y)[:, None]
        fd64, fd32 = np.max(rel(K64[i] - Kr)), np.max(rel(K32[i] - Kr))
        signal = np.max(rel(Kr), axis=0)
        strong = signal >= 1e-5
        scale = np.maximum(np.max(np.abs(Kr), axis=0, keepdims=True), 1e-300)
        col = np.max((np.abs(K64[i] - Kr) / scale)[:, strong])
        info = (i, fd64, fd32, col, int(strong.sum()), float(signal.min()))
        assert fd64 <= 1e-11, info
        assert col <= 1e-7, info
        assert fd32 <= 2e-5, info
    ora.close()
    # K^T W K with W from a 0.2 K noise-equivalent temperature at 250 K
    nu = np.asarray(ctl.nu)
    x = 1.43877506 * nu / 250.0
    sig = 0.2 * 1.19104259e-8 * nu ** 3 * x * np.exp(x) / (250.0 * np.expm1(x) ** 2)
    ws = [1.0 / sig for _ in K64]
    dys = [np.random.default_rng(7 + i).standard_normal(150) * sig for i in range(len(K64))]
    A32, b32 = ctx.normal_equations(K64, ws, dys, native.MIXED)
    A64, b64 = ctx.normal_equations(K64, ws, dys, native.FP64)
    for i in range(len(K64)):
        Aref = K64[i].T @ (ws[i][:, None] ** 2 * K64[i])
        assert np.max(np.abs(A64[i] - Aref)) <= 1e-10 * np.max(np.abs(Aref))
        assert np.max(np.abs(A32[i] - A64[i])) <= 1e-5 * np.max(np.abs(A64[i]))
        assert np.max(np.abs(b32[i] - b64[i])) <= 1e-5 * np.max(np.abs(b64[i]))
    ctx.close()
