"""Pin the CPU oracle (oracle/jrc_oracle.c) to the reference.

1. Known-answer test from the reference's own integration tests: the
   tangent-point columns of tests/{limb,nadir}_test/rad.org, printed with
   %g, must be reproduced exactly by the oracle's ray tracer.
2. Full-precision outputs of the reference build on small synthetic inputs
   (tests/golden/ref_*.npz): forward model (EGA, CGA, BT, surface,
   reflection, solar term, clouds, extinction, hydrostatic), Jacobian and
   retrieval.  On the machine that generated them the oracle agrees to the
   last bit; elsewhere libm may differ in the last bits, hence the 1e-12
   relative tolerance.
3. Where the reference build itself is present, a direct comparison on a
   fresh case.
"""
import copy

import numpy as np
import pytest

import golden_io as G
from jurassic_gb300.tables import Tables

RTOL = 1e-12


def _oracle(ctl, tables=None, filters=None):
    from oracle import oracle
    if tables is None:
        tables = Tables.empty(ctl.nd, ctl.ng, 32, 2, 2)
    if filters is None:
        filters = [(np.array([n - 0.5, n + 0.5]), np.array([1.0, 1.0])) for n in ctl.nu]
    return oracle.Oracle(ctl, tables, filters)


@pytest.mark.parametrize("name", ["limb_test", "nadir_test"])
def test_reference_tangent_points_kat(built_oracle, name):
    f = G.load("reftests.npz")
    ctl = G.ctl_from(f[name + "_ctl"])
    atm = G.atm_from(f, name + "_atm_", ctl)
    obs = G.obs_from(f, name + "_obs_", ctl.nd)
    expected = f[name + "_tp_str"]
    ora = _oracle(ctl)
    assert len(expected) == obs.nr
    for ir in range(obs.nr):
        _, tp = ora.raytrace(atm, obs, ir)
        got = ["%g" % v for v in tp]
        assert got == list(expected[ir]), "ray %d: %s != %s" % (ir, got, list(expected[ir]))


def _rel(a, b):
    fin = np.isfinite(b)
    assert np.array_equal(fin, np.isfinite(a))
    return np.max(np.abs(a[fin] - b[fin]) / np.maximum(np.abs(b[fin]), 1e-300))


@pytest.mark.parametrize("case", ["ega", "cga", "bbt"])
def test_formod_limb_vs_reference(built_oracle, case):
    f = G.load("ref_formod_limb.npz")
    ctl = G.ctl_from(f[case + "_ctl"])
    tbl = G.tables_from(f)
    atm = G.atm_from(f, "atm_", ctl)
    obs = G.obs_from(f, "obs_", ctl.nd)
    ora = _oracle(ctl, tbl, G.filters_from(f, ctl.nd))
    rad, tau, tp, _ = ora.formod(atm, obs)
    assert _rel(rad, f[case + "_rad"]) <= RTOL
    assert np.max(np.abs(tau - f[case + "_tau"])) <= 1e-14
    assert np.max(np.abs(tp - f[case + "_tp"])) <= 1e-9


def test_formod_nadir_surface_vs_reference(built_oracle):
    f = G.load("ref_formod_nadir.npz")
    ctl = G.ctl_from(f["ctl"])
    tbl = G.tables_from(f)
    atm = G.atm_from(f, "atm_", ctl)
    obs = G.obs_from(f, "obs_", ctl.nd)
    ora = _oracle(ctl, tbl, G.filters_from(f, ctl.nd))
    rad, tau, tp, p = ora.formod(atm, obs)
    assert np.isnan(rad[1, 1])                      # masked channel stays masked
    # With surface reflection the reference re-reads the segment emissivity
    # of every LOS point (jurassic.c:3292-3299), but never writes it at
    # points skipped because an emitter saturated (tau_gas == 0,
    # jurassic.c:3250): it reads stale heap memory there.  The oracle uses
    # zero for those points.  Channels whose path saturated (tau < 1e-8)
    # are therefore held to 1e-9 instead of rounding level.
    sat = tau < 1e-8
    fin = np.isfinite(f["rad"])
    rel = np.abs(rad - f["rad"]) / np.abs(f["rad"])
    assert np.all(rel[fin & ~sat] <= RTOL)
    assert np.all(rel[fin & sat] <= 1e-9)
    assert np.max(np.abs(tau - f["tau"])) <= 1e-14
    assert np.max(np.abs(p - f["p_after"]) / f["p_after"]) <= RTOL


def test_kernel_vs_reference(built_oracle):
    f = G.load("ref_kernel.npz")
    ctl = G.ctl_from(f["ctl"])
    ora = _oracle(ctl, G.tables_from(f), G.filters_from(f, ctl.nd))
    atm = G.atm_from(f, "atm_", ctl)
    obs = G.obs_from(f, "obs_", ctl.nd)
    K = ora.kernel(atm, obs)
    Kr = f["K"]
    assert K.shape == Kr.shape
    scale = np.max(np.abs(Kr), axis=0, keepdims=True)
    assert np.max(np.abs(K - Kr) / np.maximum(scale, 1e-300)) <= 1e-9


def test_retrieval_vs_reference(built_oracle):
    f = G.load("ref_retrieval.npz")
    ctl = G.ctl_from(f["ctl"])
    ret = G.ret_from(f["ret"])
    ora = _oracle(ctl, G.tables_from(f), G.filters_from(f, ctl.nd))
    apr = G.atm_from(f, "atm_", ctl)
    meas = G.obs_from(f, "obs_", ctl.nd)
    r = ora.retrieval(ret, apr, meas)
    assert r["n"] == len(f["x"])
    assert np.max(np.abs(r["x"] - f["x"]) / np.maximum(np.abs(f["x"]), 1e-300)) <= 1e-8
    # costs.tab is written with %g by the reference
    assert np.allclose(r["costs"], f["costs"], rtol=1e-5)
    assert np.max(np.abs(r["cov"] - f["cov"])) <= 1e-8 * np.max(np.abs(f["cov"]))
    # error analysis (retrieval.c:668-726): gain, averaging kernel, error
    # standard deviations and analyze_avk's contribution/resolution
    for k in ("gain", "avk", "err_total", "err_noise", "err_formod", "cont", "res"):
        assert r[k].shape == f[k].shape, k
        assert np.max(np.abs(r[k] - f[k])) <= 1e-8 * np.max(np.abs(f[k])), k


def test_oracle_direct_vs_reference_build(built_oracle):
    from oracle import refimpl
    if not refimpl.available("std"):
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    from jurassic_gb300 import synth
    w = synth.config_limb_ega(seed=21, n_rays=3)
    for formod in (0, 1):
        ctl = copy.deepcopy(w.ctl)
        ctl.formod = formod
        atm, obs = w.batch.item(ctl, 0)
        ora = _oracle(ctl, w.tables, w.filters)
        rad, tau, tp, _ = ora.formod(atm, obs)
        r = refimpl.run(ctl, w.tables, w.filters, [("formod", atm, obs, None)])[0]
        assert np.array_equal(rad, r["rad"]) and np.array_equal(tau, r["tau"])
        assert np.array_equal(tp, r["tp"])


@pytest.mark.parametrize("case", ["ega", "bbt"])
def test_formod_fov_vs_reference(built_oracle, case):
    """Field-of-view convolution (formod_fov, jurassic.c:3121-3192) after the
    pencil beams, before BT conversion and masking."""
    from oracle import oracle
    f = G.load("ref_formod_fov.npz")
    ctl = G.ctl_from(f[case + "_ctl"])
    ora = oracle.Oracle(ctl, G.tables_from(f), G.filters_from(f, ctl.nd),
                        fov=(f["fov_dz"], f["fov_w"]))
    atm = G.atm_from(f, "atm_", ctl)
    obs = G.obs_from(f, "obs_", ctl.nd)
    rad, tau, tp, _ = ora.formod(atm, obs)
    assert np.isnan(rad[2, 5]) and np.isnan(f[case + "_rad"][2, 5])
    fin = np.isfinite(rad)
    assert np.array_equal(fin, np.isfinite(f[case + "_rad"]))
    assert _rel(rad[fin], f[case + "_rad"][fin]) <= RTOL
    assert np.max(np.abs(tau - f[case + "_tau"])) <= 1e-14
    assert np.max(np.abs(tp - f[case + "_tp"])) <= 1e-9
