#!/usr/bin/env python3
"""Generate the golden fixtures under tests/golden/ (run in a container that
has the reference tree and oracle/_ref built).

reftests.npz  -- the reference's own integration-test inputs
                 (tests/limb_test, tests/nadir_test: control files, atm.tab,
                 obs.tab) and the tangent-point columns 8-10 of their
                 rad.org as the printed strings.  Those columns depend only on
                 raytrace()/tangent_point(), so they pin the ray tracer (the
                 emissivity tables behind the radiance columns are not in the
                 reference tree).
ref_*.npz     -- full-precision outputs of the reference build (oracle/_ref,
                 the unmodified reference sources) on small synthetic inputs,
                 stored together with those inputs: forward model (EGA, CGA,
                 BT, surface/reflection/solar, clouds, hydrostatic), Jacobian
                 and a retrieval.

usage: python tests/golden/make_golden.py [/path/to/reference]
"""
import copy
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from jurassic_gb300 import synth  # noqa: E402
from jurassic_gb300.model import Ctl, Ret, read_atm, read_ctl, read_obs  # noqa: E402
from oracle import refimpl  # noqa: E402


def ctl_json(ctl):
    d = {}
    for k, v in ctl.__dict__.items():
        d[k] = v.tolist() if isinstance(v, np.ndarray) else v
    return json.dumps(d)


def small_tables(ctl, seed):
    return synth.make_tables(ctl, seed, tp=32, tt=6, tu=64, umin=1e12, umax=1e26)


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote %s (%d bytes)" % (path, os.path.getsize(path)))


def atm_arrays(prefix, ctl, atm):
    return {prefix + "time": atm.time, prefix + "z": atm.z, prefix + "lon": atm.lon,
            prefix + "lat": atm.lat, prefix + "p": atm.p, prefix + "t": atm.t,
            prefix + "q": atm.q, prefix + "k": atm.k, prefix + "scal": atm.scal(ctl)}


def obs_arrays(prefix, obs):
    return {prefix + "geo": obs.geo(), prefix + "rad": obs.rad}


def table_arrays(tbl, filters):
    d = {"tbl_np": tbl.np_, "tbl_p": tbl.p, "tbl_nt": tbl.nt, "tbl_t": tbl.t,
         "tbl_nu": tbl.nu, "tbl_u": tbl.u, "tbl_eps": tbl.eps}
    for i, (fnu, f) in enumerate(filters):
        d["filt%d_nu" % i] = fnu
        d["filt%d_f" % i] = f
    return d


def reftests(ref):
    out = {}
    for name, ctlname in (("limb_test", "limb.ctl"), ("nadir_test", "nadir.ctl")):
        d = os.path.join(ref, "tests", name)
        ctl = read_ctl(["x", os.path.join(d, ctlname)])
        atm = read_atm(d, "atm.tab", ctl)
        obs = read_obs(d, "obs.tab", ctl)
        tps = []
        with open(os.path.join(d, "rad.org")) as f:
            for line in f:
                tok = line.split()
                if len(tok) >= 10 and not line.startswith("#"):
                    tps.append(tok[7:10])
        out[name + "_ctl"] = ctl_json(ctl)
        out.update(atm_arrays(name + "_atm_", ctl, atm))
        out.update(obs_arrays(name + "_obs_", obs))
        out[name + "_tp_str"] = np.array(tps)
    save("reftests.npz", **out)


def formod_cases():
    # limb: 5 rays, 3 channels, CO2+H2O, EGA / CGA / BT
    w = synth.config_limb_ega(n_rays=5)
    tbl = small_tables(w.ctl, 11)
    atm, obs = w.batch.item(w.ctl, 0)
    res = {}
    for label, mod in (("ega", {}), ("cga", {"formod": 0}), ("bbt", {"write_bbt": 1})):
        ctl = copy.deepcopy(w.ctl)
        for k, v in mod.items():
            setattr(ctl, k, v)
        r = refimpl.run(ctl, tbl, w.filters, [("formod", atm, obs, None)])[0]
        res.update({label + "_ctl": ctl_json(ctl), label + "_rad": r["rad"],
                    label + "_tau": r["tau"], label + "_tp": r["tp"]})
    save("ref_formod_limb.npz", **res, **table_arrays(tbl, w.filters),
         **atm_arrays("atm_", w.ctl, atm), **obs_arrays("obs_", obs))

    # nadir with surface emissivity/reflection/solar, clouds, extinction,
    # hydrostatic pressure
    w = synth.config_nadir(1, nd=3, nlev=61, ztop=60.0, numin=700.0, numax=2300.0,
                           emitters=("CO2", "H2O"))
    ctl = copy.deepcopy(w.ctl)
    ctl.sfnu = np.array([600.0, 1500.0, 2500.0])
    ctl.sftype = 3
    ctl.clnu = np.array([600.0, 2500.0])
    ctl.hydz = 5.0
    tbl = small_tables(ctl, 12)
    atm, obs = w.batch.item(w.ctl, 0)
    atm.sfz, atm.sfp, atm.sft = 0.0, 0.0, 291.0
    atm.sfeps = np.array([0.97, 0.85, 0.9])
    atm.clz, atm.cldz = 9.0, 1.5
    atm.clk = np.array([2e-3, 1e-3])
    atm.k[0] = 2e-4 * np.exp(-atm.z / 8.0)
    obs = synth.nadir_obs(ctl.nd, [10.0, 20.0, 30.0], obsz=705.0, time=86400.0 * 120.5,
                          scan_deg=[0.0, 2.0, -3.0])
    obs.rad[1, 1] = np.nan
    r = refimpl.run(ctl, tbl, w.filters, [("formod", atm, obs, None)])[0]
    save("ref_formod_nadir.npz", ctl=ctl_json(ctl), rad=r["rad"], tau=r["tau"], tp=r["tp"],
         p_after=r["p"], **table_arrays(tbl, w.filters), **atm_arrays("atm_", ctl, atm),
         **obs_arrays("obs_", obs))


def fov_shape():
    dz = np.linspace(-2.0, 2.0, 21)
    return dz, np.exp(-dz ** 2)


def fov_case():
    """Limb with field-of-view convolution (formod_fov, jurassic.c:3121-3192):
    8 rays at 10-31 km, a masked channel, radiance and BT output."""
    w = synth.config_limb_ega(n_rays=8)
    tbl = small_tables(w.ctl, 15)
    atm, obs = w.batch.item(w.ctl, 0)
    obs.rad[2, 5] = np.nan
    res = {}
    for label, mod in (("ega", {}), ("bbt", {"write_bbt": 1})):
        ctl = copy.deepcopy(w.ctl)
        for k, v in mod.items():
            setattr(ctl, k, v)
        r = refimpl.run(ctl, tbl, w.filters, [("formod", atm, obs, None)], fov=fov_shape())[0]
        res.update({label + "_ctl": ctl_json(ctl), label + "_rad": r["rad"],
                    label + "_tau": r["tau"], label + "_tp": r["tp"]})
    dz, wf = fov_shape()
    save("ref_formod_fov.npz", fov_dz=dz, fov_w=wf, **res, **table_arrays(tbl, w.filters),
         **atm_arrays("atm_", w.ctl, atm), **obs_arrays("obs_", obs))


def tbl_ascii_case():
    """ASCII tables (read_tbl TBLFMT=1) with lines the reader must skip (out
    of range, text) or fold (a point that does not increase u and eps
    overwrites the previous one): the reference's forward model with these
    files, and the files themselves."""
    w = synth.config_limb_ega(n_rays=4)
    ctl = copy.deepcopy(w.ctl)
    ctl.tblfmt = 1
    tbl = small_tables(ctl, 16)
    atm, obs = w.batch.item(w.ctl, 0)
    texts = {}

    def mangle(workdir):
        c2 = copy.copy(ctl)
        c2.tblbase = os.path.join(workdir, "tbl")
        for id in range(ctl.nd):
            for ig in range(ctl.ng):
                fn = c2.table_filename(id, ig)
                lines = open(fn).read().splitlines()
                out = []
                for k, line in enumerate(lines):
                    out.append(line)
                    parts = line.split()
                    if len(parts) != 4:
                        continue
                    p, t, u, e = parts
                    if k % 97 == 5:
                        out.append("%s %s %s %s" % (p, t, u, "1.5"))         # eps > EPSMAX
                        out.append("%s %s %s %s" % (p, t, "-1", e))          # u < UMIN
                        out.append("this line is not data")
                    if k % 89 == 7:
                        # u and eps not above the last point: it overwrites that point
                        out.append("%s %s %.9e %.9e" % (p, t, 0.9995 * float(u), 0.9995 * float(e)))
                txt = "\n".join(out) + "\n"
                open(fn, "w").write(txt)
                texts["tbl_%d_%d" % (id, ig)] = np.frombuffer(txt.encode(), dtype=np.uint8)

    r = refimpl.run(ctl, tbl, w.filters, [("formod", atm, obs, None)], post_write=mangle)[0]
    save("ref_tbl_ascii.npz", ctl=ctl_json(ctl), rad=r["rad"], tau=r["tau"], **texts,
         **table_arrays(tbl, w.filters), **atm_arrays("atm_", ctl, atm),
         **obs_arrays("obs_", obs))


def kernel_case():
    ctl = Ctl(emitter=["CO2", "H2O"], nu=[667.78, 792.0], formod=1)
    z = np.arange(0.0, 82.0, 2.0)
    ctl.rett_zmin, ctl.rett_zmax = 8.0, 50.0
    ctl.retq_zmin = np.array([10.0, 8.0])
    ctl.retq_zmax = np.array([40.0, 30.0])
    ctl.retp_zmin, ctl.retp_zmax = 20.0, 26.0
    ctl.retk_zmin, ctl.retk_zmax = np.array([12.0]), np.array([16.0])
    rng = np.random.default_rng(5)
    atm = synth.profile(ctl.emitter, z, rng=rng, noise=0.01)
    obs = synth.limb_obs(ctl.nd, [12.0, 18.0, 25.0])
    tbl = small_tables(ctl, 13)
    filters = synth.make_filters(ctl)
    K = refimpl.run(ctl, tbl, filters, [("kernel", atm, obs, {"maxm": 64, "maxn": 256})])[0]
    save("ref_kernel.npz", ctl=ctl_json(ctl), K=K, **table_arrays(tbl, filters),
         **atm_arrays("atm_", ctl, atm), **obs_arrays("obs_", obs))


def retrieval_case():
    ctl = Ctl(emitter=["CO2", "H2O"], nu=[667.78, 700.0, 792.0, 1000.0], formod=1)
    z = np.arange(0.0, 62.0, 2.0)
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 40.0
    ctl.retq_zmin = np.array([-999.0, 0.0])
    ctl.retq_zmax = np.array([-999.0, 14.0])
    rng = np.random.default_rng(6)
    truth = synth.profile(ctl.emitter, z, rng=rng, noise=0.01)
    apr = synth.profile(ctl.emitter, z)
    obs = synth.nadir_obs(ctl.nd, [0.0, 1.0], obsz=705.0, scan_deg=[0.0, 1.0])
    tbl = small_tables(ctl, 14)
    filters = synth.make_filters(ctl)
    meas = refimpl.run(ctl, tbl, filters, [("formod", truth, obs, None)])[0]
    obs_meas = obs.copy()
    obs_meas.rad = meas["rad"] * (1 + 1e-3 * rng.standard_normal(meas["rad"].shape))
    ret = Ret(kernel_recomp=1, conv_itmax=4, conv_dmin=0.1, err_ana=1,
              err_noise=np.full(ctl.nd, 2e-4), err_formod=np.full(ctl.nd, 1.0),
              err_temp=2.0, err_temp_cz=3.0, err_temp_ch=500.0,
              err_q=np.array([0.0, 30.0]), err_q_cz=np.array([-999.0, 3.0]),
              err_q_ch=np.array([-999.0, 500.0]))
    r = refimpl.run(ctl, tbl, filters, [("retrieval", apr, obs_meas, {"maxn": 256})],
                    ret=ret)[0]
    rj = {k: (v.tolist() if isinstance(v, np.ndarray) else v) for k, v in ret.sized(ctl).__dict__.items()}
    ana = {k: r[k] for k in ("gain", "avk", "err_total", "err_noise", "err_formod", "cont",
                             "res")}
    save("ref_retrieval.npz", ctl=ctl_json(ctl), ret=json.dumps(rj), x=r["x"], cov=r["cov"],
         costs=r["costs"], **ana, **table_arrays(tbl, filters), **atm_arrays("atm_", ctl, apr),
         **obs_arrays("obs_", obs_meas))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else refimpl.source_dir()
    if not ref:
        raise SystemExit("usage: make_golden.py <reference tree> (or set JURASSIC_REF_DIR)")
    if not refimpl.available("std"):
        refimpl.build("std")
    reftests(ref)
    formod_cases()
    kernel_case()
    retrieval_case()
    fov_case()
    tbl_ascii_case()


if __name__ == "__main__":
    main()
