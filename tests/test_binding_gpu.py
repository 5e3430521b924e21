"""The reference-side binding (jurassic_gb300/binding/jurassic_unified_library.c)
run on the GPU with reference-layout structs.

The binding is what a maintainer compiles into the reference's build with
UNIFIED=1 (formod.c:26-27, 60-76): jur_unified_init / init_ctl,
jur_unified_formod_multiple_packages (all packages in ONE batched library
call), and drop-ins for kernel() (jurassic.c:4004-4099, the caller's
gsl_matrix with its tda) and optimal_estimation (retrieval.c:448-749).
Here it is compiled with gcc against tests/refabi/jurassic.h (the
reference's struct layouts restated; tests/test_abi.py checks them against
the reference's own header) and driven through tests/refabi/driver.c:
packages are filled as atm_t / obs_t, the library reads the table and
filter files the test writes (read_tbl's names), and the results read back
out of the structs are compared with the CPU oracle and the reference's own
golden retrieval.
"""
import copy
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

import golden_io as G
from jurassic_gb300 import native, synth
from jurassic_gb300.model import brightness
from jurassic_gb300.tables import write_filters, write_tbl

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIMS = dict(ND=16, NG=4, NW=2, NP=128, NR=16, NCL=8, NSF=8, LEN=4096)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def _c_str(s):
    return '"' + s.replace("\\", "\\\\").replace('"', '\\"') + '"'


def _fill_source(ctl):
    """C source of drv_fill_ctl: the control set as ctl_t assignments."""
    L = ["#include \"jurassic.h\"", "void drv_fill_ctl(ctl_t *c) {"]
    L.append("  c->ng = %d; c->nd = %d; c->nw = %d; c->ncl = %d; c->nsf = %d;"
             % (ctl.ng, ctl.nd, ctl.nw, ctl.ncl, ctl.nsf))
    for ig, e in enumerate(ctl.emitter):
        L.append("  strcpy(c->emitter[%d], %s);" % (ig, _c_str(e)))
    for id_ in range(ctl.nd):
        L.append("  c->nu[%d] = %.17g; c->window[%d] = %d;" % (id_, ctl.nu[id_], id_,
                                                             int(ctl.window[id_])))
    for i, v in enumerate(ctl.clnu):
        L.append("  c->clnu[%d] = %.17g;" % (i, v))
    for i, v in enumerate(ctl.sfnu):
        L.append("  c->sfnu[%d] = %.17g;" % (i, v))
    for k in ("sftype", "tblfmt", "ctm_co2", "ctm_h2o", "ctm_n2", "ctm_o2", "refrac", "ret_clz",
              "ret_cldz", "ret_clk", "ret_sfz", "ret_sfp", "ret_sft", "ret_sfeps", "write_bbt",
              "write_matrix", "formod"):
        L.append("  c->%s = %d;" % (k, int(getattr(ctl, k))))
    for k in ("sfsza", "hydz", "rayds", "raydz", "retp_zmin", "retp_zmax", "rett_zmin",
              "rett_zmax"):
        L.append("  c->%s = %.17g;" % (k, float(getattr(ctl, k))))
    for k, n in (("retq_zmin", ctl.ng), ("retq_zmax", ctl.ng), ("retk_zmin", ctl.nw),
                 ("retk_zmax", ctl.nw)):
        for i in range(n):
            L.append("  c->%s[%d] = %.17g;" % (k, i, float(getattr(ctl, k)[i])))
    L.append("  strcpy(c->tblbase, %s);" % _c_str(ctl.tblbase))
    L.append("  strcpy(c->fov, %s);" % _c_str(ctl.fov))
    L.append("}")
    return "\n".join(L) + "\n"


class Binding:
    """The binding + test driver compiled for one control set."""

    def __init__(self, tmp_path, ctl, tables, filters):
        cc = shutil.which("gcc") or shutil.which("cc")
        assert cc, "a C compiler is needed to build the binding"
        self.ctl = copy.deepcopy(ctl)
        self.ctl.tblbase = str(tmp_path / "tbl")
        self.ctl.tblfmt = 2
        write_tbl(self.ctl, tables)
        write_filters(self.ctl, filters)
        fill = tmp_path / "fill.c"
        fill.write_text(_fill_source(self.ctl))
        lib = tmp_path / "libjgb_refbind.so"
        libdir = os.path.dirname(native.LIB_PATH)
        cmd = [cc, "-std=gnu99", "-O1", "-fPIC", "-shared", "-Wall", "-Werror"]
        cmd += ["-D%s=%d" % kv for kv in DIMS.items()]
        cmd += ["-I", os.path.join(ROOT, "tests", "refabi"),
                "-isystem", os.path.join(ROOT, "oracle", "gsl_shim"),
                "-I", os.path.join(ROOT, "include"),
                "-I", os.path.join(ROOT, "jurassic_gb300", "binding"),
                os.path.join(ROOT, "tests", "refabi", "driver.c"),
                os.path.join(ROOT, "jurassic_gb300", "binding", "jurassic_unified_library.c"),
                str(fill), "-o", str(lib), "-L", libdir, "-ljurassic_gb300",
                "-Wl,-rpath," + libdir, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        native.load()            # the library first, so that the driver finds it loaded
        self.L = C.CDLL(str(lib))
        L = self.L
        L.drv_init.argtypes = [C.c_int, C.c_int, C.c_int]
        L.drv_set_atm.argtypes = [C.c_int, C.c_int] + [_dp] * 9
        L.drv_set_obs.argtypes = [C.c_int, C.c_int, _dp, _dp]
        L.drv_get.argtypes = [C.c_int, C.c_int] + [_dp] * 6
        L.drv_formod.argtypes = [C.c_int]
        L.drv_kernel.argtypes = [C.c_int, _ip, _ip, C.c_int, _dp]
        L.drv_retrieve.argtypes = [C.c_void_p, C.c_int, _ip, _dp]

    def init(self, npack, precision):
        assert self.L.drv_init(npack, 0, precision) == 0

    def set_packages(self, batch):
        ctl = self.ctl
        for i in range(batch.nobs):
            atm, obs = batch.item(ctl, i)
            a = [np.ascontiguousarray(v, dtype=np.float64) for v in
                 (atm.time, atm.z, atm.lon, atm.lat, atm.p, atm.t,
                  np.reshape(atm.q, (ctl.ng, -1)), np.reshape(atm.k, (ctl.nw, -1)) if ctl.nw
                  else np.zeros(1), atm.scal(ctl))]
            self.L.drv_set_atm(i, len(atm.z), *[v.ctypes.data_as(_dp) for v in a])
            geo = np.ascontiguousarray(obs.geo(), dtype=np.float64)
            rad = np.ascontiguousarray(obs.rad, dtype=np.float64)
            self.L.drv_set_obs(i, obs.nr, geo.ctypes.data_as(_dp), rad.ctypes.data_as(_dp))

    def get(self, which, i, nr, npl):
        ctl = self.ctl
        out = dict(rad=np.zeros((ctl.nd, nr)), tau=np.zeros((ctl.nd, nr)), tp=np.zeros((3, nr)),
                   p=np.zeros(npl), t=np.zeros(npl), q=np.zeros((ctl.ng, npl)))
        self.L.drv_get(which, i, *[out[k].ctypes.data_as(_dp)
                                   for k in ("rad", "tau", "tp", "p", "t", "q")])
        return out

    def close(self):
        self.L.drv_finalize()


def _nadir(nobs, hydz=-999.0):
    w = synth.config_nadir(nobs, nd=6, nlev=51, ztop=50.0, emitters=("CO2", "H2O", "O3"),
                           numin=660.0, numax=1600.0)
    w.ctl.hydz = hydz
    return w


@pytest.mark.parametrize("hydz", [-999.0, 0.0])
def test_formod_multiple_packages(built_lib, built_oracle, tmp_path, hydz):
    """n packages through one jur_unified_formod_multiple_packages call:
    FP64 within 1e-9 of the oracle and bit-identical to jgb_formod_batch;
    mixed within 10 mK; masked channels stay NaN; hydrostatic pressures come
    back in atm.p."""
    from oracle import oracle
    w = _nadir(5, hydz)
    b = w.batch.fresh_outputs()
    b.rad[1, 2] = np.nan
    ora = oracle.Oracle(w.ctl, w.tables, w.filters)
    ref = ora.formod_batch(b)
    ctx = native.Context(w.ctl, w.tables, w.filters)
    direct = ctx.formod_batch(b.copy(), native.FP64)
    ctx.close()
    B = Binding(tmp_path, w.ctl, w.tables, w.filters)
    nu = np.asarray(w.ctl.nu)[:, None]
    for prec in (native.FP64, native.MIXED):
        B.init(b.nobs, prec)
        B.set_packages(b)
        B.L.drv_formod(b.nobs)
        for i in range(b.nobs):
            r0, r1 = b.ray_off[i], b.ray_off[i + 1]
            l0, l1 = b.lev_off[i], b.lev_off[i + 1]
            o = B.get(0, i, r1 - r0, l1 - l0)
            rr = ref.rad[:, r0:r1]
            fin = np.isfinite(rr)
            assert np.array_equal(fin, np.isfinite(o["rad"])), i
            if prec == native.FP64:
                assert np.max(np.abs(o["rad"][fin] - rr[fin]) / np.abs(rr[fin])) <= 1e-9
                assert np.array_equal(o["rad"], direct.rad[:, r0:r1], equal_nan=True)
                assert np.array_equal(o["tp"], direct.tp[:, r0:r1])
                assert np.max(np.abs(o["p"] - ref.p[l0:l1]) / ref.p[l0:l1]) <= 1e-9
            else:
                dbt = np.abs(brightness(o["rad"], nu) - brightness(rr, nu))[fin]
                assert np.max(dbt) <= 0.010, i
        if hydz >= 0:
            assert np.max(np.abs(ref.p - b.p) / b.p) > 1e-6   # pressures did change
    B.close()
    ora.close()


def test_kernel_dropin(built_lib, built_oracle, tmp_path):
    """kernel() drop-in: K written into the caller's gsl_matrix row by row
    with its tda (rows padded here), single package and three at once,
    FP64 within 1e-7 of each column's largest entry of the oracle's
    kernel(); obs gets the unperturbed forward model."""
    from oracle import oracle
    w = _nadir(3)
    ctl = w.ctl
    ctl.rett_zmin, ctl.rett_zmax = 0.0, 40.0
    ctl.retq_zmin = np.array([-999.0, 0.0, 15.0])
    ctl.retq_zmax = np.array([-999.0, 12.0, 35.0])
    b = w.batch.fresh_outputs()
    b.rad[4, 0] = np.nan
    ora = oracle.Oracle(ctl, w.tables, w.filters)
    ctx = native.Context(ctl, w.tables, w.filters)
    m, n = ctx.kernel_sizes(b)
    ctx.close()
    Kref = [ora.kernel(*b.item(ctl, i)) for i in range(b.nobs)]
    fm = ora.formod_batch(b)
    B = Binding(tmp_path, ctl, w.tables, w.filters)
    B.init(b.nobs, native.FP64)
    for npk in (1, 3):
        B.set_packages(b)
        mi = np.ascontiguousarray(m[:npk], np.int32)
        ni = np.ascontiguousarray(n[:npk], np.int32)
        kout = np.zeros(int(np.sum(mi.astype(np.int64) * ni)))
        B.L.drv_kernel(npk, mi.ctypes.data_as(_ip), ni.ctypes.data_as(_ip), 3,
                       kout.ctypes.data_as(_dp))
        off = 0
        for i in range(npk):
            K = kout[off:off + m[i] * n[i]].reshape(m[i], n[i])
            off += m[i] * n[i]
            assert K.shape == Kref[i].shape
            scale = np.maximum(np.max(np.abs(Kref[i]), axis=0, keepdims=True), 1e-300)
            assert np.max(np.abs(K - Kref[i]) / scale) <= 1e-7, (npk, i)
            r0, r1 = b.ray_off[i], b.ray_off[i + 1]
            o = B.get(0, i, r1 - r0, b.lev_off[i + 1] - b.lev_off[i])
            fin = np.isfinite(fm.rad[:, r0:r1])
            assert np.max(np.abs(o["rad"][fin] - fm.rad[:, r0:r1][fin])
                          / np.abs(fm.rad[:, r0:r1][fin])) <= 1e-9
    B.close()
    ora.close()


def test_optimal_estimation_dropin(built_lib, built_oracle, tmp_path):
    """optimal_estimation drop-in on the reference's own golden retrieval
    (FP64): atm_i gets x2atm of the final state (the reference's x within
    1e-6), cov its covariance (within 1e-6 of the largest entry); three
    packages at once give each package the single call's results."""
    f = G.load("ref_retrieval.npz")
    ctl = G.ctl_from(f["ctl"])
    ret = G.ret_from(f["ret"])
    tbl, filt = G.tables_from(f), G.filters_from(f, ctl.nd)
    apr = G.atm_from(f, "atm_", ctl)
    meas = G.obs_from(f, "obs_", ctl.nd)
    ctx = native.Context(ctl, tbl, filt)
    _, sr, keep = ctx._ret_struct(ret)
    B = Binding(tmp_path, ctl, tbl, filt)
    B.init(3, native.FP64)
    one = synth.pack(ctl, [(apr, meas)])
    npx = len(f["x"])
    ni = np.array([npx], np.int32)
    cov = np.zeros(npx * npx)
    B.set_packages(one)
    B.L.drv_retrieve(C.addressof(sr), 1, ni.ctypes.data_as(_ip), cov.ctypes.data_as(_dp))
    nr, npl = meas.nr, len(apr.z)
    res = B.get(1, 0, nr, npl)
    # the final state from the result atmosphere (atm2x with the context's windows)
    x = np.zeros(npx)
    nx = C.c_int(0)
    L = native.load()
    qa = np.ascontiguousarray(res["q"])
    assert L.jgb_atm2x(ctx.h, npl, apr.z.ctypes.data_as(_dp), res["p"].ctypes.data_as(_dp),
                       res["t"].ctypes.data_as(_dp), qa.ctypes.data_as(_dp), None, None,
                       x.ctypes.data_as(_dp), C.byref(nx)) == 0
    assert nx.value == npx
    assert np.max(np.abs(x - f["x"]) / np.maximum(np.abs(f["x"]), 1e-300)) <= 1e-6
    assert np.max(np.abs(cov - f["cov"].ravel())) <= 1e-6 * np.max(np.abs(f["cov"]))
    # three packages (the golden one three times) in one call
    three = synth.pack(ctl, [(apr, meas)] * 3)
    B.set_packages(three)
    ni3 = np.full(3, npx, np.int32)
    cov3 = np.zeros(3 * npx * npx)
    B.L.drv_retrieve(C.addressof(sr), 3, ni3.ctypes.data_as(_ip), cov3.ctypes.data_as(_dp))
    for i in range(3):
        r = B.get(1, i, nr, npl)
        for k in ("p", "t", "q", "rad", "tau", "tp"):
            assert np.array_equal(r[k], res[k], equal_nan=True), (i, k)
        assert np.array_equal(cov3[i * npx * npx:(i + 1) * npx * npx], cov)
    del keep
    B.close()
    ctx.close()
