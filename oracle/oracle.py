"""ctypes binding to the CPU restatement (oracle/jrc_oracle.c).

TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the
benchmark's CPU-baseline leg as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libjrc_oracle.so")
CONTINUA = os.path.join(os.path.dirname(HERE), "jurassic_gb300", "data", "continua.bin")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


def build(force=False):
    """Compile the restatement (plain C, OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "jrc_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "jrc_oracle.h"))):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + ".%d.tmp" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
                           "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class _Ctl(C.Structure):
    _fields_ = [("ng", C.c_int), ("nd", C.c_int), ("nw", C.c_int), ("ncl", C.c_int),
                ("nsf", C.c_int), ("emitter_kind", _ip), ("nu", _dp), ("window", _ip),
                ("clnu", _dp), ("sfnu", _dp), ("sftype", C.c_int), ("sfsza", C.c_double),
                ("hydz", C.c_double), ("ctm_co2", C.c_int), ("ctm_h2o", C.c_int),
                ("ctm_n2", C.c_int), ("ctm_o2", C.c_int), ("refrac", C.c_int),
                ("rayds", C.c_double), ("raydz", C.c_double), ("formod", C.c_int),
                ("write_bbt", C.c_int), ("retp_zmin", C.c_double), ("retp_zmax", C.c_double),
                ("rett_zmin", C.c_double), ("rett_zmax", C.c_double), ("retq_zmin", _dp),
                ("retq_zmax", _dp), ("retk_zmin", _dp), ("retk_zmax", _dp),
                ("ret_clz", C.c_int), ("ret_cldz", C.c_int), ("ret_clk", C.c_int),
                ("ret_sfz", C.c_int), ("ret_sfp", C.c_int), ("ret_sft", C.c_int),
                ("ret_sfeps", C.c_int), ("nlos_max", C.c_int)]


class _Atm(C.Structure):
    _fields_ = [("np", C.c_int), ("time", _dp), ("z", _dp), ("lon", _dp), ("lat", _dp),
                ("p", _dp), ("t", _dp), ("q", _dp), ("k", _dp), ("scal", _dp)]


class _Obs(C.Structure):
    _fields_ = [("nr", C.c_int), ("geo", _dp), ("rad", _dp), ("tau", _dp), ("tp", _dp)]


class _Ret(C.Structure):
    _fields_ = [("kernel_recomp", C.c_int), ("conv_itmax", C.c_int), ("err_ana", C.c_int),
                ("conv_dmin", C.c_double), ("err_formod", _dp), ("err_noise", _dp),
                ("err_press", C.c_double), ("err_press_cz", C.c_double),
                ("err_press_ch", C.c_double), ("err_temp", C.c_double),
                ("err_temp_cz", C.c_double), ("err_temp_ch", C.c_double),
                ("err_q", _dp), ("err_q_cz", _dp), ("err_q_ch", _dp), ("err_k", _dp),
                ("err_k_cz", _dp), ("err_k_ch", _dp), ("err_clz", C.c_double),
                ("err_cldz", C.c_double), ("err_clk", _dp), ("err_sfz", C.c_double),
                ("err_sfp", C.c_double), ("err_sft", C.c_double), ("err_sfeps", _dp)]


class _Ana(C.Structure):
    _fields_ = [(k, _dp) for k in ("gain", "avk", "err_total", "err_noise", "err_formod", "cont",
                                   "res")]


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t)


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.jrc_create.restype = C.c_void_p
        L.jrc_create.argtypes = [C.POINTER(_Ctl), C.c_int, C.c_int, C.c_int]
        L.jrc_destroy.argtypes = [C.c_void_p]
        L.jrc_error.restype = C.c_char_p
        L.jrc_error.argtypes = [C.c_void_p]
        L.jrc_set_table.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _ip, _dp,
                                    _ip, _fp, _fp]
        L.jrc_init_srcfunc.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp, _dp]
        L.jrc_get_srcfunc.argtypes = [C.c_void_p, _dp, _dp]
        L.jrc_set_continua.argtypes = [C.c_void_p, _dp, C.c_long]
        L.jrc_formod.argtypes = [C.c_void_p, C.POINTER(_Atm), C.POINTER(_Obs)]
        L.jrc_formod_batch.argtypes = [C.c_void_p, C.c_int, _ip, _dp, _dp, _dp, _dp, _dp,
                                       _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp, _dp, C.c_int]
        L.jrc_raytrace.argtypes = [C.c_void_p, C.POINTER(_Atm), C.POINTER(_Obs), C.c_int,
                                   C.c_int, _dp]
        L.jrc_sizes.argtypes = [C.c_void_p, C.POINTER(_Atm), C.POINTER(_Obs), _ip, _ip]
        L.jrc_atm2x.argtypes = [C.c_void_p, C.POINTER(_Atm), _dp, _ip, _ip]
        L.jrc_kernel.argtypes = [C.c_void_p, C.POINTER(_Atm), C.POINTER(_Obs), _dp, C.c_int]
        L.jrc_retrieval.argtypes = [C.c_void_p, C.POINTER(_Ret), C.POINTER(_Atm),
                                    C.POINTER(_Obs), _dp, _dp, _dp, _dp, C.c_int, _ip, C.c_int]
        L.jrc_set_fov.argtypes = [C.c_void_p, C.c_int, _dp, _dp]
        L.jrc_retrieval_ex.argtypes = [C.c_void_p, C.POINTER(_Ret), C.POINTER(_Atm),
                                       C.POINTER(_Obs), _dp, _dp, _dp, _dp, C.c_int, _ip, C.c_int,
                                       C.POINTER(_Ana)]
        L.jrc_matrix_invert.argtypes = [_dp, C.c_int]
        _lib = L
    return _lib


def matrix_invert(a):
    """matrix_invert (retrieval.c:373-399) of one square matrix: returns
    (inverse, ok); ok is False where the matrix is not positive definite."""
    a = np.array(a, dtype=np.float64, order="C")
    rc = lib().jrc_matrix_invert(_ptr(a), a.shape[0])
    return a, rc == 0


def continua_blob():
    return np.fromfile(CONTINUA, dtype="<f8")


class Oracle:
    """One CPU-oracle context: a control set, its tables and source functions."""

    def __init__(self, ctl, tables, filters, nlos_max=4096, fov=None):
        L = lib()
        self.ctl = ctl
        self._keep = []
        kinds = ctl.emitter_kinds()
        arrs = dict(kind=np.ascontiguousarray(kinds, np.int32), nu=_d(ctl.nu),
                    window=np.ascontiguousarray(ctl.window, np.int32), clnu=_d(ctl.clnu),
                    sfnu=_d(ctl.sfnu), rqn=_d(ctl.retq_zmin), rqx=_d(ctl.retq_zmax),
                    rkn=_d(ctl.retk_zmin), rkx=_d(ctl.retk_zmax))
        self._keep.append(arrs)
        c = _Ctl(ng=ctl.ng, nd=ctl.nd, nw=ctl.nw, ncl=ctl.ncl, nsf=ctl.nsf,
                 emitter_kind=_ptr(arrs["kind"], _ip), nu=_ptr(arrs["nu"]),
                 window=_ptr(arrs["window"], _ip), clnu=_ptr(arrs["clnu"]),
                 sfnu=_ptr(arrs["sfnu"]), sftype=ctl.sftype, sfsza=ctl.sfsza, hydz=ctl.hydz,
                 ctm_co2=ctl.ctm_co2, ctm_h2o=ctl.ctm_h2o, ctm_n2=ctl.ctm_n2,
                 ctm_o2=ctl.ctm_o2, refrac=ctl.refrac, rayds=ctl.rayds, raydz=ctl.raydz,
                 formod=ctl.formod, write_bbt=ctl.write_bbt, retp_zmin=ctl.retp_zmin,
                 retp_zmax=ctl.retp_zmax, rett_zmin=ctl.rett_zmin, rett_zmax=ctl.rett_zmax,
                 retq_zmin=_ptr(arrs["rqn"]), retq_zmax=_ptr(arrs["rqx"]),
                 retk_zmin=_ptr(arrs["rkn"]), retk_zmax=_ptr(arrs["rkx"]),
                 ret_clz=ctl.ret_clz, ret_cldz=ctl.ret_cldz, ret_clk=ctl.ret_clk,
                 ret_sfz=ctl.ret_sfz, ret_sfp=ctl.ret_sfp, ret_sft=ctl.ret_sft,
                 ret_sfeps=ctl.ret_sfeps, nlos_max=nlos_max)
        tp, tt, tu = tables.u.shape[2:]
        self.h = L.jrc_create(C.byref(c), tp, tt, tu)
        if fov is not None:
            dz, w = _d(fov[0]), _d(fov[1])
            self._keep.append((dz, w))
            self._check(L.jrc_set_fov(self.h, len(dz), _ptr(dz), _ptr(w)))
        blob = continua_blob()
        self._check(L.jrc_set_continua(self.h, _ptr(blob), len(blob)))
        for id in range(ctl.nd):
            for ig in range(ctl.ng):
                n = int(tables.np_[id, ig])
                if n < 0:
                    continue
                p = _d(tables.p[id, ig])
                nt = np.ascontiguousarray(tables.nt[id, ig], np.int32)
                t = _d(tables.t[id, ig])
                nu = np.ascontiguousarray(tables.nu[id, ig], np.int32)
                u = np.ascontiguousarray(tables.u[id, ig], np.float32)
                e = np.ascontiguousarray(tables.eps[id, ig], np.float32)
                self._check(L.jrc_set_table(self.h, id, ig, n, _ptr(p), _ptr(nt, _ip),
                                            _ptr(t), _ptr(nu, _ip), _ptr(u, _fp), _ptr(e, _fp)))
        for id, (fnu, f) in enumerate(filters):
            fnu, f = _d(fnu), _d(f)
            self._check(L.jrc_init_srcfunc(self.h, id, len(fnu), _ptr(fnu), _ptr(f)))

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: %s" % lib().jrc_error(self.h).decode())

    def close(self):
        if self.h:
            lib().jrc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def srcfunc(self):
        st = np.zeros(1200)
        sr = np.zeros((1200, self.ctl.nd))
        lib().jrc_get_srcfunc(self.h, _ptr(st), _ptr(sr))
        return st, sr

    # ---------------------------------------------------------------
    def _atm(self, atm):
        ctl = self.ctl
        a = dict(time=_d(atm.time), z=_d(atm.z), lon=_d(atm.lon), lat=_d(atm.lat),
                 p=_d(atm.p).copy(), t=_d(atm.t).copy(),
                 q=_d(np.asarray(atm.q).reshape(ctl.ng, atm.np)).copy(),
                 k=_d(np.asarray(atm.k).reshape(ctl.nw, atm.np)).copy(),
                 scal=_d(atm.scal(ctl)).copy())
        s = _Atm(np=atm.np, time=_ptr(a["time"]), z=_ptr(a["z"]), lon=_ptr(a["lon"]),
                 lat=_ptr(a["lat"]), p=_ptr(a["p"]), t=_ptr(a["t"]), q=_ptr(a["q"]),
                 k=_ptr(a["k"]), scal=_ptr(a["scal"]))
        return s, a

    def _obs(self, obs):
        o = dict(geo=_d(obs.geo()), rad=_d(obs.rad).copy(), tau=np.zeros((self.ctl.nd, obs.nr)),
                 tp=np.zeros((3, obs.nr)))
        s = _Obs(nr=obs.nr, geo=_ptr(o["geo"]), rad=_ptr(o["rad"]), tau=_ptr(o["tau"]),
                 tp=_ptr(o["tp"]))
        return s, o

    def formod(self, atm, obs):
        """Forward model; returns (rad, tau, tp, p_after_hydrostatic)."""
        sa, a = self._atm(atm)
        so, o = self._obs(obs)
        self._check(lib().jrc_formod(self.h, C.byref(sa), C.byref(so)))
        return o["rad"], o["tau"], o["tp"], a["p"]

    def formod_batch(self, b, nthreads=0):
        b = b.copy()
        L = lib()
        arr = {k: _d(getattr(b, k)) for k in ("time", "z", "lon", "lat", "p", "t", "q", "k",
                                               "scal", "geo", "rad", "tau", "tp")}
        lev = np.ascontiguousarray(b.lev_off, np.int32)
        ray = np.ascontiguousarray(b.ray_off, np.int32)
        self._check(L.jrc_formod_batch(self.h, b.nobs, _ptr(lev, _ip), _ptr(arr["time"]),
                                       _ptr(arr["z"]), _ptr(arr["lon"]), _ptr(arr["lat"]),
                                       _ptr(arr["p"]), _ptr(arr["t"]), _ptr(arr["q"]),
                                       _ptr(arr["k"]), _ptr(arr["scal"]), _ptr(ray, _ip),
                                       _ptr(arr["geo"]), _ptr(arr["rad"]), _ptr(arr["tau"]),
                                       _ptr(arr["tp"]), nthreads))
        b.rad, b.tau, b.tp, b.p = arr["rad"], arr["tau"], arr["tp"], arr["p"]
        return b

    def raytrace(self, atm, obs, ir, maxpts=8192):
        sa, a = self._atm(atm)
        so, o = self._obs(obs)
        w = 7 + 5 * self.ctl.ng + 2 * self.ctl.nd
        out = np.zeros((maxpts, w))
        n = lib().jrc_raytrace(self.h, C.byref(sa), C.byref(so), ir, maxpts, _ptr(out))
        if n < 0:
            raise RuntimeError("oracle raytrace failed (%d)" % n)
        return out[:n], o["tp"][:, ir]

    def sizes(self, atm, obs):
        sa, a = self._atm(atm)
        so, o = self._obs(obs)
        m, n = C.c_int(), C.c_int()
        lib().jrc_sizes(self.h, C.byref(sa), C.byref(so), C.byref(m), C.byref(n))
        return m.value, n.value

    def atm2x(self, atm):
        sa, a = self._atm(atm)
        n = lib().jrc_atm2x(self.h, C.byref(sa), None, None, None)
        x = np.zeros(n)
        iqa = np.zeros(n, np.int32)
        ipa = np.zeros(n, np.int32)
        lib().jrc_atm2x(self.h, C.byref(sa), _ptr(x), _ptr(iqa, _ip), _ptr(ipa, _ip))
        return x, iqa, ipa

    def kernel(self, atm, obs, nthreads=0):
        m, n = self.sizes(atm, obs)
        sa, a = self._atm(atm)
        so, o = self._obs(obs)
        K = np.zeros((m, n))
        self._check(lib().jrc_kernel(self.h, C.byref(sa), C.byref(so), _ptr(K), nthreads))
        return K

    def retrieval(self, ret, atm_apr, obs_meas, nthreads=0, maxcost=64):
        ctl = self.ctl
        r = ret.sized(ctl)
        keep = {k: _d(getattr(r, k)) for k in ("err_formod", "err_noise", "err_q", "err_q_cz",
                                                "err_q_ch", "err_k", "err_k_cz", "err_k_ch",
                                                "err_clk", "err_sfeps")}
        sr = _Ret(kernel_recomp=r.kernel_recomp, conv_itmax=r.conv_itmax, err_ana=r.err_ana,
                  conv_dmin=r.conv_dmin, err_press=r.err_press, err_press_cz=r.err_press_cz,
                  err_press_ch=r.err_press_ch, err_temp=r.err_temp, err_temp_cz=r.err_temp_cz,
                  err_temp_ch=r.err_temp_ch, err_clz=r.err_clz, err_cldz=r.err_cldz,
                  err_sfz=r.err_sfz, err_sfp=r.err_sfp, err_sft=r.err_sft,
                  **{k: _ptr(v) for k, v in keep.items()})
        m, n = self.sizes(atm_apr, obs_meas)
        sa, a = self._atm(atm_apr)
        so, o = self._obs(obs_meas)
        x = np.zeros(n)
        y = np.zeros(m)
        cov = np.zeros((n, n))
        costs = np.zeros(maxcost)
        info = np.zeros(4, np.int32)
        ana = dict(gain=np.zeros((n, m)), avk=np.zeros((n, n)), err_total=np.zeros(n),
                   err_noise=np.zeros(n), err_formod=np.zeros(n), cont=np.zeros(n),
                   res=np.zeros(n))
        sana = _Ana(**{k: _ptr(v) for k, v in ana.items()})
        self._check(lib().jrc_retrieval_ex(self.h, C.byref(sr), C.byref(sa), C.byref(so),
                                           _ptr(x), _ptr(y), _ptr(cov), _ptr(costs), maxcost,
                                           _ptr(info, _ip), nthreads, C.byref(sana)))
        out = dict(x=x, y=y, cov=cov if r.err_ana else None, costs=costs[:info[2]],
                   n=int(info[0]), m=int(info[1]), iters=int(info[3]))
        if r.err_ana:
            out.update(ana)
        return out
