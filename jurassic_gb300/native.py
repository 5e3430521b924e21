"""ctypes binding to libjurassic_gb300.so and the Python mirror of the
reference's forward-model interface.

``Context`` owns one device context (``jgb_ctx``); its methods follow the
reference functions they replace:

* ``formod(atm, obs)``        -- formod (src/jurassic.c:3026-3071)
* ``formod_batch(batch)``     -- jur_unified_formod_multiple_packages seam
                                 (src/formod.c:72-73), host buffers
* ``formod_batch_dev(dev)``   -- same on device-resident inputs

The CUDA library is the only compute path: if it cannot be loaded the
import fails with an error; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

from .model import Atm, Ctl, JurassicError, Obs

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libjurassic_gb300.so")

JGB_OK = 0
# status codes of the C ABI (jurassic_gb300.h)
ERR_ARG, ERR_CUDA, ERR_STATE, ERR_LOS, ERR_SURFACE, ERR_UNSUPPORTED, ERR_IO, ERR_NUMERIC = range(1, 9)
FP64 = 0
MIXED = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_fp = C.POINTER(C.c_float)


class _Ctl(C.Structure):
    _fields_ = [("ng", C.c_int), ("emitter", C.POINTER(C.c_char_p)), ("nd", C.c_int),
                ("nu", _dp), ("nw", C.c_int), ("window", _ip), ("ncl", C.c_int),
                ("clnu", _dp), ("nsf", C.c_int), ("sfnu", _dp), ("sftype", C.c_int),
                ("sfsza", C.c_double), ("hydz", C.c_double), ("ctm_co2", C.c_int),
                ("ctm_h2o", C.c_int), ("ctm_n2", C.c_int), ("ctm_o2", C.c_int),
                ("refrac", C.c_int), ("rayds", C.c_double), ("raydz", C.c_double),
                ("formod", C.c_int), ("write_bbt", C.c_int), ("retp_zmin", C.c_double),
                ("retp_zmax", C.c_double), ("rett_zmin", C.c_double), ("rett_zmax", C.c_double),
                ("retq_zmin", _dp), ("retq_zmax", _dp), ("retk_zmin", _dp), ("retk_zmax", _dp),
                ("ret_clz", C.c_int), ("ret_cldz", C.c_int), ("ret_clk", C.c_int),
                ("ret_sfz", C.c_int), ("ret_sfp", C.c_int), ("ret_sft", C.c_int),
                ("ret_sfeps", C.c_int), ("nlos_max", C.c_int)]


class _Batch(C.Structure):
    _fields_ = [("nobs", C.c_int), ("lev_off", _ip), ("time", _dp), ("z", _dp), ("lon", _dp),
                ("lat", _dp), ("p", _dp), ("t", _dp), ("q", _dp), ("k", _dp), ("scal", _dp),
                ("ray_off", _ip), ("geo", _dp), ("rad", _dp), ("tau", _dp), ("tp", _dp)]


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


class Stats(C.Structure):
    _fields_ = [("h2d_ms", C.c_double), ("hydro_ms", C.c_double), ("trace_ms", C.c_double),
                ("pack_ms", C.c_double), ("path_ms", C.c_double), ("d2h_ms", C.c_double),
                ("total_ms", C.c_double), ("los_points", C.c_longlong),
                ("path_launches", C.c_int), ("path_variant", C.c_int),
                ("tune_ms", C.c_float * 16), ("trace_passes", C.c_int),
                ("resume_skip", C.c_double)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["tune_ms"] = list(self.tune_ms)
        return d


class EngineStats(C.Structure):
    _fields_ = [("submitted", C.c_ulonglong), ("finished", C.c_ulonglong),
                ("failed", C.c_ulonglong), ("steps", C.c_ulonglong), ("rebuilds", C.c_ulonglong),
                ("forward_calls", C.c_ulonglong), ("lm_trials", C.c_ulonglong),
                ("jacobians", C.c_ulonglong), ("step_ms", C.c_double),
                ("rebuild_ms", C.c_double), ("init_ms", C.c_double), ("jacobian_ms", C.c_double),
                ("normal_ms", C.c_double), ("trial_ms", C.c_double), ("finish_ms", C.c_double),
                ("trial_fwd_ms", C.c_double), ("trial_trace_ms", C.c_double),
                ("trial_path_ms", C.c_double),
                ("active", C.c_int),
                ("queued", C.c_int), ("done", C.c_int), ("used_bytes", C.c_ulonglong)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class _RetOut(C.Structure):
    _fields_ = [(k, _dp) for k in ("x", "cov", "costs", "rad", "tau", "tp", "p", "gain", "avk",
                                   "err_total", "err_noise", "err_formod", "cont", "res")] + \
               [("iters", C.c_int), ("status", C.c_int), ("has_err_ana", C.c_int)]


# exported symbols and their signatures (the contract of include/jurassic_gb300.h)
SIGNATURES = {
    "jgb_create": (C.c_int, [C.POINTER(_Ctl), C.c_int, C.POINTER(C.c_void_p)]),
    "jgb_destroy": (None, [C.c_void_p]),
    "jgb_last_error": (C.c_char_p, [C.c_void_p]),
    "jgb_tables_init": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "jgb_set_table": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _ip, _dp, _ip, _fp,
                                _fp, C.c_int, C.c_int]),
    "jgb_set_filter": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp, _dp]),
    "jgb_read_tables": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "jgb_read_table_file": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, _ip, _dp, _ip,
                                      _dp, _ip, _fp, _fp]),
    "jgb_write_table_file": (C.c_int, [C.c_char_p, C.c_int, C.c_int, _dp, _ip, _dp, _ip, _fp, _fp,
                                       C.c_int, C.c_int]),
    "jgb_set_fov": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "jgb_set_los_bound_scale": (C.c_int, [C.c_void_p, C.c_double]),
    "jgb_set_path_split": (C.c_int, [C.c_void_p, C.c_int]),
    "jgb_set_fd_resume": (C.c_int, [C.c_void_p, C.c_int]),
    "jgb_set_srcfunc": (C.c_int, [C.c_void_p, _dp]),
    "jgb_get_srcfunc": (C.c_int, [C.c_void_p, _dp, _dp]),
    "jgb_formod": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                             C.c_int, _dp, _dp, _dp, _dp, C.c_int]),
    "jgb_formod_batch": (C.c_int, [C.c_void_p, C.POINTER(_Batch), C.c_int]),
    "jgb_formod_batch_dev": (C.c_int, [C.c_void_p, C.POINTER(_Batch), C.c_int]),
    "jgb_kernel_sizes": (C.c_int, [C.c_void_p, C.POINTER(_Batch), _ip, _ip]),
    "jgb_kernel_batch": (C.c_int, [C.c_void_p, C.POINTER(_Batch), _dp, C.c_int]),
    "jgb_normal_equations": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, _dp, _dp, _dp, _dp, _dp,
                                       C.c_int]),
    "jgb_formod_contrib": (C.c_int, [C.c_void_p, C.POINTER(_Batch), _dp, _dp, C.c_int]),
    "jgb_normal_equations_dev": (C.c_int, [C.c_void_p, C.c_int, _ip, _ip, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                           C.POINTER(C.c_float)]),
    "jgb_matrix_invert": (C.c_int, [C.c_void_p, C.c_int, _ip, _dp, _ip]),
    "jgb_matrix_invert_dev": (C.c_int, [C.c_void_p, C.c_int, _ip, C.c_void_p, _ip,
                                        C.POINTER(C.c_float)]),
    "jgb_retrieve_batch": (C.c_int, [C.c_void_p, C.POINTER(_Ret), C.POINTER(_Batch), _dp, _dp,
                                     _dp, _ip, C.c_int]),
    "jgb_get_stats": (C.c_int, [C.c_void_p, C.POINTER(Stats)]),
    "jgb_engine_create": (C.c_int, [C.c_void_p, C.POINTER(_Ret), C.c_int, C.c_ulonglong, C.c_int,
                                    C.c_int, C.POINTER(C.c_void_p)]),
    "jgb_engine_destroy": (None, [C.c_void_p]),
    "jgb_engine_submit": (C.c_int, [C.c_void_p, C.POINTER(_Batch), C.POINTER(C.c_ulonglong)]),
    "jgb_engine_step": (C.c_int, [C.c_void_p, _ip, _ip, _ip]),
    "jgb_engine_finished": (C.c_int, [C.c_void_p, C.POINTER(C.c_ulonglong), C.c_int, _ip]),
    "jgb_engine_sizes": (C.c_int, [C.c_void_p, C.c_ulonglong, _ip, _ip, _ip, _ip]),
    "jgb_engine_result": (C.c_int, [C.c_void_p, C.c_ulonglong, C.POINTER(_RetOut)]),
    "jgb_engine_get_stats": (C.c_int, [C.c_void_p, C.POINTER(EngineStats)]),
    "jgb_formod_batch_dev_noalloc": (C.c_int, [C.c_void_p, C.POINTER(_Batch)]),
    "jgb_atm2x": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]),
    "jgb_x2atm": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "jgb_read_shape": (C.c_int, [C.c_char_p, C.c_int, _dp, _dp, _ip]),
    "jgb_host_alloc": (C.c_void_p, [C.c_ulonglong]),
    "jgb_host_free": (None, [C.c_void_p]),
    "jgb_dev_alloc": (C.c_void_p, [C.c_ulonglong]),
    "jgb_measure_l2_read": (C.c_int, [C.c_ulonglong, C.c_int, C.POINTER(C.c_double)]),
    "jgb_selftest_bounded_wait": (C.c_int, [C.c_int, C.c_int, _ip, C.POINTER(C.c_double)]),
    "jgb_dev_free": (None, [C.c_void_p]),
    "jgb_memcpy_h2d": (C.c_int, [C.c_void_p, C.c_void_p, C.c_ulonglong]),
    "jgb_memcpy_d2h": (C.c_int, [C.c_void_p, C.c_void_p, C.c_ulonglong]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load the CUDA library (raises if it is missing: no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise ImportError("libjurassic_gb300.so not built (run __graft_entry__.build())")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


class Context:
    """One device context: control set, tables and source function."""

    def __init__(self, ctl: Ctl, tables=None, filters=None, device: int = 0,
                 nlos_max: int = 4096, srcfunc: Optional[np.ndarray] = None, fov=None):
        L = load()
        self.ctl = ctl
        self._keep = dict(
            names=(C.c_char_p * max(ctl.ng, 1))(*[e.encode() for e in ctl.emitter]),
            nu=_d(ctl.nu), window=np.ascontiguousarray(ctl.window, np.int32),
            clnu=_d(ctl.clnu), sfnu=_d(ctl.sfnu), rqn=_d(ctl.retq_zmin), rqx=_d(ctl.retq_zmax),
            rkn=_d(ctl.retk_zmin), rkx=_d(ctl.retk_zmax))
        k = self._keep
        c = _Ctl(ng=ctl.ng, emitter=C.cast(k["names"], C.POINTER(C.c_char_p)), nd=ctl.nd,
                 nu=_p(k["nu"]), nw=ctl.nw, window=_p(k["window"], _ip), ncl=ctl.ncl,
                 clnu=_p(k["clnu"]), nsf=ctl.nsf, sfnu=_p(k["sfnu"]), sftype=ctl.sftype,
                 sfsza=ctl.sfsza, hydz=ctl.hydz, ctm_co2=ctl.ctm_co2, ctm_h2o=ctl.ctm_h2o,
                 ctm_n2=ctl.ctm_n2, ctm_o2=ctl.ctm_o2, refrac=ctl.refrac, rayds=ctl.rayds,
                 raydz=ctl.raydz, formod=ctl.formod, write_bbt=ctl.write_bbt,
                 retp_zmin=ctl.retp_zmin, retp_zmax=ctl.retp_zmax, rett_zmin=ctl.rett_zmin,
                 rett_zmax=ctl.rett_zmax, retq_zmin=_p(k["rqn"]), retq_zmax=_p(k["rqx"]),
                 retk_zmin=_p(k["rkn"]), retk_zmax=_p(k["rkx"]), ret_clz=ctl.ret_clz,
                 ret_cldz=ctl.ret_cldz, ret_clk=ctl.ret_clk, ret_sfz=ctl.ret_sfz,
                 ret_sfp=ctl.ret_sfp, ret_sft=ctl.ret_sft, ret_sfeps=ctl.ret_sfeps,
                 nlos_max=nlos_max)
        h = C.c_void_p()
        rc = L.jgb_create(C.byref(c), device, C.byref(h))
        if rc != JGB_OK:
            raise JurassicError("jgb_create failed (%d)" % rc)
        self.h = h
        if tables is not None:
            self.set_tables(tables)
        if srcfunc is not None:
            self.set_srcfunc(srcfunc)
        elif filters is not None:
            self.set_filters(filters)
        if fov is not None:
            self.set_fov(*fov)

    def set_fov(self, dz, w):
        """Field of view (formod_fov): shape samples dz [km], w (read_shape
        of the file named by the FOV control parameter); empty arrays turn it
        off."""
        dz, w = _d(dz), _d(w)
        self._check(load().jgb_set_fov(self.h, len(dz), _p(dz), _p(w)))

    def set_los_bound_scale(self, scale: float):
        """Factor on the per-ray LOS-point bound of one-pass mixed ray tracing
        of large batches (0: always count the rays first)."""
        self._check(load().jgb_set_los_bound_scale(self.h, float(scale)))

    def set_path_split(self, mode: int):
        """Mixed path loop split over the emitters: -1 for batches too small
        to fill the device (default), 0 never, 1 always."""
        self._check(load().jgb_set_path_split(self.h, int(mode)))

    def set_fd_resume(self, mode: int):
        """Resume perturbed paths of mixed Jacobians from their base's saved
        state: 1 when the estimated schedule is shorter (default), 2 always,
        0 never; 3 always, with the emitters a perturbation leaves unchanged
        always taken from the base (the results do not depend on it)."""
        self._check(load().jgb_set_fd_resume(self.h, int(mode)))

    def _check(self, rc):
        if rc != JGB_OK:
            raise JurassicError("libjurassic_gb300 error %d: %s" % (
                rc, load().jgb_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            load().jgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_tables(self, tbl):
        L = load()
        nd, ng, tp, tt, tu = tbl.u.shape
        self._check(L.jgb_tables_init(self.h, tp, tt, tu))
        for id in range(nd):
            for ig in range(ng):
                n = int(tbl.np_[id, ig])
                p = _d(tbl.p[id, ig])
                nt = np.ascontiguousarray(tbl.nt[id, ig], np.int32)
                t = _d(tbl.t[id, ig])
                nu = np.ascontiguousarray(tbl.nu[id, ig], np.int32)
                u = np.ascontiguousarray(tbl.u[id, ig], np.float32)
                e = np.ascontiguousarray(tbl.eps[id, ig], np.float32)
                self._check(L.jgb_set_table(self.h, id, ig, n, _p(p), _p(nt, _ip), _p(t),
                                            _p(nu, _ip), _p(u, _fp), _p(e, _fp), tt, tu))

    def read_tables(self, tblbase: str, tblfmt: int, tp=41, tt=30, tu=320):
        """Emissivity tables from the reference's files (read_tbl,
        jurassic.c:4949-5110), read by the library and uploaded; tp, tt, tu
        are the capacities (TBLNP, TBLNT, TBLNU)."""
        L = load()
        self._check(L.jgb_tables_init(self.h, tp, tt, tu))
        self._check(L.jgb_read_tables(self.h, tblbase.encode(), int(tblfmt)))

    def set_filters(self, filters):
        for id, (fnu, f) in enumerate(filters):
            fnu, f = _d(fnu), _d(f)
            self._check(load().jgb_set_filter(self.h, id, len(fnu), _p(fnu), _p(f)))

    def set_srcfunc(self, sr):
        sr = _d(sr)
        self._check(load().jgb_set_srcfunc(self.h, _p(sr)))

    def srcfunc(self):
        st = np.zeros(1200)
        sr = np.zeros((1200, self.ctl.nd))
        self._check(load().jgb_get_srcfunc(self.h, _p(st), _p(sr)))
        return st, sr

    def stats(self) -> dict:
        s = Stats()
        load().jgb_get_stats(self.h, C.byref(s))
        return s.as_dict()

    # --------------------------------------------------------------
    def formod(self, atm: Atm, obs: Obs, precision: int = FP64) -> Obs:
        """Forward model of one observation; returns a new Obs with rad/tau/tp
        filled (and updates atm.p when hydrostatic equilibrium is on)."""
        ctl = self.ctl
        out = obs.copy()
        a = dict(time=_d(atm.time), z=_d(atm.z), lon=_d(atm.lon), lat=_d(atm.lat),
                 p=_d(atm.p).copy(), t=_d(atm.t), q=_d(np.asarray(atm.q).reshape(ctl.ng, -1)),
                 k=_d(np.asarray(atm.k).reshape(max(ctl.nw, 0), -1)), scal=_d(atm.scal(ctl)))
        geo = _d(obs.geo())
        rad = _d(obs.rad).copy()
        tau = np.zeros((ctl.nd, obs.nr))
        tp = np.zeros((3, obs.nr))
        self._check(load().jgb_formod(self.h, atm.np, _p(a["time"]), _p(a["z"]), _p(a["lon"]),
                                      _p(a["lat"]), _p(a["p"]), _p(a["t"]), _p(a["q"]),
                                      _p(a["k"]), _p(a["scal"]), obs.nr, _p(geo), _p(rad),
                                      _p(tau), _p(tp), precision))
        out.rad, out.tau = rad, tau
        out.tpz, out.tplon, out.tplat = tp[0].copy(), tp[1].copy(), tp[2].copy()
        atm.p = a["p"]
        return out

    def formod_batch(self, batch, precision: int = FP64):
        """Batched forward model on host arrays; returns a new Batch."""
        b = batch.copy()
        arr = {k: _d(getattr(b, k)) for k in ("time", "z", "lon", "lat", "p", "t", "q", "k",
                                               "scal", "geo", "rad", "tau", "tp")}
        lev = np.ascontiguousarray(b.lev_off, np.int32)
        ray = np.ascontiguousarray(b.ray_off, np.int32)
        s = _Batch(nobs=b.nobs, lev_off=_p(lev, _ip), ray_off=_p(ray, _ip),
                   **{k: _p(v) for k, v in arr.items()})
        self._check(load().jgb_formod_batch(self.h, C.byref(s), precision))
        for k in ("rad", "tau", "tp", "p"):
            setattr(b, k, arr[k])
        return b

    def formod_batch_ptrs(self, ptrs: dict, nobs: int, precision: int = FP64,
                          device: bool = True):
        """Batched forward model on raw pointers (device pointers by default);
        ``ptrs`` maps jgb_batch field names to integer addresses."""
        s = _Batch(nobs=nobs, **{k: C.cast(C.c_void_p(v), _ip if k in ("lev_off", "ray_off") else _dp)
                                 for k, v in ptrs.items()})
        fn = load().jgb_formod_batch_dev if device else load().jgb_formod_batch
        self._check(fn(self.h, C.byref(s), precision))

    # --------------------------------------------------------------
    def _batch_struct(self, b):
        arr = {k: _d(getattr(b, k)) for k in ("time", "z", "lon", "lat", "p", "t", "q", "k",
                                               "scal", "geo", "rad", "tau", "tp")}
        lev = np.ascontiguousarray(b.lev_off, np.int32)
        ray = np.ascontiguousarray(b.ray_off, np.int32)
        s = _Batch(nobs=b.nobs, lev_off=_p(lev, _ip), ray_off=_p(ray, _ip),
                   **{k: _p(v) for k, v in arr.items()})
        return s, arr, (lev, ray)

    def kernel_sizes(self, batch):
        s, arr, keep = self._batch_struct(batch)
        m = np.zeros(batch.nobs, np.int32)
        n = np.zeros(batch.nobs, np.int32)
        self._check(load().jgb_kernel_sizes(self.h, C.byref(s), _p(m, _ip), _p(n, _ip)))
        return m, n

    def kernel_batch(self, batch, precision: int = FP64):
        """Finite-difference Jacobians of every observation (kernel,
        src/jurassic.c:4004-4099).  Returns (list of K_i [m_i, n_i], Batch with
        the unperturbed forward model)."""
        m, n = self.kernel_sizes(batch)
        b = batch.copy()
        s, arr, keep = self._batch_struct(b)
        kmat = np.zeros(int(np.sum(m.astype(np.int64) * n)))
        self._check(load().jgb_kernel_batch(self.h, C.byref(s), _p(kmat), precision))
        for k in ("rad", "tau", "tp", "p"):
            setattr(b, k, arr[k])
        out, o = [], 0
        for mi, ni in zip(m, n):
            out.append(kmat[o:o + mi * ni].reshape(mi, ni))
            o += mi * ni
        return out, b

    def kernel(self, atm: Atm, obs: Obs, precision: int = FP64):
        """Jacobian of one observation (the reference kernel())."""
        from .synth import pack
        K, b = self.kernel_batch(pack(self.ctl, [(atm, obs)]), precision)
        return K[0]

    def normal_equations(self, Ks, ws, dys, precision: int = MIXED):
        """A_i = K_i^T diag(w_i^2) K_i and b_i = K_i^T diag(w_i^2) dy_i for
        lists of K_i [m_i, n_i], w_i [m_i], dy_i [m_i]."""
        m = np.array([k.shape[0] for k in Ks], np.int32)
        n = np.array([k.shape[1] for k in Ks], np.int32)
        K = _d(np.concatenate([np.ravel(k) for k in Ks]))
        w = _d(np.concatenate(ws))
        dy = _d(np.concatenate(dys))
        A = np.zeros(int(np.sum(n.astype(np.int64) ** 2)))
        b = np.zeros(int(np.sum(n)))
        self._check(load().jgb_normal_equations(self.h, len(Ks), _p(m, _ip), _p(n, _ip), _p(K),
                                                _p(w), _p(dy), _p(A), _p(b), precision))
        outA, outb, oa, ob = [], [], 0, 0
        for ni in n:
            outA.append(A[oa:oa + ni * ni].reshape(ni, ni))
            outb.append(b[ob:ob + ni])
            oa += ni * ni
            ob += ni
        return outA, outb

    def matrix_invert(self, As):
        """Inverses of a list of symmetric positive-definite matrices
        (matrix_invert, retrieval.c:373-399), FP64 on the device.  Returns
        (inverses, status); status[i] = 1 where A_i is not positive definite
        (its entry is then A_i unchanged)."""
        n = np.array([a.shape[0] for a in As], np.int32)
        A = _d(np.concatenate([np.ravel(a) for a in As]))
        st = np.zeros(len(As), np.int32)
        self._check(load().jgb_matrix_invert(self.h, len(As), _p(n, _ip), _p(A), _p(st, _ip)))
        out, o = [], 0
        for ni in n:
            out.append(A[o:o + ni * ni].reshape(ni, ni))
            o += ni * ni
        return out, st

    def contributions(self, batch, precision: int = FP64):
        """Emitter contributions (TASK c, src/formod.c:200-249): continua off,
        one forward model per emitter with only that emitter's mixing ratio
        (no extinction), then one with the extinction only.  ``batch`` holds
        the atmosphere as after formod.  Returns (rad, tau) of shape
        [ng+1, nd, nray]; entry ng is "EXTINCT"."""
        ctl = self.ctl
        s, arr, keep = self._batch_struct(batch)
        rad = np.zeros((ctl.ng + 1, ctl.nd, batch.nray))
        tau = np.zeros_like(rad)
        self._check(load().jgb_formod_contrib(self.h, C.byref(s), _p(rad), _p(tau), precision))
        return rad, tau

    def _ret_struct(self, ret):
        r = ret.sized(self.ctl)
        keep = {k: _d(getattr(r, k)) for k in ("err_formod", "err_noise", "err_q", "err_q_cz",
                                                "err_q_ch", "err_k", "err_k_cz", "err_k_ch",
                                                "err_clk", "err_sfeps")}
        sr = _Ret(kernel_recomp=r.kernel_recomp, conv_itmax=r.conv_itmax, err_ana=r.err_ana,
                  conv_dmin=r.conv_dmin, err_press=r.err_press, err_press_cz=r.err_press_cz,
                  err_press_ch=r.err_press_ch, err_temp=r.err_temp, err_temp_cz=r.err_temp_cz,
                  err_temp_ch=r.err_temp_ch, err_clz=r.err_clz, err_cldz=r.err_cldz,
                  err_sfz=r.err_sfz, err_sfp=r.err_sfp, err_sft=r.err_sft,
                  **{k: _p(v) for k, v in keep.items()})
        return r, sr, keep

    def engine(self, ret, precision: int = FP64, mem_budget: int = 0, max_active: int = 0,
               keep_gain: bool = False) -> "Engine":
        """Continuous-batching retrieval engine on this context."""
        return Engine(self, ret, precision, mem_budget, max_active, keep_gain)

    def retrieve_batch(self, ret, batch, precision: int = FP64):
        """Optimal-estimation retrievals (optimal_estimation,
        src/retrieval.c:448-749) of every observation of a batch: the batch
        holds the a-priori atmospheres and, in rad, the measurements.
        Returns dict(x=[state vectors], cov=[covariances or None],
        costs=[chi^2/m histories], iters=[...], batch=final forward model)."""
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
                  **{k: _p(v) for k, v in keep.items()})
        m, n = self.kernel_sizes(batch)
        b = batch.copy()
        s, arr, ks = self._batch_struct(b)
        nx = int(np.sum(n))
        x = np.zeros(nx)
        cov = np.zeros(int(np.sum(n.astype(np.int64) ** 2))) if r.err_ana else None
        ncost = r.conv_itmax + 1
        costs = np.zeros(b.nobs * ncost)
        iters = np.zeros(b.nobs, np.int32)
        self._check(load().jgb_retrieve_batch(self.h, C.byref(sr), C.byref(s), _p(x),
                                              _p(cov) if cov is not None else None, _p(costs),
                                              _p(iters, _ip), precision))
        for k in ("rad", "tau", "tp", "p"):
            setattr(b, k, arr[k])
        xs, covs, ox, oc = [], [], 0, 0
        for ni in n:
            xs.append(x[ox:ox + ni])
            covs.append(cov[oc:oc + ni * ni].reshape(ni, ni) if cov is not None else None)
            ox += ni
            oc += ni * ni
        cs = costs.reshape(b.nobs, ncost)
        return dict(x=xs, cov=covs, costs=[c[np.isfinite(c)] for c in cs],
                    iters=iters.tolist(), batch=b)


class Engine:
    """Continuous-batching retrieval engine (jgb_engine_*): submit
    observations as requests, step, collect results per request id.

    Results are dicts with x, costs (finite entries), iters, status, rad,
    tau, tp, p and, with error analysis, cov, avk, gain (if kept),
    err_total, err_noise, err_formod, cont, res."""

    def __init__(self, ctx: Context, ret, precision: int = FP64, mem_budget: int = 0,
                 max_active: int = 0, keep_gain: bool = False):
        self.ctx = ctx
        self.keep_gain = bool(keep_gain)
        self.r, sr, self._keep = ctx._ret_struct(ret)
        h = C.c_void_p()
        ctx._check(load().jgb_engine_create(ctx.h, C.byref(sr), precision, int(mem_budget),
                                            int(max_active), int(keep_gain), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            load().jgb_engine_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, batch) -> list:
        s, arr, keep = self.ctx._batch_struct(batch)
        ids = (C.c_ulonglong * batch.nobs)()
        self.ctx._check(load().jgb_engine_submit(self.h, C.byref(s), ids))
        return list(ids)

    def step(self):
        a, q, d = C.c_int(), C.c_int(), C.c_int()
        self.ctx._check(load().jgb_engine_step(self.h, C.byref(a), C.byref(q), C.byref(d)))
        return a.value, q.value, d.value

    def finished(self, max_ids: int = 65536) -> list:
        ids = (C.c_ulonglong * max_ids)()
        n = C.c_int()
        self.ctx._check(load().jgb_engine_finished(self.h, ids, max_ids, C.byref(n)))
        return list(ids[:n.value])

    def stats(self) -> dict:
        st = EngineStats()
        self.ctx._check(load().jgb_engine_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def result(self, rid: int) -> dict:
        n, m, npl, nr = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        L = load()
        self.ctx._check(L.jgb_engine_sizes(self.h, rid, C.byref(n), C.byref(m), C.byref(npl),
                                           C.byref(nr)))
        n, m, npl, nr = n.value, m.value, npl.value, nr.value
        nd = self.ctx.ctl.nd
        ana = bool(self.r.err_ana)
        out = dict(x=np.zeros(n), costs=np.zeros(self.r.conv_itmax + 1), rad=np.zeros((nd, nr)),
                   tau=np.zeros((nd, nr)), tp=np.zeros((3, nr)), p=np.zeros(npl))
        if ana:
            out.update(cov=np.zeros((n, n)), avk=np.zeros((n, n)), gain=np.zeros((n, m)),
                       err_total=np.zeros(n), err_noise=np.zeros(n), err_formod=np.zeros(n),
                       cont=np.zeros(n), res=np.zeros(n))
        ro = _RetOut(**{k: _p(v) for k, v in out.items()})
        self.ctx._check(L.jgb_engine_result(self.h, rid, C.byref(ro)))
        out["costs"] = out["costs"][np.isfinite(out["costs"])]
        out["iters"] = ro.iters
        out["status"] = ro.status
        if ana and not ro.has_err_ana:
            for k in ("cov", "avk", "gain", "err_total", "err_noise", "err_formod", "cont", "res"):
                out[k] = None
        if ana and not self.keep_gain:
            out["gain"] = None
        return out

    def run(self, batch) -> list:
        """Submit a batch, step until all of it is done, results in order."""
        ids = self.submit(batch)
        want = set(ids)
        res = {}
        while want - set(res):
            self.step()
            for rid in self.finished():
                if rid in want:
                    res[rid] = self.result(rid)
        return [res[i] for i in ids]
