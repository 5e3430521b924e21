"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every input is generated here from a
``numpy.random.default_rng(seed)`` stream so that the library, the CPU
oracle and the reference build read identical numbers.

* Emissivity tables: log-spaced pressures, regular temperature grid,
  log-spaced column densities (factor ~1.122 per step), band emissivity
  ``eps = 1 - exp(-k u)`` with ``k = k0 (p/1013)^a (T/250)^b`` and seeded
  ``k0, a, b`` per (channel, emitter).  Rows are truncated as table
  generators do (1e-6 <= eps <= 0.999999, strictly increasing in float32),
  so rows are ragged.
* Filter functions: trapezoidal channel responses.
* Atmospheres: an analytic standard atmosphere (piecewise-linear temperature
  with tropospheric lapse rate, hydrostatic pressure, analytic trace-gas
  profiles) with seeded perturbations.
* Geometry: limb rays (view point = geometric tangent point) and nadir
  rays with a small seeded scan angle.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence

import numpy as np

from .model import Atm, Ctl, Obs, Ret, limb_vplat
from .tables import Tables

RE = 6367.421

# typical total vertical columns [molec/cm^2] used to place k0 so that
# band optical depths span ~0.01 .. 100
_COLUMNS = {"CO2": 8.6e21, "H2O": 3e22, "O3": 8e18, "CH4": 3.5e19,
            "N2O": 6e18, "F11": 5e15, "CCL4": 2e15, "CO": 2e18}


def std_temperature(z):
    """Piecewise-linear temperature [K] (tropospheric lapse rate 6.5 K/km)."""
    z = np.asarray(z, dtype=np.float64)
    nodes = np.array([0, 11, 20, 32, 47, 51, 71, 86, 100, 120], float)
    temps = [288.15]
    rates = [-6.5, 0.0, 1.0, 2.8, 0.0, -2.8, -2.0, 0.0, 3.0]
    for i, r in enumerate(rates):
        temps.append(temps[-1] + r * (nodes[i + 1] - nodes[i]))
    return np.interp(z, nodes, np.array(temps))


def hydrostatic_pressure(z, t, p0=1013.25):
    """Pressure [hPa] from T(z) by integrating dp/p = -g M/(R T) dz."""
    z = np.asarray(z, dtype=np.float64)
    g, M, R = 9.80665, 28.9644e-3, 8.3144598
    p = np.empty_like(z)
    p[0] = p0 * math.exp(-g * M / (R * t[0]) * z[0] * 1000.0)
    for i in range(1, len(z)):
        tm = 0.5 * (t[i] + t[i - 1])
        p[i] = p[i - 1] * math.exp(-g * M / (R * tm) * (z[i] - z[i - 1]) * 1000.0)
    return p


def std_vmr(name, z):
    z = np.asarray(z, dtype=np.float64)
    n = name.upper()
    if n == "CO2":
        return np.full_like(z, 4e-4)
    if n == "H2O":
        return 1e-2 * np.exp(-z / 2.0) + 4e-6
    if n == "O3":
        return 8e-6 * np.exp(-((z - 32.0) / 9.0) ** 2) + 3e-8
    if n == "CH4":
        return np.where(z < 15, 1.8e-6, 1.8e-6 * np.exp(-(z - 15) / 25.0))
    if n == "N2O":
        return np.where(z < 15, 3.2e-7, 3.2e-7 * np.exp(-(z - 15) / 7.0))
    if n in ("F11", "CCL4"):
        return np.where(z < 15, 2.5e-10, 2.5e-10 * np.exp(-(z - 15) / 5.0))
    return np.full_like(z, 1e-9)


def make_tables(ctl: Ctl, seed: int, tp=41, tt=30, tu=320, pmin=1e-3, pmax=1100.0,
                tmin=180.0, tmax=320.0, umin=1e10, umax=1e26, descending_p=False,
                t_shift_per_level=0.0, missing=()) -> Tables:
    """Synthetic emissivity tables for every (channel, emitter)."""
    rng = np.random.default_rng(seed)
    nd, ng = ctl.nd, ctl.ng
    tbl = Tables.empty(nd, ng, tp, tt, tu)
    pgrid = np.logspace(np.log10(pmin), np.log10(pmax), tp)
    if descending_p:
        pgrid = pgrid[::-1].copy()
    ugrid = np.logspace(np.log10(umin), np.log10(umax), tu)
    uu = ugrid.astype(np.float32)
    tgrid = np.linspace(tmin, tmax, tt)[None, :] + t_shift_per_level * (np.arange(tp)[:, None] - tp // 2)
    for ig in range(ng):
        col = _COLUMNS.get(ctl.emitter[ig].upper(), 1e18)
        lo, hi = max(0.01 / col, 1.5e-25), min(100.0 / col, 1e-17)
        lo = min(lo, hi / 10)
        k0 = np.exp(rng.uniform(np.log(lo), np.log(hi), nd))
        aexp = rng.uniform(0.0, 0.5, nd)
        bexp = rng.uniform(-1.0, 1.0, nd)
        for id in range(nd):
            if (id, ig) in missing:
                continue
            tbl.np_[id, ig] = tp
            tbl.p[id, ig, :] = pgrid
            tbl.nt[id, ig, :] = tt
            tbl.t[id, ig] = tgrid
            k = k0[id] * (pgrid[:, None] / 1013.0) ** aexp[id] * (tgrid / 250.0) ** bexp[id]
            eps = (-np.expm1(-k[:, :, None] * ugrid[None, None, :])).astype(np.float32)
            # keep 1e-6 <= eps <= 0.999999 and strictly increasing (float32)
            keep = (eps >= 1e-6) & (eps <= 0.999999)
            prev = np.concatenate([np.full(eps.shape[:2] + (1,), -1.0, np.float32), eps[:, :, :-1]], 2)
            keep &= eps > prev
            order = np.argsort(~keep, axis=2, kind="stable")
            n = keep.sum(axis=2)
            e_sorted = np.take_along_axis(eps, order, axis=2)
            u_sorted = np.broadcast_to(uu, eps.shape)
            u_sorted = np.take_along_axis(u_sorted, order, axis=2)
            valid = np.arange(tu)[None, None, :] < n[:, :, None]
            tbl.nu[id, ig] = n
            tbl.eps[id, ig] = np.where(valid, e_sorted, 0.0)
            tbl.u[id, ig] = np.where(valid, u_sorted, 0.0)
    return tbl


def make_filters(ctl: Ctl, width=1.0, step=0.02):
    """Trapezoidal channel responses: flat over `width`, linear shoulders."""
    out = []
    for nu in ctl.nu:
        n = int(round(1.5 * width / step))
        fnu = nu + (np.arange(-n, n + 1) * step)
        f = np.clip((0.75 * width - np.abs(fnu - nu)) / (0.25 * width), 0.0, 1.0)
        out.append((fnu, f))
    return out


def profile(emitters: Sequence[str], z, rng=None, dt=0.0, dq=None, noise=0.0,
            nw=1, time=0.0, lon=0.0, lat=0.0) -> Atm:
    """Standard-atmosphere profile on altitude grid z with perturbations:
    temperature offset ``dt`` (scalar or per level), per-gas factors ``dq``
    and multiplicative seeded noise of relative size ``noise``."""
    z = np.asarray(z, dtype=np.float64)
    t = std_temperature(z) + dt
    p = hydrostatic_pressure(z, std_temperature(z))
    q = np.stack([std_vmr(e, z) for e in emitters]) if emitters else np.zeros((0, len(z)))
    if dq is not None:
        q = q * np.asarray(dq)[:, None]
    if noise and rng is not None:
        t = t * (1 + noise * rng.standard_normal(len(z)))
        p = p * (1 + noise * rng.standard_normal(len(z)))
        q = q * (1 + noise * rng.standard_normal(q.shape))
    n = len(z)
    return Atm(time=np.full(n, time), z=z.copy(), lon=np.full(n, lon), lat=np.full(n, lat),
               p=p, t=t, q=q, k=np.zeros((nw, n)))


def limb_obs(nd, tangent_heights, obsz=800.0, time=0.0, lon=0.0, lat=0.0) -> Obs:
    zt = np.asarray(tangent_heights, dtype=np.float64)
    n = len(zt)
    return Obs.geometry(np.full(n, time), np.full(n, obsz), np.full(n, lon), np.full(n, lat),
                        zt, np.full(n, lon), lat + limb_vplat(zt, obsz), nd)


def nadir_obs(nd, lats, obsz=705.0, time=0.0, lon=0.0, scan_deg=None) -> Obs:
    lats = np.asarray(lats, dtype=np.float64)
    n = len(lats)
    off = np.zeros(n) if scan_deg is None else np.asarray(scan_deg)
    return Obs.geometry(np.full(n, time), np.full(n, obsz), np.full(n, lon), lats,
                        np.zeros(n), np.full(n, lon), lats + off, nd)


# --------------------------------------------------------------------------
# packed batches of independent observations


@dataclass
class Batch:
    """Many independent observations, each with its own atmosphere and rays,
    packed level-major and ray-major (the C-ABI batch layout)."""

    nobs: int
    lev_off: np.ndarray  # int32 [nobs+1]
    time: np.ndarray     # per level
    z: np.ndarray
    lon: np.ndarray
    lat: np.ndarray
    p: np.ndarray
    t: np.ndarray
    q: np.ndarray        # [ng][L]
    k: np.ndarray        # [nw][L]
    scal: np.ndarray     # [nobs][nscal]
    ray_off: np.ndarray  # int32 [nobs+1]
    geo: np.ndarray      # [7][R]
    rad: np.ndarray      # [nd][R]  in: NaN mask; out: radiance
    tau: np.ndarray      # [nd][R]
    tp: np.ndarray       # [3][R]

    @property
    def nlev(self) -> int:
        return int(self.lev_off[-1])

    @property
    def nray(self) -> int:
        return int(self.ray_off[-1])

    def copy(self) -> "Batch":
        return Batch(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                        for k, v in self.__dict__.items()})

    def fresh_outputs(self) -> "Batch":
        b = self.copy()
        b.rad = np.where(np.isfinite(self.rad), 0.0, np.nan)
        b.tau = np.zeros_like(self.tau)
        b.tp = np.zeros_like(self.tp)
        return b

    def item(self, ctl: Ctl, i: int):
        """(Atm, Obs) of observation i."""
        l0, l1 = self.lev_off[i], self.lev_off[i + 1]
        r0, r1 = self.ray_off[i], self.ray_off[i + 1]
        atm = Atm(time=self.time[l0:l1].copy(), z=self.z[l0:l1].copy(),
                  lon=self.lon[l0:l1].copy(), lat=self.lat[l0:l1].copy(),
                  p=self.p[l0:l1].copy(), t=self.t[l0:l1].copy(),
                  q=self.q[:, l0:l1].copy(), k=self.k[:, l0:l1].copy())
        atm.set_scal(ctl, self.scal[i])
        g = self.geo[:, r0:r1]
        obs = Obs(*[g[j].copy() for j in range(7)], tpz=self.tp[0, r0:r1].copy(),
                  tplon=self.tp[1, r0:r1].copy(), tplat=self.tp[2, r0:r1].copy(),
                  rad=self.rad[:, r0:r1].copy(), tau=self.tau[:, r0:r1].copy())
        return atm, obs


def pack(ctl: Ctl, items) -> Batch:
    """Pack a list of (Atm, Obs) pairs into a Batch."""
    lev = np.zeros(len(items) + 1, np.int32)
    ray = np.zeros(len(items) + 1, np.int32)
    for i, (a, o) in enumerate(items):
        lev[i + 1] = lev[i] + a.np
        ray[i + 1] = ray[i] + o.nr
    cat = lambda f: np.concatenate([f(a, o) for a, o in items], axis=-1)
    return Batch(nobs=len(items), lev_off=lev,
                 time=cat(lambda a, o: a.time), z=cat(lambda a, o: a.z),
                 lon=cat(lambda a, o: a.lon), lat=cat(lambda a, o: a.lat),
                 p=cat(lambda a, o: a.p), t=cat(lambda a, o: a.t),
                 q=cat(lambda a, o: a.q.reshape(ctl.ng, -1)),
                 k=cat(lambda a, o: a.k.reshape(ctl.nw, -1)),
                 scal=np.stack([a.scal(ctl) for a, o in items]),
                 ray_off=ray, geo=cat(lambda a, o: o.geo()),
                 rad=cat(lambda a, o: o.rad), tau=cat(lambda a, o: o.tau),
                 tp=cat(lambda a, o: np.stack([o.tpz, o.tplon, o.tplat])))


# --------------------------------------------------------------------------
# the benchmark configurations


@dataclass
class Workload:
    name: str
    ctl: Ctl
    tables: Tables
    filters: list
    batch: Batch
    ret: Optional[Ret] = None
    notes: Dict[str, object] = field(default_factory=dict)


def config_limb_ega(seed=1, n_rays=10, formod=1) -> Workload:
    """Limb EGA: 81 levels (0-80 km), 10 rays with tangent heights 10-40 km
    from 800 km, 3 channels, CO2 + H2O, +-2% seeded noise."""
    ctl = Ctl(emitter=["CO2", "H2O"], nu=[667.78, 792.0, 832.0], formod=formod)
    rng = np.random.default_rng(seed)
    z = np.arange(0.0, 81.0)
    atm = profile(ctl.emitter, z, rng=rng, noise=0.02)
    atm.t = np.where(z <= 11, 288.0 - 6.5 * z, atm.t)
    obs = limb_obs(ctl.nd, np.linspace(10.0, 40.0, n_rays))
    tbl = make_tables(ctl, seed + 100)
    return Workload("limb_ega_81lev_10rays_3ch_2gas", ctl, tbl, make_filters(ctl),
                    pack(ctl, [(atm, obs)]))


def config_nadir(nobs, seed=2, nd=100, nlev=101, ztop=100.0, emitters=("CO2", "H2O", "O3", "CH4", "N2O"),
                 numin=650.0, numax=2400.0, formod=1, obsz=705.0) -> Workload:
    """Batched nadir: `nobs` profiles on 0-ztop km, one nadir ray each from
    705 km with a small scan angle, `nd` channels, seeded +-5 K temperature and
    +-20 % gas perturbations of the standard atmosphere (vectorised)."""
    ctl = Ctl(emitter=list(emitters), nu=np.linspace(numin, numax, nd), formod=formod)
    rng = np.random.default_rng(seed)
    z = np.linspace(0.0, ztop, nlev)
    t0 = std_temperature(z)
    p0 = hydrostatic_pressure(z, t0)
    q0 = np.stack([std_vmr(e, z) for e in ctl.emitter])
    off = rng.uniform(-2.5, 2.5, nobs)
    amp = rng.uniform(-2.5, 2.5, nobs)
    ph = rng.uniform(0, 6.3, nobs)
    dq = 1 + rng.uniform(-0.2, 0.2, (nobs, ctl.ng))
    lat = rng.uniform(-60, 60, nobs)
    lon = rng.uniform(-180, 180, nobs)
    scan = rng.uniform(-3, 3, nobs)
    t = t0[None, :] + off[:, None] + amp[:, None] * np.sin(z[None, :] / 15.0 + ph[:, None])
    q = q0[None, :, :] * dq[:, :, None]                     # [nobs, ng, nlev]
    L = nobs * nlev
    time = np.repeat(np.arange(nobs, dtype=np.float64), nlev)
    nscal = 5 + ctl.ncl + ctl.nsf
    b = Batch(nobs=nobs, lev_off=(np.arange(nobs + 1) * nlev).astype(np.int32),
              time=time, z=np.tile(z, nobs), lon=np.repeat(lon, nlev), lat=np.repeat(lat, nlev),
              p=np.tile(p0, nobs), t=t.reshape(-1), q=q.transpose(1, 0, 2).reshape(ctl.ng, L).copy(),
              k=np.zeros((ctl.nw, L)), scal=np.zeros((nobs, nscal)),
              ray_off=np.arange(nobs + 1).astype(np.int32),
              geo=np.stack([np.arange(nobs, dtype=np.float64), np.full(nobs, obsz), lon, lat,
                            np.zeros(nobs), lon, lat + scan]),
              rad=np.zeros((nd, nobs)), tau=np.zeros((nd, nobs)), tp=np.zeros((3, nobs)))
    return Workload("nadir_%dobs_%dlev_%dch_%dgas" % (nobs, nlev, nd, ctl.ng), ctl,
                    make_tables(ctl, seed + 100), make_filters(ctl), b)


def config_jacobian(nobs, seed=4) -> Workload:
    """FD Jacobian workload: nadir profiles, 81 levels on 0-80 km, 150
    channels on 650-2400 cm^-1, CO2 + H2O + O3 + CH4, state = T and the four
    gases on all levels (n = 405 state elements)."""
    w = config_nadir(nobs, seed=seed, nd=150, nlev=81, ztop=80.0,
                     emitters=("CO2", "H2O", "O3", "CH4"))
    w.ctl.rett_zmin, w.ctl.rett_zmax = 0.0, 80.0
    w.ctl.retq_zmin = np.zeros(w.ctl.ng)
    w.ctl.retq_zmax = np.full(w.ctl.ng, 80.0)
    w.name = "fd_jacobian_nadir_%dobs_81lev_150ch_4gas_n405" % nobs
    return w


def config_limb_cga(nobs, seed=3, nd=32, emitters=("CO2", "H2O", "O3"), raydz=0.5,
                    zmin_t=5.0, zmax_t=60.0, nlev=81, ztop=80.0) -> Workload:
    """Batched limb CGA: `nobs` single-ray observations with tangent heights
    uniform on [5, 60] km (uneven path lengths), `nd` channels."""
    ctl = Ctl(emitter=list(emitters), nu=np.linspace(650.0, 1400.0, nd), formod=0,
              raydz=raydz)
    rng = np.random.default_rng(seed)
    z = np.linspace(0.0, ztop, nlev)
    items = []
    for i in range(nobs):
        dt = rng.uniform(-3, 3)
        dq = 1 + rng.uniform(-0.2, 0.2, ctl.ng)
        atm = profile(ctl.emitter, z, dt=dt, dq=dq, time=float(i))
        obs = limb_obs(nd, [rng.uniform(zmin_t, zmax_t)], obsz=800.0, time=float(i))
        items.append((atm, obs))
    return Workload("limb_cga_%dobs_%dch_%dgas" % (nobs, nd, ctl.ng), ctl,
                    make_tables(ctl, seed + 100), make_filters(ctl), pack(ctl, items))


def retrieval_requests(ctl: Ctl, forward, n, seed, nlev=(21, 31), ztop=60.0,
                       kinds=("nadir", "limb"), nch=None, limb_rays=3, noise=2e-3,
                       dt=3.0, dq=0.2):
    """Retrieval requests of uneven size: (a-priori Atm, measured Obs) pairs.

    Request i has a level count uniform on ``nlev`` (0-ztop km), is nadir (one
    ray) or limb (``limb_rays`` tangent heights on 8-30 km) in turn from
    ``kinds``, and measures the first ``nch[i]`` channels (others NaN, all if
    ``nch`` is None).  The truth is the standard atmosphere with a seeded
    temperature offset (+-dt K) and gas factors (+-dq); the measurement is
    ``forward(truth batch)`` with multiplicative noise; the a priori is the
    unperturbed standard atmosphere."""
    rng = np.random.default_rng(seed)
    truths, obss, aprs = [], [], []
    for i in range(n):
        nl = int(rng.integers(nlev[0], nlev[1] + 1))
        z = np.linspace(0.0, ztop, nl)
        lat = float(rng.uniform(-60, 60))
        lon = float(rng.uniform(-180, 180))
        truths.append(profile(ctl.emitter, z, dt=float(rng.uniform(-dt, dt)),
                              dq=1 + rng.uniform(-dq, dq, ctl.ng), nw=ctl.nw, time=float(i),
                              lon=lon, lat=lat))
        aprs.append(profile(ctl.emitter, z, nw=ctl.nw, time=float(i), lon=lon, lat=lat))
        if kinds[i % len(kinds)] == "nadir":
            obs = nadir_obs(ctl.nd, [lat], time=float(i), lon=lon)
        else:
            obs = limb_obs(ctl.nd, np.sort(rng.uniform(8.0, 30.0, limb_rays)), time=float(i),
                           lon=lon, lat=lat)
        obss.append(obs)
    fw = forward(pack(ctl, list(zip(truths, obss))))
    items = []
    for i in range(n):
        _, o = fw.item(ctl, i)
        o.rad = o.rad * (1 + noise * rng.standard_normal(o.rad.shape))
        if nch is not None:
            o.rad[int(nch[i]):, :] = np.nan
        items.append((aprs[i], o))
    return items
