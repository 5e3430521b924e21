"""Emissivity look-up tables and filter functions on the host.

:class:`Tables` holds the reference's ragged table set (``tbl_t``,
src/jurassic.h:778-807) as dense arrays with runtime capacities:

  ``np[nd][ng]``, ``p[nd][ng][TP]``, ``nt[nd][ng][TP]``,
  ``t[nd][ng][TP][TT]``, ``nu[nd][ng][TP][TT]``,
  ``u``/``eps[nd][ng][TP][TT][TU]`` (float32, as in the reference).

File formats follow read_tbl / write_tbl (src/jurassic.c:4949-5110,
5810-5892): ASCII ``p T u eps`` lines (TBLFMT=1) or the binary record
``int np; double p[np]; {int nt; double t[nt]; {int nu; float u[nu];
float eps[nu]}}`` (TBLFMT=2), one file per (channel, emitter).
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np

from .model import Ctl, JurassicError


@dataclass
class Tables:
    np_: np.ndarray   # int32 [nd, ng]  (-1: table missing)
    p: np.ndarray     # float64 [nd, ng, TP]
    nt: np.ndarray    # int32 [nd, ng, TP]
    t: np.ndarray     # float64 [nd, ng, TP, TT]
    nu: np.ndarray    # int32 [nd, ng, TP, TT]
    u: np.ndarray     # float32 [nd, ng, TP, TT, TU]
    eps: np.ndarray   # float32 [nd, ng, TP, TT, TU]

    @property
    def shape(self):
        return self.u.shape

    @staticmethod
    def empty(nd, ng, tp=41, tt=30, tu=320) -> "Tables":
        return Tables(np_=np.full((nd, ng), -1, np.int32), p=np.zeros((nd, ng, tp)),
                      nt=np.zeros((nd, ng, tp), np.int32), t=np.zeros((nd, ng, tp, tt)),
                      nu=np.zeros((nd, ng, tp, tt), np.int32),
                      u=np.zeros((nd, ng, tp, tt, tu), np.float32),
                      eps=np.zeros((nd, ng, tp, tt, tu), np.float32))

    def nbytes(self) -> int:
        return int(self.u.nbytes + self.eps.nbytes)


def write_tbl(ctl: Ctl, tbl: Tables) -> None:
    """Write one table file per (channel, emitter) (write_tbl,
    src/jurassic.c:5810-5892) under ``ctl.tblbase``."""
    nd, ng = tbl.np_.shape
    for id in range(nd):
        for ig in range(ng):
            n = int(tbl.np_[id, ig])
            if n < 0:
                continue
            fn = ctl.table_filename(id, ig)
            if ctl.tblfmt == 2:
                with open(fn, "wb") as f:
                    f.write(np.int32(n).tobytes())
                    f.write(tbl.p[id, ig, :n].astype("<f8").tobytes())
                    for ip in range(n):
                        ntt = int(tbl.nt[id, ig, ip])
                        f.write(np.int32(ntt).tobytes())
                        f.write(tbl.t[id, ig, ip, :ntt].astype("<f8").tobytes())
                        for it in range(ntt):
                            nu = int(tbl.nu[id, ig, ip, it])
                            f.write(np.int32(nu).tobytes())
                            f.write(tbl.u[id, ig, ip, it, :nu].astype("<f4").tobytes())
                            f.write(tbl.eps[id, ig, ip, it, :nu].astype("<f4").tobytes())
            else:
                with open(fn, "w") as f:
                    f.write("# $1 = pressure [hPa]\n# $2 = temperature [K]\n"
                            "# $3 = column density [molecules/cm^2]\n# $4 = emissivity [-]\n")
                    for ip in range(n):
                        for it in range(int(tbl.nt[id, ig, ip])):
                            f.write("\n")
                            for iu in range(int(tbl.nu[id, ig, ip, it])):
                                f.write("%.17g %.17g %.9e %.9e\n" % (
                                    tbl.p[id, ig, ip], tbl.t[id, ig, ip, it],
                                    tbl.u[id, ig, ip, it, iu], tbl.eps[id, ig, ip, it, iu]))


UMIN, UMAX, EPSMIN, EPSMAX = 0.0, 1e30, 0.0, 1.0   # jurassic.h:264-339


def _read_ascii_table(fn, tp, tt, tu):
    """One ASCII table (read_tbl TBLFMT=1, src/jurassic.c:4991-5047): lines
    ``p T u eps``; points outside [UMIN, UMAX] x [EPSMIN, EPSMAX] are skipped;
    a new pressure or temperature opens a new block; within a block a point
    is appended only if both u and eps exceed the last appended point,
    otherwise it overwrites that point."""
    p = np.zeros(tp)
    nt = np.zeros(tp, np.int32)
    t = np.zeros((tp, tt))
    nu = np.zeros((tp, tt), np.int32)
    u = np.zeros((tp, tt, tu), np.float32)
    e = np.zeros((tp, tt, tu), np.float32)
    ip = it = iu = -1
    p_old = t_old = u_old = e_old = -999.0
    nrange = 0
    with open(fn) as f:
        for line in f:
            parts = line.split()
            if len(parts) < 4:
                continue
            try:
                press, temp, uu, eps = (float(v) for v in parts[:4])
            except ValueError:
                continue
            if uu < UMIN or uu > UMAX or eps < EPSMIN or eps > EPSMAX:
                nrange += 1
                continue
            if press != p_old:
                p_old = press
                ip += 1
                if ip >= tp:
                    raise JurassicError("Too many pressure levels!")
                it = -1
            if temp != t_old or it < 0:   # a level opens a row even at the last row's T
                t_old = temp
                it += 1
                if it >= tt:
                    raise JurassicError("Too many temperatures!")
                iu = -1
            if (eps > e_old and uu > u_old) or iu < 0:
                e_old, u_old = eps, uu
                iu += 1
                if iu >= tu:
                    raise JurassicError("Too many column densities!")
            p[ip] = press
            t[ip, it] = temp
            u[ip, it, iu] = np.float32(uu)
            e[ip, it, iu] = np.float32(eps)
            nt[ip] = it + 1
            nu[ip, it] = iu + 1
    return ip + 1, p, nt, t, nu, u, e, nrange


def _read_binary_table(fn, tp, tt, tu):
    """One binary table (read_tbl TBLFMT=2, src/jurassic.c:5050-5082)."""
    buf = open(fn, "rb").read()
    o = 0

    def take(dt, n):
        nonlocal o
        a = np.frombuffer(buf, dtype=dt, count=n, offset=o)
        o += a.nbytes
        return a

    n = int(take("<i4", 1)[0])
    if n > tp:
        raise JurassicError("Too many pressure levels!")
    p = np.zeros(tp)
    nt = np.zeros(tp, np.int32)
    t = np.zeros((tp, tt))
    nu = np.zeros((tp, tt), np.int32)
    u = np.zeros((tp, tt, tu), np.float32)
    e = np.zeros((tp, tt, tu), np.float32)
    p[:n] = take("<f8", n)
    for ip in range(n):
        ntt = int(take("<i4", 1)[0])
        if ntt > tt:
            raise JurassicError("Too many temperatures!")
        nt[ip] = ntt
        t[ip, :ntt] = take("<f8", ntt)
        for it in range(ntt):
            k = int(take("<i4", 1)[0])
            if k > tu:
                raise JurassicError("Too many column densities!")
            nu[ip, it] = k
            u[ip, it, :k] = take("<f4", k)
            e[ip, it, :k] = take("<f4", k)
    return n, p, nt, t, nu, u, e, 0


def read_tbl(ctl: Ctl, tp=41, tt=30, tu=320) -> Tables:
    """Read every (channel, emitter) table named by ``ctl.tblbase``,
    ``ctl.nu`` and ``ctl.emitter`` in format ``ctl.tblfmt`` (read_tbl,
    src/jurassic.c:4949-5110); a missing file leaves np = -1 (the reference
    warns and goes on).  Capacities tp x tt x tu play TBLNP/TBLNT/TBLNU."""
    if ctl.tblfmt not in (1, 2):
        raise JurassicError("Unknown look-up table format!")
    tbl = Tables.empty(ctl.nd, ctl.ng, tp, tt, tu)
    reader = _read_ascii_table if ctl.tblfmt == 1 else _read_binary_table
    for id in range(ctl.nd):
        for ig in range(ctl.ng):
            fn = ctl.table_filename(id, ig)
            if not os.path.exists(fn):
                continue
            n, p, nt, t, nu, u, e, _ = reader(fn, tp, tt, tu)
            tbl.np_[id, ig] = n
            tbl.p[id, ig], tbl.nt[id, ig], tbl.t[id, ig] = p, nt, t
            tbl.nu[id, ig], tbl.u[id, ig], tbl.eps[id, ig] = nu, u, e
    return tbl


def read_filter(path: str):
    """Two-column filter/shape file (read_shape, src/jurassic.c:4907-4945)."""
    xs, ys = [], []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if len(tok) >= 2:
                try:
                    x, y = float(tok[0]), float(tok[1])
                except ValueError:
                    continue
                xs.append(x)
                ys.append(y)
    if len(xs) < 2:
        raise JurassicError("Could not read any data!")
    return np.array(xs), np.array(ys)


def write_filter(path: str, fnu: np.ndarray, f: np.ndarray) -> None:
    """Shape file (write_shape, src/jurassic.c:5780-5806), full precision."""
    with open(path, "w") as fo:
        fo.write("# $1 = shape function x-value [-]\n# $2 = shape function y-value [-]\n\n")
        for a, b in zip(fnu, f):
            fo.write("%.17g %.17g\n" % (a, b))


def write_filters(ctl: Ctl, filters) -> None:
    for id in range(ctl.nd):
        fnu, f = filters[id]
        write_filter(ctl.filter_filename(id), fnu, f)


def read_filters(ctl: Ctl):
    return [read_filter(ctl.filter_filename(id)) for id in range(ctl.nd)]
