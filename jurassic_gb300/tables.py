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
from typing import Optional

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
