"""Host-side data model mirroring the reference's public structs and files.

* :class:`Ctl`  -- forward-model control parameters (``ctl_t``,
  src/jurassic.h:541-675) with :func:`scan_ctl` / :func:`read_ctl`
  semantics of src/jurassic.c:5114-5179 and 4547-4653 (``NAME = value``
  lines, ``NAME[i]`` / ``NAME[*]`` keys, argv overrides, defaults, an error
  for a missing key without default).
* :class:`Ret`  -- retrieval settings (``ret_t``, src/retrieval.c:32-112,
  read by ``read_ret``, src/retrieval.c:753-804).
* :class:`Atm`  -- atmosphere (``atm_t``, src/jurassic.h:488-538).
* :class:`Obs`  -- observation geometry and radiances (``obs_t``,
  src/jurassic.h:734-775); ``rad``/``tau`` are channel-major ``[nd][nr]``.

Dimensions are runtime sizes here (the reference fixes them with ``-D``
macros); arrays are numpy float64.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np


class JurassicError(RuntimeError):
    """Raised where the reference prints an error and exits (ERRMSG)."""


# --------------------------------------------------------------------------
# control file parsing


def scan_ctl(argv: Sequence[str], varname: str, arridx: int = -1,
             defvalue: str = "") -> str:
    """Value of a control parameter (scan_ctl, src/jurassic.c:5114-5179).

    ``argv[1]`` is the control file unless it starts with ``-``; later
    ``NAME value`` pairs in argv override the file.  Matching is
    case-insensitive on ``NAME`` or ``NAME[i]``/``NAME[*]`` for arrays.
    Returns the string value; use float() for numbers like the reference's
    ``atof`` return value.
    """
    if arridx >= 0:
        full1, full2 = "%s[%d]" % (varname, arridx), "%s[*]" % varname
    else:
        full1 = full2 = varname
    keys = (full1.lower(), full2.lower())
    rval = None
    if len(argv) > 1 and not argv[1].startswith("-"):
        try:
            with open(argv[1]) as f:
                for line in f:
                    tok = line.split()
                    if len(tok) >= 3 and tok[0].lower() in keys:
                        rval = tok[2]
                        break
        except OSError as e:
            raise JurassicError("Cannot open file!") from e
    for i in range(1, len(argv) - 1):
        if argv[i].lower() in keys:
            rval = argv[i + 1]
            break
    if rval is None:
        if defvalue:
            rval = defvalue
        else:
            raise JurassicError("Missing variable %s!" % full1)
    return rval


def _atof(s: str) -> float:
    """C atof: leading numeric prefix, 0.0 if none."""
    s = s.strip()
    best = 0.0
    for end in range(len(s), 0, -1):
        try:
            return float(s[:end])
        except ValueError:
            continue
    return best


EMITTER_KIND = {"CO2": 1, "H2O": 2}


@dataclass
class Ctl:
    """Forward-model control parameters (ctl_t, src/jurassic.h:541-675)."""

    emitter: List[str] = field(default_factory=list)
    nu: np.ndarray = field(default_factory=lambda: np.zeros(0))
    nw: int = 1
    window: np.ndarray = field(default_factory=lambda: np.zeros(0, dtype=np.int32))
    clnu: np.ndarray = field(default_factory=lambda: np.zeros(0))
    sfnu: np.ndarray = field(default_factory=lambda: np.zeros(0))
    sftype: int = 2
    sfsza: float = -999.0
    tblbase: str = "-"
    tblfmt: int = 1
    hydz: float = -999.0
    ctm_co2: int = 1
    ctm_h2o: int = 1
    ctm_n2: int = 1
    ctm_o2: int = 1
    refrac: int = 1
    rayds: float = 10.0
    raydz: float = 0.1
    fov: str = "-"
    retp_zmin: float = -999.0
    retp_zmax: float = -999.0
    rett_zmin: float = -999.0
    rett_zmax: float = -999.0
    retq_zmin: np.ndarray = field(default_factory=lambda: np.zeros(0))
    retq_zmax: np.ndarray = field(default_factory=lambda: np.zeros(0))
    retk_zmin: np.ndarray = field(default_factory=lambda: np.zeros(0))
    retk_zmax: np.ndarray = field(default_factory=lambda: np.zeros(0))
    ret_clz: int = 0
    ret_cldz: int = 0
    ret_clk: int = 0
    ret_sfz: int = 0
    ret_sfp: int = 0
    ret_sft: int = 0
    ret_sfeps: int = 0
    write_bbt: int = 0
    write_matrix: int = 0
    formod: int = 1

    @property
    def ng(self) -> int:
        return len(self.emitter)

    @property
    def nd(self) -> int:
        return int(len(self.nu))

    @property
    def ncl(self) -> int:
        return int(len(self.clnu))

    @property
    def nsf(self) -> int:
        return int(len(self.sfnu))

    def __post_init__(self):
        self.nu = np.asarray(self.nu, dtype=np.float64)
        if len(self.window) != len(self.nu):
            self.window = np.zeros(len(self.nu), dtype=np.int32)
        self.window = np.asarray(self.window, dtype=np.int32)
        self.clnu = np.asarray(self.clnu, dtype=np.float64)
        self.sfnu = np.asarray(self.sfnu, dtype=np.float64)
        for name in ("retq_zmin", "retq_zmax"):
            v = np.asarray(getattr(self, name), dtype=np.float64)
            if len(v) != self.ng:
                v = np.full(self.ng, -999.0)
            setattr(self, name, v)
        for name in ("retk_zmin", "retk_zmax"):
            v = np.asarray(getattr(self, name), dtype=np.float64)
            if len(v) != self.nw:
                v = np.full(self.nw, -999.0)
            setattr(self, name, v)

    def emitter_kinds(self) -> np.ndarray:
        return np.array([EMITTER_KIND.get(e.upper(), 0) for e in self.emitter],
                        dtype=np.int32)

    def find_emitter(self, name: str) -> int:
        """Index of an emitter, -1 if absent (find_emitter, jurassic.c:3013)."""
        for i, e in enumerate(self.emitter):
            if e.lower() == name.lower():
                return i
        return -1

    def table_filename(self, id: int, ig: int) -> str:
        """Table file of (channel, emitter) (read_tbl, jurassic.c:4968)."""
        return "%s_%.4f_%s.%s" % (self.tblbase, self.nu[id], self.emitter[ig],
                                  "tab" if self.tblfmt == 1 else "bin")

    def filter_filename(self, id: int) -> str:
        """Filter function file of a channel (init_srcfunc, jurassic.c:3649)."""
        return "%s_%.4f.filt" % (self.tblbase, self.nu[id])

    def to_lines(self) -> List[str]:
        """Control-file lines that read_ctl parses back into this object."""
        L = ["NG = %d" % self.ng]
        L += ["EMITTER[%d] = %s" % (i, e) for i, e in enumerate(self.emitter)]
        L += ["ND = %d" % self.nd]
        L += ["NU[%d] = %.17g" % (i, v) for i, v in enumerate(self.nu)]
        L += ["NW = %d" % self.nw]
        L += ["WINDOW[%d] = %d" % (i, w) for i, w in enumerate(self.window)]
        L += ["NCL = %d" % self.ncl] + ["CLNU[%d] = %.17g" % (i, v) for i, v in enumerate(self.clnu)]
        L += ["NSF = %d" % self.nsf] + ["SFNU[%d] = %.17g" % (i, v) for i, v in enumerate(self.sfnu)]
        L += ["SFTYPE = %d" % self.sftype, "SFSZA = %.17g" % self.sfsza,
              "TBLBASE = %s" % self.tblbase, "TBLFMT = %d" % self.tblfmt,
              "HYDZ = %.17g" % self.hydz,
              "CTM_CO2 = %d" % self.ctm_co2, "CTM_H2O = %d" % self.ctm_h2o,
              "CTM_N2 = %d" % self.ctm_n2, "CTM_O2 = %d" % self.ctm_o2,
              "REFRAC = %d" % self.refrac, "RAYDS = %.17g" % self.rayds,
              "RAYDZ = %.17g" % self.raydz, "FOV = %s" % self.fov,
              "RETP_ZMIN = %.17g" % self.retp_zmin, "RETP_ZMAX = %.17g" % self.retp_zmax,
              "RETT_ZMIN = %.17g" % self.rett_zmin, "RETT_ZMAX = %.17g" % self.rett_zmax]
        for i in range(self.ng):
            L += ["RETQ_ZMIN[%d] = %.17g" % (i, self.retq_zmin[i]),
                  "RETQ_ZMAX[%d] = %.17g" % (i, self.retq_zmax[i])]
        for i in range(self.nw):
            L += ["RETK_ZMIN[%d] = %.17g" % (i, self.retk_zmin[i]),
                  "RETK_ZMAX[%d] = %.17g" % (i, self.retk_zmax[i])]
        L += ["RET_CLZ = %d" % self.ret_clz, "RET_CLDZ = %d" % self.ret_cldz,
              "RET_CLK = %d" % self.ret_clk, "RET_SFZ = %d" % self.ret_sfz,
              "RET_SFP = %d" % self.ret_sfp, "RET_SFT = %d" % self.ret_sft,
              "RET_SFEPS = %d" % self.ret_sfeps, "WRITE_BBT = %d" % self.write_bbt,
              "WRITE_MATRIX = %d" % self.write_matrix, "FORMOD = %d" % self.formod]
        return L


def read_ctl(argv: Sequence[str]) -> Ctl:
    """Parse control parameters (read_ctl, src/jurassic.c:4547-4653)."""
    def num(name, idx=-1, d=""):
        return _atof(scan_ctl(argv, name, idx, d))

    ng = int(num("NG", -1, "0"))
    if ng < 0:
        raise JurassicError("Set 0 <= NG <= MAX!")
    emitter = [scan_ctl(argv, "EMITTER", i, "") for i in range(ng)]
    nd = int(num("ND", -1, "0"))
    if nd < 0:
        raise JurassicError("Set 0 <= ND <= MAX!")
    nu = np.array([num("NU", i, "") for i in range(nd)])
    nw = int(num("NW", -1, "1"))
    if nw < 0:
        raise JurassicError("Set 0 <= NW <= MAX!")
    window = np.array([int(num("WINDOW", i, "0")) for i in range(nd)], dtype=np.int32)
    ncl = int(num("NCL", -1, "0"))
    if ncl < 0:
        raise JurassicError("Set 0 <= NCL <= MAX!")
    if ncl == 1:
        raise JurassicError("Set NCL > 1!")
    clnu = np.array([num("CLNU", i, "") for i in range(ncl)])
    nsf = int(num("NSF", -1, "0"))
    if nsf < 0:
        raise JurassicError("Set 0 <= NSF <= MAX!")
    if nsf == 1:
        raise JurassicError("Set NSF > 1!")
    sfnu = np.array([num("SFNU", i, "") for i in range(nsf)])
    sftype = int(num("SFTYPE", -1, "2"))
    if sftype < 0 or sftype > 3:
        raise JurassicError("Set 0 <= SFTYPE <= 3!")
    c = Ctl(emitter=emitter, nu=nu, nw=nw, window=window, clnu=clnu, sfnu=sfnu,
            sftype=sftype, sfsza=num("SFSZA", -1, "-999"),
            tblbase=scan_ctl(argv, "TBLBASE", -1, "-"),
            tblfmt=int(num("TBLFMT", -1, "1")), hydz=num("HYDZ", -1, "-999"),
            ctm_co2=int(num("CTM_CO2", -1, "1")), ctm_h2o=int(num("CTM_H2O", -1, "1")),
            ctm_n2=int(num("CTM_N2", -1, "1")), ctm_o2=int(num("CTM_O2", -1, "1")),
            refrac=int(num("REFRAC", -1, "1")), rayds=num("RAYDS", -1, "10"),
            raydz=num("RAYDZ", -1, "0.1"), fov=scan_ctl(argv, "FOV", -1, "-"),
            retp_zmin=num("RETP_ZMIN", -1, "-999"), retp_zmax=num("RETP_ZMAX", -1, "-999"),
            rett_zmin=num("RETT_ZMIN", -1, "-999"), rett_zmax=num("RETT_ZMAX", -1, "-999"),
            retq_zmin=np.array([num("RETQ_ZMIN", i, "-999") for i in range(ng)]),
            retq_zmax=np.array([num("RETQ_ZMAX", i, "-999") for i in range(ng)]),
            retk_zmin=np.array([num("RETK_ZMIN", i, "-999") for i in range(nw)]),
            retk_zmax=np.array([num("RETK_ZMAX", i, "-999") for i in range(nw)]),
            ret_clz=int(num("RET_CLZ", -1, "0")), ret_cldz=int(num("RET_CLDZ", -1, "0")),
            ret_clk=int(num("RET_CLK", -1, "0")), ret_sfz=int(num("RET_SFZ", -1, "0")),
            ret_sfp=int(num("RET_SFP", -1, "0")), ret_sft=int(num("RET_SFT", -1, "0")),
            ret_sfeps=int(num("RET_SFEPS", -1, "0")),
            write_bbt=int(num("WRITE_BBT", -1, "0")),
            write_matrix=int(num("WRITE_MATRIX", -1, "0")),
            formod=int(num("FORMOD", -1, "1")))
    return c


@dataclass
class Ret:
    """Retrieval settings (ret_t, src/retrieval.c:32-112)."""

    kernel_recomp: int = 3
    conv_itmax: int = 30
    conv_dmin: float = 0.1
    err_ana: int = 1
    err_formod: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_noise: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_press: float = 0.0
    err_press_cz: float = -999.0
    err_press_ch: float = -999.0
    err_temp: float = 0.0
    err_temp_cz: float = -999.0
    err_temp_ch: float = -999.0
    err_q: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_q_cz: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_q_ch: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_k: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_k_cz: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_k_ch: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_clz: float = 0.0
    err_cldz: float = 0.0
    err_clk: np.ndarray = field(default_factory=lambda: np.zeros(0))
    err_sfz: float = 0.0
    err_sfp: float = 0.0
    err_sft: float = 0.0
    err_sfeps: np.ndarray = field(default_factory=lambda: np.zeros(0))

    def sized(self, ctl: Ctl) -> "Ret":
        """Pad per-channel/emitter/window arrays to the control sizes."""
        def fit(v, n, d):
            v = np.asarray(v, dtype=np.float64)
            return v if len(v) == n else np.full(n, d)
        r = Ret(**self.__dict__)
        r.err_formod = fit(r.err_formod, ctl.nd, 0.0)
        r.err_noise = fit(r.err_noise, ctl.nd, 0.0)
        r.err_q = fit(r.err_q, ctl.ng, 0.0)
        r.err_q_cz = fit(r.err_q_cz, ctl.ng, -999.0)
        r.err_q_ch = fit(r.err_q_ch, ctl.ng, -999.0)
        r.err_k = fit(r.err_k, ctl.nw, 0.0)
        r.err_k_cz = fit(r.err_k_cz, ctl.nw, -999.0)
        r.err_k_ch = fit(r.err_k_ch, ctl.nw, -999.0)
        r.err_clk = fit(r.err_clk, ctl.ncl, 0.0)
        r.err_sfeps = fit(r.err_sfeps, ctl.nsf, 0.0)
        return r

    def to_lines(self, ctl: Ctl) -> List[str]:
        r = self.sized(ctl)
        L = ["KERNEL_RECOMP = %d" % r.kernel_recomp, "CONV_ITMAX = %d" % r.conv_itmax,
             "CONV_DMIN = %.17g" % r.conv_dmin, "ERR_ANA = %d" % r.err_ana]
        L += ["ERR_FORMOD[%d] = %.17g" % (i, v) for i, v in enumerate(r.err_formod)]
        L += ["ERR_NOISE[%d] = %.17g" % (i, v) for i, v in enumerate(r.err_noise)]
        L += ["ERR_PRESS = %.17g" % r.err_press, "ERR_PRESS_CZ = %.17g" % r.err_press_cz,
              "ERR_PRESS_CH = %.17g" % r.err_press_ch, "ERR_TEMP = %.17g" % r.err_temp,
              "ERR_TEMP_CZ = %.17g" % r.err_temp_cz, "ERR_TEMP_CH = %.17g" % r.err_temp_ch]
        for i in range(ctl.ng):
            L += ["ERR_Q[%d] = %.17g" % (i, r.err_q[i]), "ERR_Q_CZ[%d] = %.17g" % (i, r.err_q_cz[i]),
                  "ERR_Q_CH[%d] = %.17g" % (i, r.err_q_ch[i])]
        for i in range(ctl.nw):
            L += ["ERR_K[%d] = %.17g" % (i, r.err_k[i]), "ERR_K_CZ[%d] = %.17g" % (i, r.err_k_cz[i]),
                  "ERR_K_CH[%d] = %.17g" % (i, r.err_k_ch[i])]
        L += ["ERR_CLZ = %.17g" % r.err_clz, "ERR_CLDZ = %.17g" % r.err_cldz]
        L += ["ERR_CLK[%d] = %.17g" % (i, v) for i, v in enumerate(r.err_clk)]
        L += ["ERR_SFZ = %.17g" % r.err_sfz, "ERR_SFP = %.17g" % r.err_sfp,
              "ERR_SFT = %.17g" % r.err_sft]
        L += ["ERR_SFEPS[%d] = %.17g" % (i, v) for i, v in enumerate(r.err_sfeps)]
        return L


def read_ret(argv: Sequence[str], ctl: Ctl) -> Ret:
    """Retrieval settings (read_ret, src/retrieval.c:753-804)."""
    def num(name, idx=-1, d=""):
        return _atof(scan_ctl(argv, name, idx, d))
    return Ret(
        kernel_recomp=int(num("KERNEL_RECOMP", -1, "3")),
        conv_itmax=int(num("CONV_ITMAX", -1, "30")),
        conv_dmin=num("CONV_DMIN", -1, "0.1"),
        err_ana=int(num("ERR_ANA", -1, "1")),
        err_formod=np.array([num("ERR_FORMOD", i, "0") for i in range(ctl.nd)]),
        err_noise=np.array([num("ERR_NOISE", i, "0") for i in range(ctl.nd)]),
        err_press=num("ERR_PRESS", -1, "0"), err_press_cz=num("ERR_PRESS_CZ", -1, "-999"),
        err_press_ch=num("ERR_PRESS_CH", -1, "-999"), err_temp=num("ERR_TEMP", -1, "0"),
        err_temp_cz=num("ERR_TEMP_CZ", -1, "-999"), err_temp_ch=num("ERR_TEMP_CH", -1, "-999"),
        err_q=np.array([num("ERR_Q", i, "0") for i in range(ctl.ng)]),
        err_q_cz=np.array([num("ERR_Q_CZ", i, "-999") for i in range(ctl.ng)]),
        err_q_ch=np.array([num("ERR_Q_CH", i, "-999") for i in range(ctl.ng)]),
        err_k=np.array([num("ERR_K", i, "0") for i in range(ctl.nw)]),
        err_k_cz=np.array([num("ERR_K_CZ", i, "-999") for i in range(ctl.nw)]),
        err_k_ch=np.array([num("ERR_K_CH", i, "-999") for i in range(ctl.nw)]),
        err_clz=num("ERR_CLZ", -1, "0"), err_cldz=num("ERR_CLDZ", -1, "0"),
        err_clk=np.array([num("ERR_CLK", i, "0") for i in range(ctl.ncl)]),
        err_sfz=num("ERR_SFZ", -1, "0"), err_sfp=num("ERR_SFP", -1, "0"),
        err_sft=num("ERR_SFT", -1, "0"),
        err_sfeps=np.array([num("ERR_SFEPS", i, "0") for i in range(ctl.nsf)]))


# --------------------------------------------------------------------------
# atmosphere and observations


@dataclass
class Atm:
    """Atmospheric profile (atm_t, src/jurassic.h:488-538); q is [ng][np]."""

    time: np.ndarray
    z: np.ndarray
    lon: np.ndarray
    lat: np.ndarray
    p: np.ndarray
    t: np.ndarray
    q: np.ndarray
    k: np.ndarray
    clz: float = 0.0
    cldz: float = 0.0
    clk: np.ndarray = field(default_factory=lambda: np.zeros(0))
    sfz: float = 0.0
    sfp: float = 0.0
    sft: float = 0.0
    sfeps: np.ndarray = field(default_factory=lambda: np.zeros(0))

    @property
    def np(self) -> int:
        return int(len(self.z))

    def scal(self, ctl: Ctl) -> np.ndarray:
        """{clz, cldz, clk[ncl], sfz, sfp, sft, sfeps[nsf]} for the C layers."""
        clk = np.zeros(ctl.ncl) if len(self.clk) != ctl.ncl else self.clk
        sfe = np.ones(ctl.nsf) if len(self.sfeps) != ctl.nsf else self.sfeps
        return np.concatenate([[self.clz, self.cldz], clk, [self.sfz, self.sfp, self.sft],
                               sfe]).astype(np.float64)

    def set_scal(self, ctl: Ctl, s: np.ndarray) -> None:
        self.clz, self.cldz = float(s[0]), float(s[1])
        self.clk = np.array(s[2:2 + ctl.ncl])
        o = 2 + ctl.ncl
        self.sfz, self.sfp, self.sft = float(s[o]), float(s[o + 1]), float(s[o + 2])
        self.sfeps = np.array(s[o + 3:o + 3 + ctl.nsf])

    def copy(self) -> "Atm":
        return Atm(**{k: (v.copy() if isinstance(v, np.ndarray) else v)
                      for k, v in self.__dict__.items()})


@dataclass
class Obs:
    """Observation geometry and results (obs_t, src/jurassic.h:734-775)."""

    time: np.ndarray
    obsz: np.ndarray
    obslon: np.ndarray
    obslat: np.ndarray
    vpz: np.ndarray
    vplon: np.ndarray
    vplat: np.ndarray
    tpz: np.ndarray
    tplon: np.ndarray
    tplat: np.ndarray
    rad: np.ndarray  # [nd][nr]
    tau: np.ndarray  # [nd][nr]

    @property
    def nr(self) -> int:
        return int(len(self.time))

    @staticmethod
    def geometry(time, obsz, obslon, obslat, vpz, vplon, vplat, nd) -> "Obs":
        a = [np.asarray(v, dtype=np.float64).copy() for v in
             (time, obsz, obslon, obslat, vpz, vplon, vplat)]
        nr = len(a[0])
        return Obs(*a, tpz=np.zeros(nr), tplon=np.zeros(nr), tplat=np.zeros(nr),
                   rad=np.zeros((nd, nr)), tau=np.zeros((nd, nr)))

    def geo(self) -> np.ndarray:
        return np.stack([self.time, self.obsz, self.obslon, self.obslat,
                         self.vpz, self.vplon, self.vplat]).astype(np.float64)

    def copy(self) -> "Obs":
        return Obs(**{k: v.copy() for k, v in self.__dict__.items()})


def _path(dirname: Optional[str], filename: str) -> str:
    return os.path.join(dirname, filename) if dirname else filename


def read_atm(dirname: Optional[str], filename: str, ctl: Ctl) -> Atm:
    """Read an atmosphere file (read_atm, src/jurassic.c:4442-4543)."""
    rows, extra = [], None
    ncol = 6 + ctl.ng + ctl.nw
    with open(_path(dirname, filename)) as f:
        for line in f:
            tok = line.split()
            vals = []
            for t in tok:
                try:
                    vals.append(float(t))
                except ValueError:
                    break
            if len(vals) < ncol:
                continue
            if not rows:
                extra = vals[ncol:]
            rows.append(vals[:ncol])
    if not rows:
        raise JurassicError("Could not read any data!")
    a = np.array(rows)
    atm = Atm(time=a[:, 0].copy(), z=a[:, 1].copy(), lon=a[:, 2].copy(), lat=a[:, 3].copy(),
              p=a[:, 4].copy(), t=a[:, 5].copy(), q=a[:, 6:6 + ctl.ng].T.copy(),
              k=a[:, 6 + ctl.ng:ncol].T.copy())
    e = list(extra or [])
    if ctl.ncl > 0 and len(e) >= 2 + ctl.ncl:
        atm.clz, atm.cldz = e[0], e[1]
        atm.clk = np.array(e[2:2 + ctl.ncl])
        e = e[2 + ctl.ncl:]
    if ctl.nsf > 0 and len(e) >= 3 + ctl.nsf:
        atm.sfz, atm.sfp, atm.sft = e[0], e[1], e[2]
        atm.sfeps = np.array(e[3:3 + ctl.nsf])
    return atm


def write_atm(dirname: Optional[str], filename: str, ctl: Ctl, atm: Atm,
              full_precision: bool = True) -> None:
    """Write an atmosphere file in the reference column layout
    (write_atm, src/jurassic.c:5336-5450); full precision by default."""
    g = "%.17g" if full_precision else "%g"
    with open(_path(dirname, filename), "w") as f:
        f.write("# $1 = time (seconds since 2000-01-01T00:00Z)\n# $2 = altitude [km]\n"
                "# $3 = longitude [deg]\n# $4 = latitude [deg]\n# $5 = pressure [hPa]\n"
                "# $6 = temperature [K]\n")
        for ip in range(atm.np):
            if ip == 0 or atm.time[ip] != atm.time[ip - 1]:
                f.write("\n")
            cols = [("%.2f" if not full_precision else g) % atm.time[ip]]
            cols += [g % v for v in (atm.z[ip], atm.lon[ip], atm.lat[ip], atm.p[ip], atm.t[ip])]
            cols += [g % atm.q[ig][ip] for ig in range(ctl.ng)]
            cols += [g % atm.k[iw][ip] for iw in range(ctl.nw)]
            if ctl.ncl > 0:
                cols += [g % v for v in np.concatenate([[atm.clz, atm.cldz], atm.clk])]
            if ctl.nsf > 0:
                cols += [g % v for v in np.concatenate([[atm.sfz, atm.sfp, atm.sft], atm.sfeps])]
            f.write(" ".join(cols) + "\n")


def read_obs(dirname: Optional[str], filename: str, ctl: Ctl) -> Obs:
    """Read an observation file (read_obs, src/jurassic.c:4697-4794)."""
    rows = []
    ncol = 10 + 2 * ctl.nd
    with open(_path(dirname, filename)) as f:
        for line in f:
            vals = []
            for t in line.split():
                try:
                    vals.append(float(t))
                except ValueError:
                    break
            if len(vals) >= ncol:
                rows.append(vals[:ncol])
    if not rows:
        raise JurassicError("Could not read any data!")
    a = np.array(rows)
    return Obs(*[a[:, i].copy() for i in range(10)],
               rad=a[:, 10:10 + ctl.nd].T.copy(), tau=a[:, 10 + ctl.nd:ncol].T.copy())


def write_obs(dirname: Optional[str], filename: str, ctl: Ctl, obs: Obs,
              full_precision: bool = False) -> None:
    """Write an observation file (write_obs, src/jurassic.c:5670-5776);
    ``%g`` columns like the reference unless full_precision."""
    g = "%.17g" if full_precision else "%g"
    with open(_path(dirname, filename), "w") as f:
        f.write("# $1 = time (seconds since 2000-01-01T00:00Z)\n# $2 = observer altitude [km]\n"
                "# $3 = observer longitude [deg]\n# $4 = observer latitude [deg]\n"
                "# $5 = view point altitude [km]\n# $6 = view point longitude [deg]\n"
                "# $7 = view point latitude [deg]\n# $8 = tangent point altitude [km]\n"
                "# $9 = tangent point longitude [deg]\n# $10 = tangent point latitude [deg]\n")
        n = 10
        for id in range(ctl.nd):
            n += 1
            if ctl.write_bbt:
                f.write("# $%d = brightness temperature (%.4f cm^-1) [K]\n" % (n, ctl.nu[id]))
            else:
                f.write("# $%d = radiance (%.4f cm^-1) [W/(m^2 sr cm^-1)]\n" % (n, ctl.nu[id]))
        for id in range(ctl.nd):
            n += 1
            f.write("# $%d = transmittance (%.4f cm^-1) [-]\n" % (n, ctl.nu[id]))
        for ir in range(obs.nr):
            if ir == 0 or obs.time[ir] != obs.time[ir - 1]:
                f.write("\n")
            cols = [("%.2f" if not full_precision else g) % obs.time[ir]]
            cols += [g % v for v in (obs.obsz[ir], obs.obslon[ir], obs.obslat[ir], obs.vpz[ir],
                                     obs.vplon[ir], obs.vplat[ir], obs.tpz[ir], obs.tplon[ir],
                                     obs.tplat[ir])]
            cols += [g % obs.rad[id][ir] for id in range(ctl.nd)]
            cols += [g % obs.tau[id][ir] for id in range(ctl.nd)]
            f.write(" ".join(cols) + "\n")


def atm2x(ctl: Ctl, atm: Atm):
    """State vector of an atmosphere (atm2x, src/jurassic.c:29-83): p, T,
    q per emitter, k per window on the levels inside each RET* window, then
    the retrieved cloud and surface scalars.  Returns (x, kind) with kind the
    reference's index codes: 0 p, 1 T, 2+ig q, 2+ng+iw k, then cloud height,
    depth, extinctions, surface height, pressure, temperature, emissivities."""
    x, kind = [], []
    z = np.asarray(atm.z)
    ng, nw = ctl.ng, ctl.nw

    def window(lo, hi, vals, code):
        for ip in range(len(z)):
            if lo <= z[ip] <= hi:
                x.append(float(vals[ip]))
                kind.append(code)
    window(ctl.retp_zmin, ctl.retp_zmax, atm.p, 0)
    window(ctl.rett_zmin, ctl.rett_zmax, atm.t, 1)
    q = np.reshape(atm.q, (ng, -1))
    for ig in range(ng):
        window(ctl.retq_zmin[ig], ctl.retq_zmax[ig], q[ig], 2 + ig)
    k = np.reshape(atm.k, (nw, -1)) if nw else np.zeros((0, len(z)))
    for iw in range(nw):
        window(ctl.retk_zmin[iw], ctl.retk_zmax[iw], k[iw], 2 + ng + iw)
    s = atm.scal(ctl)
    o = 2 + ng + nw
    flags = [(ctl.ret_clz, [0], o), (ctl.ret_cldz, [1], o + 1),
             (ctl.ret_clk, list(range(2, 2 + ctl.ncl)), o + 2)]
    so = 2 + ctl.ncl
    flags += [(ctl.ret_sfz, [so], o + 2 + ctl.ncl), (ctl.ret_sfp, [so + 1], o + 3 + ctl.ncl),
              (ctl.ret_sft, [so + 2], o + 4 + ctl.ncl),
              (ctl.ret_sfeps, list(range(so + 3, so + 3 + ctl.nsf)), o + 5 + ctl.ncl)]
    for on, idx, code in flags:
        if on:
            for j, i in enumerate(idx):
                x.append(float(s[i]))
                kind.append(code + (j if len(idx) > 1 else 0))
    return np.array(x), np.array(kind, dtype=np.int64)


def fd_steps(ctl: Ctl, x, kind):
    """Perturbation step of every state element in kernel()
    (src/jurassic.c:4046-4068)."""
    ng, nw, ncl = ctl.ng, ctl.nw, ctl.ncl
    x = np.asarray(x, dtype=np.float64)
    h = np.empty_like(x)
    for j, (v, c) in enumerate(zip(x, kind)):
        o = 2 + ng + nw
        if c == 0:
            h[j] = max(abs(0.01 * v), 1e-7)
        elif c == 1:
            h[j] = 1.0
        elif c < 2 + ng:
            h[j] = max(abs(0.01 * v), 1e-15)
        elif c < o:
            h[j] = 1e-4
        elif c in (o, o + 1):
            h[j] = 1.0
        elif c < o + 2 + ncl:
            h[j] = 1e-4
        elif c == o + 2 + ncl:
            h[j] = 0.1
        elif c == o + 3 + ncl:
            h[j] = 10.0
        elif c == o + 4 + ncl:
            h[j] = 1.0
        else:
            h[j] = 1e-2
    return h


def obs2y(rad):
    """Measurement vector (obs2y, src/jurassic.c:4174-4197): ray-major,
    finite radiances only."""
    rad = np.asarray(rad)
    return np.array([v for col in rad.T for v in col if np.isfinite(v)])


def brightness(rad, nu):
    """Brightness temperature (BRIGHT, src/jurassic.h:126-127)."""
    C1, C2 = 1.19104259e-8, 1.43877506
    nu = np.asarray(nu, dtype=np.float64)
    return C2 * nu / np.log1p(C1 * nu ** 3 / np.asarray(rad, dtype=np.float64))


def planck(t, nu):
    """Planck radiance (PLANCK, src/jurassic.h:183-184)."""
    C1, C2 = 1.19104259e-8, 1.43877506
    nu = np.asarray(nu, dtype=np.float64)
    return C1 * nu ** 3 / np.expm1(C2 * nu / np.asarray(t, dtype=np.float64))


def limb_vplat(z, obsz, re=6367.421):
    """Latitude of a limb view point seen from (0, 0, obsz) (limb.c:54)."""
    return 180.0 / math.pi * np.arccos((re + np.asarray(z)) / (re + obsz))
