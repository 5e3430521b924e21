"""Run the reference build (oracle/_ref/libjref_<tag>.so) on given inputs.

TEST INFRASTRUCTURE ONLY.  The reference keeps process-global tables, so
every call runs in a fresh ``spawn``-ed process: the control file, the
binary emissivity tables and the filter files are written to a scratch
directory, the child reads them through the reference's own read_ctl /
read_tbl / init_srcfunc and returns full-precision results.
"""
from __future__ import annotations

import ctypes as C
import multiprocessing as mp
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def lib_path(tag="std"):
    return os.path.join(REF_DIR, "libjref_%s.so" % tag)


def source_dir():
    """The reference tree as the build recipe resolves it ($JURASSIC_REF_DIR,
    else the build container's mount), or None where there is none (the GPU
    box)."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), "--where"],
                       capture_output=True, text=True)
    return r.stdout.strip() if r.returncode == 0 and r.stdout.strip() else None


def available(tag="std"):
    return os.path.exists(lib_path(tag))


def build(tag="std", flags=()):
    """Build the reference oracle if its sources are present (this container)."""
    script = os.path.join(HERE, "build_ref.sh")
    r = subprocess.run(["bash", script, tag] + list(flags), capture_output=True, text=True)
    return r.returncode == 0


def write_inputs(workdir, ctl, tables, filters, ret=None, extra_lines=(), fov=None):
    """Files the reference reads: ctl, TBLFMT=2 tables, .filt filters and,
    with fov = (dz, w), the FOV shape file."""
    from jurassic_gb300.tables import write_filter, write_filters, write_tbl
    import copy
    c = copy.copy(ctl)
    c.tblbase = os.path.join(workdir, "tbl")
    c.tblfmt = ctl.tblfmt if ctl.tblfmt in (1, 2) else 2
    if fov is not None:
        c.fov = os.path.join(workdir, "fov.dat")
        write_filter(c.fov, np.asarray(fov[0], float), np.asarray(fov[1], float))
    write_tbl(c, tables)
    write_filters(c, filters)
    lines = c.to_lines()
    if ret is not None:
        lines += ret.to_lines(c)
    lines += list(extra_lines)
    path = os.path.join(workdir, "run.ctl")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def _child(args):
    tag, ctlfile, ng, nd, nw, ncl, nsf, jobs = args
    L = C.CDLL(lib_path(tag))
    dp = C.POINTER(C.c_double)
    argv = (C.c_char_p * 2)(b"jref", ctlfile.encode())
    L.jref_init(2, argv)
    dims = np.zeros(8, np.int32)
    L.jref_dims(dims.ctypes.data_as(C.POINTER(C.c_int)))
    out = []
    for job in jobs:
        kind, atm, geo, rad = job["kind"], job["atm"], job["geo"], job["rad"]
        npl = len(atm["z"])
        nr = geo.shape[1]
        if npl > dims[2] or nr > dims[3] or nd > dims[0] or ng > dims[1]:
            raise RuntimeError("reference build too small: dims=%s" % dims)
        keep = [np.ascontiguousarray(atm[k], dtype=np.float64) for k in
                ("time", "z", "lon", "lat", "p", "t", "q", "k", "scal")]
        L.jref_set_atm(npl, *[a.ctypes.data_as(dp) for a in keep])
        g = np.ascontiguousarray(geo, np.float64)
        r = np.ascontiguousarray(rad, np.float64)
        L.jref_set_obs(nr, g.ctypes.data_as(dp), r.ctypes.data_as(dp))
        if kind == "formod":
            L.jref_formod()
            tp = np.zeros((3, nr))
            ro = np.zeros((nd, nr))
            to = np.zeros((nd, nr))
            L.jref_get_obs(tp.ctypes.data_as(dp), ro.ctypes.data_as(dp), to.ctypes.data_as(dp))
            pa = np.zeros(npl)
            ta = np.zeros(npl)
            qa = np.zeros(ng * npl)
            ka = np.zeros(max(nw * npl, 1))
            sa = np.zeros(len(atm["scal"]))
            L.jref_get_atm(*[a.ctypes.data_as(dp) for a in (pa, ta, qa, ka, sa)])
            out.append(dict(rad=ro, tau=to, tp=tp, p=pa))
        elif kind == "raytrace":
            w = 7 + 5 * ng + 2 * nd
            res = []
            for ir in range(nr):
                buf = np.zeros((8192, w))
                tp = np.zeros(3)
                n = L.jref_raytrace(ir, 8192, buf.ctypes.data_as(dp), tp.ctypes.data_as(dp))
                res.append((buf[:n].copy(), tp))
            out.append(res)
        elif kind == "kernel":
            maxm, maxn = job["maxm"], job["maxn"]
            K = np.zeros(maxm * maxn)
            mn = np.zeros(2, np.int32)
            rc = L.jref_kernel(K.ctypes.data_as(dp), maxm, maxn,
                               mn.ctypes.data_as(C.POINTER(C.c_int)))
            if rc:
                raise RuntimeError("jref_kernel failed: m,n=%s" % mn)
            m, n = int(mn[0]), int(mn[1])
            out.append(K[:m * n].reshape(m, n))
        elif kind == "retrieval":
            maxn = job["maxn"]
            x = np.zeros(maxn)
            cov = np.zeros(maxn * maxn)
            costs = np.zeros(64)
            info = np.zeros(4, np.int32)
            rc = L.jref_retrieval(job["dir"].encode(), x.ctypes.data_as(dp), maxn,
                                  cov.ctypes.data_as(dp), costs.ctypes.data_as(dp), 64,
                                  info.ctypes.data_as(C.POINTER(C.c_int)))
            if rc:
                raise RuntimeError("jref_retrieval failed")
            n, m = int(info[0]), int(info[1])
            r = dict(x=x[:n], cov=cov[:n * n].reshape(n, n) if info[3] else None,
                     costs=costs[:info[2]], n=n, m=m)
            gain, avk, ana = np.zeros(n * m), np.zeros(n * n), np.zeros(5 * n)
            if hasattr(L, "jref_retrieval_ana") and L.jref_retrieval_ana(
                    gain.ctypes.data_as(dp), avk.ctypes.data_as(dp), ana.ctypes.data_as(dp),
                    n, m) == 0:
                r.update(gain=gain.reshape(n, m), avk=avk.reshape(n, n),
                         **{k: ana[i * n:(i + 1) * n] for i, k in enumerate(
                             ("err_total", "err_noise", "err_formod", "cont", "res"))})
            out.append(r)
        else:
            raise ValueError(kind)
    return out


def _atm_dict(ctl, atm):
    return dict(time=atm.time, z=atm.z, lon=atm.lon, lat=atm.lat, p=atm.p, t=atm.t,
                q=np.asarray(atm.q).reshape(-1), k=np.asarray(atm.k).reshape(-1),
                scal=atm.scal(ctl))


def run(ctl, tables, filters, jobs, tag="std", ret=None, workdir=None, timeout=3600, fov=None,
        post_write=None):
    """Run jobs [(kind, atm, obs, extra), ...] through the reference.

    kind in {"formod", "raytrace", "kernel", "retrieval"}.  Returns one result
    per job.
    """
    own = workdir is None
    tmp = tempfile.mkdtemp(prefix="jref_") if own else workdir
    ctlfile = write_inputs(tmp, ctl, tables, filters, ret=ret, fov=fov)
    if post_write is not None:      # e.g. rewrite table files before the reference reads them
        post_write(tmp)
    js = []
    for kind, atm, obs, extra in jobs:
        j = dict(kind=kind, atm=_atm_dict(ctl, atm), geo=obs.geo(), rad=obs.rad)
        j.update(extra or {})
        if kind == "retrieval":
            d = os.path.join(tmp, "ret%d" % len(js))
            os.makedirs(d, exist_ok=True)
            j["dir"] = d
        js.append(j)
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        res = pool.apply_async(_child, ((tag, ctlfile, ctl.ng, ctl.nd, ctl.nw, ctl.ncl,
                                         ctl.nsf, js),))
        return res.get(timeout)
