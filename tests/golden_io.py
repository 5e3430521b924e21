"""Load the golden fixtures of tests/golden/ into the host data model."""
import json
import os

import numpy as np

from jurassic_gb300.model import Atm, Ctl, Obs, Ret
from jurassic_gb300.tables import Tables

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def ctl_from(js):
    d = json.loads(str(js))
    return Ctl(**{k: (np.asarray(v) if isinstance(v, list) and k != "emitter" else v)
                  for k, v in d.items()})


def ret_from(js):
    d = json.loads(str(js))
    return Ret(**{k: (np.asarray(v) if isinstance(v, list) else v) for k, v in d.items()})


def tables_from(f):
    return Tables(np_=f["tbl_np"], p=f["tbl_p"], nt=f["tbl_nt"], t=f["tbl_t"], nu=f["tbl_nu"],
                  u=f["tbl_u"], eps=f["tbl_eps"])


def filters_from(f, nd):
    return [(f["filt%d_nu" % i], f["filt%d_f" % i]) for i in range(nd)]


def atm_from(f, prefix, ctl):
    a = Atm(time=f[prefix + "time"], z=f[prefix + "z"], lon=f[prefix + "lon"],
            lat=f[prefix + "lat"], p=f[prefix + "p"].copy(), t=f[prefix + "t"],
            q=f[prefix + "q"], k=f[prefix + "k"])
    a.set_scal(ctl, f[prefix + "scal"])
    return a


def obs_from(f, prefix, nd):
    g = f[prefix + "geo"]
    o = Obs.geometry(*g, nd=nd)
    o.rad = f[prefix + "rad"].copy()
    return o
