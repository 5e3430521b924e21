"""Emissivity tables read by the library from the reference's table files
(jgb_read_tables; read_tbl, jurassic.c:4949-5110) on the GPU.

The forward model of a context whose tables the library read from ASCII or
binary files equals, bit for bit and in both precisions, that of a context
given the same tables from the host mirror; a missing file leaves its table
empty in both.
"""
import copy

import numpy as np
import pytest

from jurassic_gb300 import native, synth
from jurassic_gb300.tables import write_tbl

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [1, 2])
def test_read_tables_forward_model(tmp_path, built_lib, fmt):
    w = synth.config_limb_ega(n_rays=6)
    ctl = copy.deepcopy(w.ctl)
    ctl.tblbase = str(tmp_path / "tbl")
    ctl.tblfmt = fmt
    tbl = copy.deepcopy(w.tables)
    tbl.np_[1, 1] = -1                       # no file for this table
    write_tbl(ctl, tbl)
    a = native.Context(ctl, tbl, w.filters)
    b = native.Context(ctl, None, w.filters)
    b.read_tables(ctl.tblbase, fmt, *tbl.u.shape[2:])
    for prec in (native.FP64, native.MIXED):
        ra = a.formod_batch(w.batch.fresh_outputs(), prec)
        rb = b.formod_batch(w.batch.fresh_outputs(), prec)
        assert np.all(np.isfinite(ra.rad))
        for k in ("rad", "tau", "tp"):
            assert np.array_equal(getattr(ra, k), getattr(rb, k), equal_nan=True), (prec, k)
