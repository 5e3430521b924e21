"""Host logic: control-file parsing (scan_ctl/read_ctl semantics), file
formats, table writer/reader round trip, batch packing."""
import os

import numpy as np
import pytest

from jurassic_gb300 import synth
from jurassic_gb300.model import (JurassicError, read_atm, read_ctl, read_obs, read_ret,
                                  scan_ctl, write_atm, write_obs)
from jurassic_gb300.tables import read_filter, write_filter, write_tbl


def test_scan_ctl_semantics(tmp_path):
    f = tmp_path / "a.ctl"
    f.write_text("NG = 2\nEMITTER[0] = CO2\nemitter[*] = H2O\nND = 1\nNU[0] = 792.0\n"
                 "RAYDZ = 0.5\n")
    argv = ["prog", str(f), "RAYDZ", "0.25"]
    assert scan_ctl(argv, "EMITTER", 0) == "CO2"        # exact index wins first match
    assert scan_ctl(argv, "EMITTER", 1) == "H2O"        # NAME[*] applies to every index
    assert scan_ctl(argv, "raydz") == "0.25"            # argv overrides, case-insensitive
    assert scan_ctl(argv, "RAYDS", -1, "10") == "10"   # default
    with pytest.raises(JurassicError):
        scan_ctl(argv, "MISSING")                      # no default -> error
    ctl = read_ctl(argv)
    assert ctl.emitter == ["CO2", "H2O"] and ctl.nd == 1 and ctl.raydz == 0.25
    assert ctl.formod == 1 and ctl.ctm_co2 == 1 and ctl.sftype == 2  # reference defaults


def test_read_ctl_errors(tmp_path):
    f = tmp_path / "b.ctl"
    f.write_text("NCL = 1\n")
    with pytest.raises(JurassicError):
        read_ctl(["p", str(f)])
    f.write_text("SFTYPE = 4\n")
    with pytest.raises(JurassicError):
        read_ctl(["p", str(f)])


def test_ctl_roundtrip(tmp_path):
    w = synth.config_limb_ega()
    f = tmp_path / "c.ctl"
    f.write_text("\n".join(w.ctl.to_lines()) + "\n")
    c2 = read_ctl(["p", str(f)])
    assert c2.emitter == w.ctl.emitter
    assert np.array_equal(c2.nu, w.ctl.nu)
    assert c2.raydz == w.ctl.raydz and c2.formod == w.ctl.formod


def test_atm_obs_file_roundtrip(tmp_path):
    w = synth.config_limb_ega()
    atm, obs = w.batch.item(w.ctl, 0)
    write_atm(str(tmp_path), "atm.tab", w.ctl, atm)
    a2 = read_atm(str(tmp_path), "atm.tab", w.ctl)
    assert np.array_equal(a2.p, atm.p) and np.array_equal(a2.q, atm.q)
    obs.rad[:] = 0.5
    write_obs(str(tmp_path), "obs.tab", w.ctl, obs, full_precision=True)
    o2 = read_obs(str(tmp_path), "obs.tab", w.ctl)
    assert np.array_equal(o2.vplat, obs.vplat) and np.array_equal(o2.rad, obs.rad)


def test_binary_table_layout(tmp_path):
    """TBLFMT=2 record layout of read_tbl/write_tbl (jurassic.c:5030-5084)."""
    w = synth.config_limb_ega()
    tbl = synth.make_tables(w.ctl, 3, tp=32, tt=4, tu=40)
    w.ctl.tblbase = str(tmp_path / "t")
    w.ctl.tblfmt = 2
    write_tbl(w.ctl, tbl)
    raw = open(w.ctl.table_filename(0, 0), "rb").read()
    np_ = np.frombuffer(raw[:4], "<i4")[0]
    assert np_ == 32
    p = np.frombuffer(raw[4:4 + 8 * 32], "<f8")
    assert np.array_equal(p, tbl.p[0, 0, :32])
    nt = np.frombuffer(raw[4 + 256:4 + 256 + 4], "<i4")[0]
    assert nt == 4


def test_filter_roundtrip(tmp_path):
    fnu, f = np.linspace(700, 701, 11), np.linspace(0, 1, 11)
    write_filter(str(tmp_path / "x.filt"), fnu, f)
    a, b = read_filter(str(tmp_path / "x.filt"))
    assert np.array_equal(a, fnu) and np.array_equal(b, f)


def test_batch_pack_item_roundtrip():
    w = synth.config_nadir(5, nd=4, nlev=21, ztop=20.0)
    b = w.batch
    assert b.nobs == 5 and b.nray == 5 and b.nlev == 5 * 21
    atm, obs = b.item(w.ctl, 3)
    assert atm.np == 21 and obs.nr == 1
    b2 = synth.pack(w.ctl, [b.item(w.ctl, i) for i in range(5)])
    for k in ("z", "p", "t", "q", "geo", "scal"):
        assert np.array_equal(getattr(b2, k), getattr(b, k))


def test_read_ret_defaults(tmp_path):
    f = tmp_path / "r.ctl"
    f.write_text("NG = 1\nEMITTER[0] = CO2\nND = 2\nNU[0] = 700\nNU[1] = 710\n"
                 "ERR_NOISE[*] = 1e-4\nERR_TEMP = 2\n")
    argv = ["p", str(f)]
    ctl = read_ctl(argv)
    r = read_ret(argv, ctl)
    assert r.kernel_recomp == 3 and r.conv_itmax == 30 and r.conv_dmin == 0.1
    assert np.array_equal(r.err_noise, [1e-4, 1e-4]) and r.err_temp == 2.0


# ---------------------------------------------------------------------------
# emissivity table files (read_tbl / write_tbl, src/jurassic.c:4949-5110,
# 5810-5892)

@pytest.mark.parametrize("fmt", [1, 2])
def test_table_files_round_trip(tmp_path, fmt):
    import copy
    from jurassic_gb300 import synth
    from jurassic_gb300.tables import read_tbl, write_tbl
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.tblbase = str(tmp_path / "tbl")
    ctl.tblfmt = fmt
    tbl = synth.make_tables(ctl, 3, tp=12, tt=5, tu=40)
    tbl.np_[1, 0] = -1                       # missing file
    write_tbl(ctl, tbl)
    back = read_tbl(ctl, 12, 5, 40)
    assert np.array_equal(back.np_, tbl.np_)
    for id in range(ctl.nd):
        for ig in range(ctl.ng):
            n = int(tbl.np_[id, ig])
            if n < 0:
                continue
            assert np.array_equal(back.p[id, ig, :n], tbl.p[id, ig, :n])
            assert np.array_equal(back.nt[id, ig, :n], tbl.nt[id, ig, :n])
            for ip in range(n):
                for it in range(int(tbl.nt[id, ig, ip])):
                    k = int(tbl.nu[id, ig, ip, it])
                    assert back.nu[id, ig, ip, it] == k
                    assert back.t[id, ig, ip, it] == tbl.t[id, ig, ip, it]
                    assert np.array_equal(back.u[id, ig, ip, it, :k], tbl.u[id, ig, ip, it, :k])
                    assert np.array_equal(back.eps[id, ig, ip, it, :k], tbl.eps[id, ig, ip, it, :k])


def test_ascii_tables_read_like_the_reference(tmp_path, built_oracle):
    """ASCII table files with skipped and folded lines: read by read_tbl here
    and by the reference; the oracle's forward model with the tables read
    here equals the reference's with the tables it read."""
    import golden_io as G
    from jurassic_gb300.tables import read_tbl
    from oracle import oracle
    f = G.load("ref_tbl_ascii.npz")
    ctl = G.ctl_from(f["ctl"])
    ctl.tblbase = str(tmp_path / "tbl")
    for id in range(ctl.nd):
        for ig in range(ctl.ng):
            with open(ctl.table_filename(id, ig), "wb") as fo:
                fo.write(f["tbl_%d_%d" % (id, ig)].tobytes())
    tbl = read_tbl(ctl, 32, 6, 64)
    ora = oracle.Oracle(ctl, tbl, G.filters_from(f, ctl.nd))
    atm = G.atm_from(f, "atm_", ctl)
    obs = G.obs_from(f, "obs_", ctl.nd)
    rad, tau, tp, _ = ora.formod(atm, obs)
    assert np.max(np.abs(rad - f["rad"]) / np.abs(f["rad"])) <= 1e-12
    assert np.max(np.abs(tau - f["tau"])) <= 1e-14
    # the folded lines changed the tables: they differ from the unmangled set
    orig = G.tables_from(f)
    assert not np.array_equal(tbl.u, orig.u)


# ---------------------------------------------------------------------------
# the library's own table-file reader and writer (jgb_read_table_file,
# jgb_write_table_file): host functions, no device work

def _c_read(L, path, fmt, tp, tt, tu):
    import ctypes as C
    p = np.zeros(tp)
    nt = np.zeros(tp, np.int32)
    t = np.zeros((tp, tt))
    nu = np.zeros((tp, tt), np.int32)
    u = np.zeros((tp, tt, tu), np.float32)
    e = np.zeros((tp, tt, tu), np.float32)
    n = C.c_int(-7)
    ptr = lambda a, ty: a.ctypes.data_as(C.POINTER(ty))
    rc = L.jgb_read_table_file(str(path).encode(), fmt, tp, tt, tu, C.byref(n),
                               ptr(p, C.c_double), ptr(nt, C.c_int), ptr(t, C.c_double),
                               ptr(nu, C.c_int), ptr(u, C.c_float), ptr(e, C.c_float))
    return rc, n.value, p, nt, t, nu, u, e


def _c_write(L, path, fmt, tbl, id, ig):
    import ctypes as C
    tp, tt, tu = tbl.u.shape[2:]
    keep = [np.ascontiguousarray(a) for a in (tbl.p[id, ig], tbl.nt[id, ig], tbl.t[id, ig],
                                              tbl.nu[id, ig], tbl.u[id, ig], tbl.eps[id, ig])]
    return L.jgb_write_table_file(str(path).encode(), fmt, int(tbl.np_[id, ig]),
                                  keep[0].ctypes.data_as(C.POINTER(C.c_double)),
                                  keep[1].ctypes.data_as(C.POINTER(C.c_int)),
                                  keep[2].ctypes.data_as(C.POINTER(C.c_double)),
                                  keep[3].ctypes.data_as(C.POINTER(C.c_int)),
                                  keep[4].ctypes.data_as(C.POINTER(C.c_float)),
                                  keep[5].ctypes.data_as(C.POINTER(C.c_float)), tt, tu)


def _same_table(got, tbl, id, ig):
    rc, n, p, nt, t, nu, u, e = got
    assert rc == 0 and n == tbl.np_[id, ig]
    assert np.array_equal(p, tbl.p[id, ig]) and np.array_equal(nt, tbl.nt[id, ig])
    assert np.array_equal(t, tbl.t[id, ig]) and np.array_equal(nu, tbl.nu[id, ig])
    assert np.array_equal(u, tbl.u[id, ig]) and np.array_equal(e, tbl.eps[id, ig])


@pytest.mark.parametrize("fmt", [1, 2])
def test_library_table_files_match_host_mirror(tmp_path, built_lib, fmt):
    """Files written by the host mirror read by the library equal the host
    mirror's reading; the library writes the same bytes; binary -> ASCII ->
    binary through the library restores every value (tblfmt conversion)."""
    import copy
    from jurassic_gb300 import native, synth
    from jurassic_gb300.tables import read_tbl, write_tbl
    L = native.load()
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.tblbase = str(tmp_path / "tbl")
    ctl.tblfmt = fmt
    tbl = synth.make_tables(ctl, 5, tp=12, tt=5, tu=40)
    write_tbl(ctl, tbl)
    back = read_tbl(ctl, 12, 5, 40)
    for id in range(ctl.nd):
        for ig in range(ctl.ng):
            fn = ctl.table_filename(id, ig)
            _same_table(_c_read(L, fn, fmt, 12, 5, 40), back, id, ig)
            out = tmp_path / ("c_%d_%d" % (id, ig))
            assert _c_write(L, out, fmt, tbl, id, ig) == 0
            assert out.read_bytes() == open(fn, "rb").read()
            other = tmp_path / ("x_%d_%d" % (id, ig))
            assert _c_write(L, other, 3 - fmt, tbl, id, ig) == 0
            _same_table(_c_read(L, other, 3 - fmt, 12, 5, 40), back, id, ig)


def test_library_reads_reference_ascii_tables(tmp_path, built_lib):
    """The ASCII table files with skipped and folded lines that the reference
    read (golden fixture): the library reads the same tables as the host
    mirror, which the oracle pins to the reference's forward model."""
    import golden_io as G
    from jurassic_gb300 import native
    from jurassic_gb300.tables import read_tbl
    L = native.load()
    f = G.load("ref_tbl_ascii.npz")
    ctl = G.ctl_from(f["ctl"])
    ctl.tblbase = str(tmp_path / "tbl")
    for id in range(ctl.nd):
        for ig in range(ctl.ng):
            with open(ctl.table_filename(id, ig), "wb") as fo:
                fo.write(f["tbl_%d_%d" % (id, ig)].tobytes())
    tbl = read_tbl(ctl, 32, 6, 64)
    for id in range(ctl.nd):
        for ig in range(ctl.ng):
            _same_table(_c_read(L, ctl.table_filename(id, ig), 1, 32, 6, 64), tbl, id, ig)


def test_library_table_file_errors(tmp_path, built_lib):
    """Missing and truncated files are JGB_ERR_IO, tables beyond the
    capacities JGB_ERR_ARG (the reference's ERRMSG cases), a bad format
    JGB_ERR_ARG."""
    import copy
    from jurassic_gb300 import native, synth
    from jurassic_gb300.tables import write_tbl
    L = native.load()
    w = synth.config_limb_ega()
    ctl = copy.deepcopy(w.ctl)
    ctl.tblbase = str(tmp_path / "tbl")
    ctl.tblfmt = 2
    tbl = synth.make_tables(ctl, 5, tp=12, tt=5, tu=40)
    write_tbl(ctl, tbl)
    fn = ctl.table_filename(0, 0)
    assert _c_read(L, tmp_path / "none.bin", 2, 12, 5, 40)[0] == native.ERR_IO
    data = open(fn, "rb").read()
    (tmp_path / "cut.bin").write_bytes(data[: len(data) // 2])
    assert _c_read(L, tmp_path / "cut.bin", 2, 12, 5, 40)[0] == native.ERR_IO
    assert _c_read(L, fn, 2, 11, 5, 40)[0] == native.ERR_ARG
    assert _c_read(L, fn, 2, 12, 4, 40)[0] == native.ERR_ARG
    assert _c_read(L, fn, 2, 12, 5, 10)[0] == native.ERR_ARG
    assert _c_read(L, fn, 3, 12, 5, 40)[0] == native.ERR_ARG


def test_ascii_table_level_starting_at_previous_temperature(tmp_path, built_lib):
    """A pressure level whose first point repeats the last temperature of the
    level before opens a temperature row (the reference's temperature index
    would stay at -1 there): both readers give the same two levels of one row
    each, with nothing written out of range."""
    from jurassic_gb300 import native
    from jurassic_gb300.model import Ctl
    from jurassic_gb300.tables import read_tbl
    L = native.load()
    ctl = Ctl(emitter=["CO2"], nu=[700.0])
    ctl.tblbase = str(tmp_path / "tbl")
    ctl.tblfmt = 1
    with open(ctl.table_filename(0, 0), "w") as f:
        f.write("1.0 250.0 1e18 0.1\n1.0 250.0 2e18 0.2\n"
                "2.0 250.0 1e18 0.15\n2.0 250.0 3e18 0.3\n")
    tbl = read_tbl(ctl, 4, 3, 5)
    assert tbl.np_[0, 0] == 2 and list(tbl.nt[0, 0, :2]) == [1, 1]
    assert list(tbl.nu[0, 0, :2, 0]) == [2, 2]
    assert tbl.t[0, 0, 1, 0] == 250.0 and tbl.eps[0, 0, 1, 0, 1] == np.float32(0.3)
    got = _c_read(L, ctl.table_filename(0, 0), 1, 4, 3, 5)
    _same_table(got, tbl, 0, 0)
