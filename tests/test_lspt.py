"""lspt import (tabulated EAM from ".spt" files): the oracle's tables are pinned against the
embedding table the reference itself exported for the W-H-He potential, and the library's
own reader and table builder reproduce the oracle's tables, including the reference's
reading of the pair lines (the first file of a line serves every pair of it)."""
import os

import numpy as np
import pytest

from msmpscu_gb300 import ForceTable, MSMError
from msmpscu_gb300 import _lib as L
from tests.lspt_util import GOLDEN, whhe, whhe_data, write_lspt

EVERG = 1.60219e-12       # the reference's eV -> erg constant (the export's dF/drho column)


def _rows():
    out = {}
    for line in open(os.path.join(GOLDEN, "whhe_lspt_embd_rows.txt")):
        f = line.split()
        if f and f[0] == "E":
            out[int(f[1])] = [float(x) for x in f[2:]]
    return out


def test_oracle_lspt_embedding_matches_reference_export(oracle, tmp_path):
    d = oracle.read_lspt(whhe(str(tmp_path)))
    assert d["elements"] == ["W", "H", "He"] and d["rhomax"] == 10.0
    t = oracle.lspt_tables(d)
    assert t["rhod"] == pytest.approx(1e-3, rel=1e-15)     # RHOD = the F(rho) file's last knot / NEMBD
    rows = _rows()
    assert len(rows) > 390
    for i, (rho, f, df) in rows.items():
        assert rho == pytest.approx((i - 1) * t["rhod"], rel=1e-9, abs=1e-15)
        # nine printed significant digits
        assert t["fembd"][i - 1, 0] == pytest.approx(f, rel=6e-9, abs=1e-12), i
        assert t["dfembd"][i - 1, 0] * EVERG == pytest.approx(df, rel=6e-9, abs=1e-20), i
    assert not t["fembd"][:, 1:].any() and not t["dfembd"][:, 1:].any()
    # H and He carry no F(rho): no density is tabulated at H or He hosts
    ne = 3
    for i in (1, 2):
        assert not t["potb"][:, i * ne:(i + 1) * ne].any()


def test_library_lspt_matches_oracle(oracle, tmp_path):
    path = whhe(str(tmp_path))
    for each in (False, True):
        ft = ForceTable.lspt(path, each_vr_file=each)
        t = oracle.lspt_tables(oracle.read_lspt(path, each_vr_file=each))
        assert ft.nkind == 9 and ft.nkind1 == 3 and ft.ngroup == 3
        assert ft.rmax == 5.4604375 and ft.rhod == pytest.approx(t["rhod"], rel=1e-15)
        for k in ("potr", "fpotr", "potb", "fpotb"):
            a, b = getattr(ft, k).reshape(ft.ntab, 9), t[k]
            assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(b)), (each, k)
        for k in ("fembd", "dfembd"):
            a, b = getattr(ft, k).reshape(ft.nembd, 3), t[k]
            assert np.max(np.abs(a - b)) <= 1e-13 * np.max(np.abs(b)), (each, k)
        assert np.array_equal(ft._kpair.reshape(3, 3).T, t["kpair"])
        assert list(ft._kembd) == [1, 2, 3]


def test_lspt_pair_line_reading(oracle, tmp_path):
    """Pair line 2 quotes pWH, pHH: the reference tabulates H-H with pWH, the opt-in flag
    with pHH."""
    path = whhe(str(tmp_path))
    el, slots, files = whhe_data()
    hh = 1 * 3 + 1
    ref = ForceTable.lspt(path, ntab=2000)
    each = ForceTable.lspt(path, ntab=2000, each_vr_file=True)
    wh = ForceTable.lspt(path, ntab=2000).potr.reshape(2000, 9)[:, 1 * 3 + 0]
    assert np.array_equal(ref.potr.reshape(2000, 9)[:, hh], wh)
    assert not np.array_equal(each.potr.reshape(2000, 9)[:, hh], wh)
    # the opt-in table is pHH's spline: 0.5 V(r) r at a knot of the file
    x, y = files[slots["vr_1_1"]]
    r = (np.arange(1, 2001) * (np.sqrt(each.rmax) / 2000)) ** 2
    k = np.searchsorted(r, 1.5)
    v = oracle.read_lspt(path, each_vr_file=True)["vr"][(1, 1)]
    assert np.array_equal(v[1], y)
    assert each.potr.reshape(2000, 9)[k, hh] == pytest.approx(
        0.5 * r[k] * np.interp(r[k], x, y), rel=1e-5)


def test_lspt_reader_errors(tmp_path):
    el, slots, files = whhe_data()
    bad = dict(slots)
    bad["rhor_0"] = "missing.spt"
    with pytest.raises(MSMError) as e:
        ForceTable.lspt(write_lspt(str(tmp_path / "a"), el, bad, files))
    assert e.value.code == L.ERR_ARG
    p = write_lspt(str(tmp_path / "b"), el, slots, files)
    txt = open(p).read().replace("&LSPT", "&SPT")
    open(p, "w").write(txt)
    with pytest.raises(MSMError):
        ForceTable.lspt(p)
    # a pair line quoting the wrong number of files
    p = write_lspt(str(tmp_path / "c"), el, slots, files)
    lines = open(p).read().split("\n")
    lines = [ln.replace('"WHHe-EAM1-pWH.spt", ', "") for ln in lines]
    open(p, "w").write("\n".join(lines))
    with pytest.raises(MSMError):
        ForceTable.lspt(p)
    # decreasing knots
    x, y = files[slots["vr_0_0"]]
    f2 = dict(files)
    f2[slots["vr_0_0"]] = (x[::-1], y)
    with pytest.raises(MSMError):
        ForceTable.lspt(write_lspt(str(tmp_path / "d"), el, slots, f2))
