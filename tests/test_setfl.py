"""Setfl import (tabulated EAM): the oracle's natural-spline tables are pinned against the
tables the reference itself exported from the same file, and the library's own file reader
and table builder reproduce the oracle's tables (single and two-element files)."""
import os

import numpy as np
import pytest

from msmpscu_gb300 import ForceTable
from tests.setfl_util import GOLDEN, cu1, two_elements, write_setfl

EVERG = 1.60219e-12       # the reference's eV -> erg constant (the export's dF/drho column)


def _golden_rows():
    p, e = {}, {}
    for line in open(os.path.join(GOLDEN, "cu1_setfl_rows.txt")):
        f = line.split()
        if not f or f[0].startswith("#"):
            continue
        (p if f[0] == "P" else e)[int(f[1])] = [float(x) for x in f[2:]]
    return p, e


def test_oracle_setfl_tables_match_reference_export(oracle):
    d = cu1()
    t = oracle.setfl_tables(d)
    pair, emb = _golden_rows()
    assert len(pair) > 400 and len(emb) > 390
    csiv = np.sqrt(d["cutoff"]) / 10000
    for i, (r, rphi, mrdphi, rho, mdrho) in pair.items():
        assert r == pytest.approx((i * csiv) ** 2, rel=1e-9)
        mine = (2.0 * t["potr"][i - 1], t["fpotr"][i - 1], t["potb"][i - 1], t["fpotb"][i - 1])
        for a, b in zip(mine, (rphi, mrdphi, rho, mdrho)):
            # ten printed significant digits
            assert abs(a - b) <= 6e-10 * abs(b) + 1e-20, (i, a, b)
    for i, (rho, f, df) in emb.items():
        assert rho == pytest.approx((i - 1) * d["drho"], rel=1e-9, abs=1e-12)
        assert t["fembd"][i - 1] == pytest.approx(f, rel=6e-9, abs=1e-12)
        if i > 1:   # the first slope of the natural spline is printed to ~1e-11 erg only
            assert t["dfembd"][i - 1] * EVERG == pytest.approx(df, rel=6e-9, abs=1e-20)


def test_library_setfl_reader_matches_oracle(oracle, tmp_path):
    d = cu1()
    path = str(tmp_path / "cu1.setfl")
    write_setfl(d, path)
    ft = ForceTable.setfl(path)
    t = oracle.setfl_tables(d)
    for k in ("potr", "fpotr", "potb", "fpotb", "fembd", "dfembd"):
        a, b = getattr(ft, k), t[k]
        assert np.max(np.abs(a - b)) <= 1e-14 * np.max(np.abs(b[np.isfinite(b)])), k
    assert ft.rhod == d["drho"] and ft.rmax == d["cutoff"] and ft.masses[0] == d["mass"][0]
    # the oracle's Python reader parses the same file to the same arrays
    r = oracle.read_setfl(path)
    assert np.array_equal(r["rphi"][(0, 0)], d["rphi"][(0, 0)])


def test_library_setfl_two_elements(oracle, tmp_path):
    d = two_elements()
    path = str(tmp_path / "cuxx.setfl")
    write_setfl(d, path)
    ft = ForceTable.setfl(path, ntab=4000)
    ne, nk = 2, 4
    assert ft.nkind == nk and ft.nkind1 == ne and ft.ngroup == ne
    kp = ft._kpair.reshape(ne, ne).T                       # KPAIR(I, J) at kp[I-1, J-1]
    for i in range(ne):
        for j in range(ne):
            k = kp[i, j] - 1
            assert k == i * ne + j
            t = oracle.setfl_tables(d, ntab=4000, i=i, j=j)
            for key in ("potr", "fpotr", "potb", "fpotb"):
                a = getattr(ft, key).reshape(4000, nk)[:, k]
                assert np.max(np.abs(a - t[key])) <= 1e-14 * np.max(np.abs(t[key])), (i, j, key)
        e = ft.fembd.reshape(d["nrho"], ne)[:, i]
        assert np.max(np.abs(e - oracle.setfl_tables(d, ntab=4000, i=i)["fembd"])) <= 1e-14 * np.max(np.abs(e))
    assert list(ft._kembd) == [1, 2]
    assert ft.masses[1] == pytest.approx(1.5 * d["mass"][0])
