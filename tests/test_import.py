"""Import of the tables the reference itself exported (Import_ForceTable +
Register_Imported_ForceTable, MDLIB/sor/Common/MD_TypeDef_ForceTable.F90:1463-1855) and the
export that writes them (Export_ForceTable, :1315-1459).

The fixtures are byte copies of the reference's own export files (tests/golden/ref_*.xz):
the Cu EAM tables it made from the NIST setfl file Cu1.eam.fs.setfl, and the five FS tables
of its W-He library.  The checks:
- the oracle's import (a restatement of the reference's SPLID1/SPLID2 re-grid) and the
  library's (its own slope-form spline) agree to rounding on any target grid;
- re-gridded onto the files' own grid, the import reproduces the exported rows;
- the imported W-He tables equal the library's own generators to the export's 10 digits;
- export then import is the identity to the printed digits, and re-exporting the reference's
  rows writes the same header and numbers;
- a PTYPE id missing from a file and a missing file are refused.
"""
import os

import numpy as np
import pytest

from msmpscu_gb300 import ForceTable, MSMError
from msmpscu_gb300 import _lib as L
from tests.helpers import reference_export


def _rel(a, b, sel=None):
    a, b = np.asarray(a), np.asarray(b)
    if sel is not None:
        a, b = a[sel], b[sel]
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _grid(rmax, ntab):
    return (np.arange(1, ntab + 1) * (np.sqrt(rmax) / ntab)) ** 2


@pytest.mark.parametrize("name,ptype,rmax,ntab,nembd", [
    ("cu1_setfl", [[1]], 5.5, 8000, 5000),
    ("cu1_setfl", [[1]], 6.0, 10000, 10000),
    ("wangjun_w_he", [[1, 4], [3, 2]], 6.0, 10000, 10000),
    ("wangjun_w_he", [[5, 4], [3, 2]], 5.0, 6000, 10000),
])
def test_library_import_matches_oracle(oracle, tmp_path, name, ptype, rmax, ntab, nembd):
    stem = reference_export(tmp_path, name)
    o = oracle.import_tables(stem, ptype, rmax, ntab, nembd)
    t = ForceTable.imported(stem, ptype, rmax, ntab, nembd)
    assert t.pottype == o["pottype"]
    assert t.nkind == len(o["ids"])
    assert np.array_equal(t._kpair.reshape(len(ptype), len(ptype)).T, o["kpair"])
    sel = _grid(rmax, ntab) > 0.5            # below: the files' r -> 0 placeholder rows
    for k in ("potr", "fpotr", "potb", "fpotb"):
        a = getattr(t, k).reshape(ntab, t.nkind)
        for c in range(t.nkind):
            if np.abs(o[k][sel, c]).max() > 0.0:
                assert _rel(a[:, c], o[k][:, c], sel) < 1e-13, (k, c)
    if t.pottype == L.EAM_TYPE:
        assert t.rhod == pytest.approx(o["rhod"], rel=1e-15)
        assert np.array_equal(t._kembd, o["kembd"])
        for k in ("fembd", "dfembd"):
            assert _rel(getattr(t, k).reshape(nembd, t.nkind1), o[k]) < 1e-13, k


@pytest.mark.parametrize("name", ["cu1_setfl", "wangjun_w_he"])
def test_import_on_file_grid_reproduces_exported_rows(oracle, tmp_path, name):
    """On the files' own grid (Rmax = their last r, same NTAB / NEMBD) the spline returns the
    rows: the grid points differ from the printed r only by the 10-digit rounding."""
    stem = reference_export(tmp_path, name)
    pair = oracle.read_imported(stem + ".pair", 4)
    embd = oracle.read_imported(stem + ".embd", 2)
    ids = pair["ids"]
    ng = len(ids)
    rmax = float(pair["x"][-1])
    # a diagonal PTYPE names every table once (groups 1..NT each with its own table)
    ptype = np.full((ng, ng), ids[0], np.int32)
    for i in range(ng):
        ptype[i, i] = ids[i]
    if ng > 1:
        ptype[0, 1:] = ids[1:]
    t = ForceTable.imported(stem, ptype, rmax, len(pair["x"]), len(embd["x"]))
    r = pair["x"]
    # the reference's grid arithmetic (T = K CSIV, CSIV = 1/CSI) can put the last T^2 one ulp
    # above the file's last r, where the import writes 0 (:1717-1723); that row is left out
    csiv = 1.0 / (len(r) / np.sqrt(rmax))
    tt = (np.arange(1, len(r) + 1) * csiv) ** 2
    sel = (r > 0.5) & (tt <= r.max())
    scale = np.array([0.5, 1.0, 1.0, 1.0])
    for k, name_ in enumerate(("potr", "fpotr", "potb", "fpotb")):
        a = getattr(t, name_).reshape(len(r), t.nkind)
        for c in range(t.nkind):
            q = pair["ids"].index(_ids_in_order(ptype)[c])
            want = pair["cols"][:, q, k] * scale[k]
            if np.abs(want[sel]).max() > 0.0:
                assert _rel(a[:, c], want, sel) < 2e-9, (name_, c)
    if t.pottype == L.EAM_TYPE:
        fe = t.fembd.reshape(len(embd["x"]), t.nkind1)[:, 0]
        dfe = t.dfembd.reshape(len(embd["x"]), t.nkind1)[:, 0]
        assert _rel(fe, embd["cols"][:, 0, 0]) < 2e-9
        assert _rel(dfe, embd["cols"][:, 0, 1] / L_EVERG) < 2e-9
        assert t.rhod == pytest.approx(embd["x"][1] - embd["x"][0], rel=1e-8)


L_EVERG = 1.60219e-12


def _ids_in_order(ptype):
    order = []
    for i in range(ptype.shape[0]):
        for j in range(ptype.shape[1]):
            if int(ptype[i, j]) not in order:
                order.append(int(ptype[i, j]))
    return order


def test_imported_w_he_tables_equal_library_generators(tmp_path):
    """The reference's W-He export against this library's own generators of the same five
    tables (already pinned row by row in test_oracle.py): on the export's own grid (10 A) the
    imported tables agree to its printed digits.  (Re-gridded onto another grid the spline
    departs from the generator near the knots of the knot-sum functions, where their second
    derivative jumps: ~1e-6 of the column's largest value for W-W on a 6 A grid, the same for
    the reference's own imported tables.)"""
    stem = reference_export(tmp_path, "wangjun_w_he")
    ru = 10.0
    imp = ForceTable.imported(stem, [[1, 4], [3, 2]], ru, 10000, 10000)
    gen = ForceTable.wangjun_w_he(rmax=ru)
    r = _grid(ru, 10000)
    sel = (r > 1.0) & (r < ru - 1e-3)
    # generator kinds are the library's registration order 1..5; imported kinds are the
    # first-appearance order of PTYPE: W-W (1), W-He (4), He-W (3), He-He (2)
    for kimp, kgen in zip(range(4), [0, 3, 2, 1]):
        for name in ("potr", "fpotr", "potb", "fpotb"):
            a = getattr(imp, name).reshape(10000, imp.nkind)[:, kimp]
            b = getattr(gen, name).reshape(10000, gen.nkind)[:, kgen]
            if np.abs(b[sel]).max() > 0.0:
                assert _rel(a, b, sel) < 2e-8, (name, kimp)


def test_export_import_roundtrip(tmp_path):
    """export() of the library's Marinica EAM2 tables, imported back on the same grid: the
    values come back to the printed digits (10 for the pair rows, 9 for the embedding rows;
    the grid points themselves are printed to 10 digits, which moves a steep column by a few
    1e-9 of its largest value)."""
    t = ForceTable.marinica_eam2()
    stem = os.path.join(str(tmp_path), "w_marinica")
    t.export(stem)
    back = ForceTable.imported(stem, [[1]], t.rmax, t.ntab, t.nembd)
    assert back.pottype == L.EAM_TYPE
    r = _grid(t.rmax, t.ntab)
    sel = r > 1.0
    for name in ("potr", "fpotr", "potb", "fpotb"):
        assert _rel(getattr(back, name), getattr(t, name), sel) < 1e-8, name
    assert back.rhod == pytest.approx(t.rhod, rel=1e-8)
    assert _rel(back.fembd, t.fembd) < 1e-8
    assert _rel(back.dfembd, t.dfembd) < 1e-8


def test_reexport_of_reference_rows(oracle, tmp_path):
    """Importing the reference's Cu export on its own grid and exporting it again writes the
    reference's header lines and its numbers (to the printed digits)."""
    stem = reference_export(tmp_path, "cu1_setfl")
    src = oracle.read_imported(stem + ".pair", 4)
    t = ForceTable.imported(stem, [[1]], float(src["x"][-1]), 10000, 10000)
    out = os.path.join(str(tmp_path), "again")
    t.export(out)
    again = oracle.read_imported(out + ".pair", 4)
    assert again["pottype"] == src["pottype"] and again["ids"] == src["ids"]
    assert np.allclose(again["x"], src["x"], rtol=2e-9, atol=0)
    sel = src["x"] > 0.5
    for c in range(4):
        assert _rel(again["cols"][:, 0, c], src["cols"][:, 0, c], sel) < 2e-9, c
    e0 = oracle.read_imported(stem + ".embd", 2)
    e1 = oracle.read_imported(out + ".embd", 2)
    assert e1["pottype"] == e0["pottype"] and e1["ids"] == e0["ids"]
    assert np.allclose(e1["x"], e0["x"], rtol=1e-8, atol=0)
    for c in range(2):
        assert _rel(e1["cols"][:, 0, c], e0["cols"][:, 0, c]) < 2e-8, c
    for key in ("&POTTYPE", "&NUMTABLE", "&NUMPOINT"):
        a = [ln for ln in open(stem + ".pair") if ln.startswith(key)]
        b = [ln for ln in open(out + ".pair") if ln.startswith(key)]
        assert a == b, key


def test_import_refuses_missing_tables(tmp_path):
    stem = reference_export(tmp_path, "cu1_setfl")
    with pytest.raises(MSMError) as ei:
        ForceTable.imported(stem, [[2]], 5.5)          # no table #2 in the files
    assert ei.value.code == L.ERR_ARG
    with pytest.raises(MSMError):
        ForceTable.imported(os.path.join(str(tmp_path), "absent"), [[1]], 5.5)


def test_nist_route_matches_reference_export(oracle, tmp_path):
    """forcelib's NIST route (the setfl file's tables generated, exported in the reference's
    format and imported onto the run's grid, MD_ForceLib_Register.F90:405-420) against the
    import of the reference's own export of the same file: the exported rows agree to their
    printed digits, so the two tables agree far below the parity bars."""
    from msmpscu_gb300 import forcelib
    from tests.setfl_util import cu1, write_setfl
    path = os.path.join(str(tmp_path), "Cu1.eam.fs.setfl")
    write_setfl(cu1(), path)
    ours = forcelib.create(path, 5.5)
    assert ours.masses is not None and ours.masses[0] == pytest.approx(63.546)
    ref = oracle.import_tables(reference_export(tmp_path, "cu1_setfl"), [[1]], 5.5, 10000, 10000)
    sel = _grid(5.5, 10000) > 0.5
    for name in ("potr", "fpotr", "potb", "fpotb"):
        assert _rel(getattr(ours, name), ref[name][:, 0], sel) < 1e-9, name
    assert ours.rhod == pytest.approx(ref["rhod"], rel=1e-14)
    assert _rel(ours.fembd, ref["fembd"][:, 0]) < 1e-12
    assert _rel(ours.dfembd, ref["dfembd"][:, 0]) < 1e-12
    # with the .pair / .embd next to the file the route imports them as they are
    os.rename(reference_export(tmp_path, "cu1_setfl") + ".pair", path + ".pair")
    os.rename(os.path.join(str(tmp_path), "cu1_setfl.embd"), path + ".embd")
    again = forcelib.create(path, 5.5)
    for name in ("potr", "fpotr", "potb", "fpotb"):
        assert _rel(getattr(again, name), ref[name][:, 0], sel) < 1e-13, name
