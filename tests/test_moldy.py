"""Moldy potential files: the library's reader and tables equal the oracle's restatement, and a
Moldy file holding the Ackland-Vitek Cu knots (coefficients in eV, knots in units of the
lattice constant) reproduces that potential's cohesive energy on the perfect fcc lattice,
which checks the a0, a0^-3 and a0^-6 scalings of the reader."""
import numpy as np
import pytest

from msmpscu_gb300 import ForceTable, MSMError, forcelib, lattice as lt

A0 = 3.615


def write_moldy_cu(path):
    a = [61.73525861, -108.1846780, 57.00053948, -12.88796578, 39.163819010]
    r = [1.225, 1.202, 1.154, 1.050, 0.866]
    big_a = [17.06363299 * A0 ** 3, 10.03718305 * A0 ** 3]
    big_r = [0.990, 1.225]
    with open(path, "w") as fh:
        fh.write("Cu\n")
        fh.write(", ".join("%.12g" % x for x in a) + "\n")
        fh.write("  ".join("%.12g" % x for x in r) + "\n")
        fh.write("(" + " ".join("%.12g" % x for x in big_a) + ")\n")
        fh.write("[" + ", ".join("%.12g" % x for x in big_r) + "]\n")
        fh.write("a0 = %.12g  29 63.546\n" % A0)
    return path


def test_moldy_library_matches_oracle(oracle, tmp_path):
    p = write_moldy_cu(str(tmp_path / "cu.moldy"))
    ft = ForceTable.moldy(p, rmax=5.0)
    d = oracle.read_moldy(p)
    assert d["a0"] == A0 and len(d["av"]) == 5 and len(d["ab"]) == 2
    t = oracle.moldy_tables(d, 5.0)
    for k in ("potr", "fpotr", "potb", "fpotb", "fembd", "dfembd"):
        assert np.max(np.abs(getattr(ft, k) - t[k])) <= 1e-13 * np.max(np.abs(t[k])), k
    assert ft.rhod == pytest.approx(t["rhod"], rel=1e-14)
    f2 = forcelib.create(p, ru=5.0)
    np.testing.assert_array_equal(f2.potr, ft.potr)


def test_moldy_cu_reproduces_ackland_vitek_energy(oracle, tmp_path):
    p = write_moldy_cu(str(tmp_path / "cu.moldy"))
    t = oracle.Tables(oracle.moldy_tables(oracle.read_moldy(p), 6.0), oracle.EAM, 6.0)
    pos, L_ = lt.fcc(5, 5, 5, A0)
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, 6.3, 200)
    r = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert np.abs(r["f"]).max() < 1e-10
    assert r["epot"].mean() == pytest.approx(-3.518, abs=2e-3)


def test_moldy_reader_errors(tmp_path):
    p = tmp_path / "bad.moldy"
    p.write_text("Cu\n1 2 3\n1 2\n1\n1\n3.6\n")          # 3 coefficients, 2 knots
    with pytest.raises(MSMError):
        ForceTable.moldy(str(p), rmax=5.0)
    with pytest.raises(MSMError):
        ForceTable.moldy(str(tmp_path / "missing.moldy"), rmax=5.0)
