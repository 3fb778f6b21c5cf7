"""GPU parity for the remaining potential libraries of the reference on multi-species boxes:
Ackland-Vitek Cu-Au (FS, four tables, geometric-mean cross density) on an L1_2 Cu3Au
crystal with displacements.  The oracle tabulates the functions independently."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu


def _cu3au(ncell, a, sigma, seed):
    pos, L_ = lt.fcc(ncell, ncell, ncell, a)
    # in each cubic cell the corner site is Au, the three face centres Cu (L1_2)
    ityp = np.ones(len(pos), np.int32)
    frac = (pos / a) % 1.0
    ityp[np.all(np.abs(frac) < 1e-6, axis=1)] = 2
    pos = pos + np.random.default_rng(seed).normal(scale=sigma, size=pos.shape)
    return pos - np.floor(pos / L_) * L_, ityp, L_


def test_ackland_vitek_cu3au_force_parity(oracle):
    rc = 5.5
    ft = ForceTable.ackland_vitek(rmax=rc)
    pots = [oracle.POT_AV_CU, oracle.POT_AV_AU, oracle.POT_AV_CUAU, oracle.POT_AV_CUAU]
    ts = [oracle.make_tables(p, None, rc, 10000, 10000, 20.0, want_embed=False) for p in pots]
    arr = {k: np.stack([t[k] for t in ts], 1) for k in ("potr", "fpotr", "potb", "fpotb")}
    t = oracle.RawTables(oracle.FS, 10000, 4, rc, rc, arr["potr"], arr["fpotr"], arr["potb"], arr["fpotb"],
                         np.array([[1, 3], [4, 2]]))
    pos, ityp, L_ = _cu3au(7, 3.75, 0.05, 4)
    assert (ityp == 2).sum() * 4 == len(pos)
    n = len(pos)
    rc_nl = rc + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 200)
    ref = oracle.force(pos, ityp, st, box, kv, ind, t)
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, rc_nl, mxkvois=128, precision=precision)
        e.init_forcetable(ft)
        e.set_masses(np.array([63.546, 196.97]) * lt.AMU)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, ityp=ityp)
        e.calforce()
        f = e.get_force()
        if precision == "mixed":
            assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
        else:
            assert rel_err(f, ref["f"]) < 1e-10, precision
            e.calepot()
            assert rel_err(e.get_epot(), ref["epot"]) < 1e-10, precision
        e.close()


def test_mendelev_zr_hcp_force_parity(oracle):
    ft = ForceTable.mendelev_zr()
    t = oracle.Tables(oracle.make_tables(oracle.POT_MENDELEV_ZR, None, 7.6, 10000, 10000, 20.0),
                      oracle.EAM, 7.6)
    pos, L_ = lt.hcp(8, 5, 5, 3.232, 3.232 * 1.593)          # every edge above 3 rc_nl
    pos = pos + np.random.default_rng(6).normal(scale=0.05, size=pos.shape)
    pos -= np.floor(pos / L_) * L_
    n = len(pos)
    rc_nl = 7.9
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 200)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert ref["nbad"] == 0
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, rc_nl, mxkvois=160, precision=precision)
        e.init_forcetable(ft)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos)
        e.calforce()
        f = e.get_force()
        if precision == "mixed":
            assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
        else:
            assert rel_err(f, ref["f"]) < 1e-10, precision
            assert rel_err(e.get_den(), ref["den"]) < 1e-10, precision
        e.close()


def _fs_parity(oracle, ft, t, pos, ityp, L_, rc_nl, masses):
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 200)
    ref = oracle.force(pos, ityp, st, box, kv, ind, t)
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, rc_nl, mxkvois=160, precision=precision)
        e.init_forcetable(ft)
        e.set_masses(masses)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, ityp=ityp)
        e.calforce()
        f = e.get_force()
        if precision == "mixed":
            assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
        else:
            assert rel_err(f, ref["f"]) < 1e-10, precision
            e.calepot()
            assert rel_err(e.get_epot(), ref["epot"]) < 1e-10, precision
        e.close()


def test_awb_zr_hcp_force_parity(oracle):
    ft = ForceTable.awb_zr(rmax=6.0)
    t = oracle.Tables(oracle.make_tables(oracle.POT_AWB_ZR, None, 6.0, 10000, 10000, 20.0, want_embed=False),
                      oracle.FS, 6.0)
    pos, L_ = lt.hcp(8, 5, 5, 3.249, 3.249 * 1.593)
    pos = pos + np.random.default_rng(8).normal(scale=0.05, size=pos.shape)
    pos -= np.floor(pos / L_) * L_
    _fs_parity(oracle, ft, t, pos, np.ones(len(pos), np.int32), L_, 6.3, np.array([91.224]) * lt.AMU)


def test_wangjun_ti_he_force_parity(oracle):
    rc = 6.0
    ft = ForceTable.wangjun_ti_he(rmax=rc)
    ti = ForceTable.cleri_rosato_element("Ti", rc=rc).prm
    ts = [oracle.make_tables(oracle.POT_CR, list(ti), rc, 10000, 10000, 20.0, want_embed=False),
          oracle.make_tables(oracle.POT_HEHE_EXP6, None, rc, 10000, 10000, 20.0, want_embed=False),
          oracle.make_tables(oracle.POT_HETI_LJ, None, rc, 10000, 10000, 20.0, want_embed=False),
          oracle.make_tables(oracle.POT_HETI_LJ, None, rc, 10000, 10000, 20.0, want_embed=False)]
    arr = {k: np.stack([t[k] for t in ts], 1) for k in ("potr", "fpotr", "potb", "fpotb")}
    t = oracle.RawTables(oracle.FS, 10000, 4, rc, rc, arr["potr"], arr["fpotr"], arr["potb"], arr["fpotb"],
                         np.array([[1, 4], [3, 2]]))
    a, c = 2.951, 2.951 * 1.5874
    pos, L_ = lt.hcp(9, 5, 5, a, c)
    rng = np.random.default_rng(9)
    # He in octahedral sites of the first 12 orthorhombic cells
    he = np.array([[a * (i % 9) + 0.5 * a, a * np.sqrt(3.0) * ((i // 9) % 5) + a * np.sqrt(3.0) / 6.0, 0.25 * c]
                   for i in range(12)])
    pos = np.vstack([pos, he]) + rng.normal(scale=0.03, size=(len(pos) + len(he), 3))
    pos -= np.floor(pos / L_) * L_
    ityp = np.concatenate([np.ones(len(pos) - len(he), np.int32), np.full(len(he), 2, np.int32)])
    _fs_parity(oracle, ft, t, pos, ityp, L_, rc + 0.3, np.array([47.867, 4.0026]) * lt.AMU)


def test_moldy_cu_force_parity(oracle, tmp_path):
    from tests.test_moldy import write_moldy_cu
    p = write_moldy_cu(str(tmp_path / "cu.moldy"))
    ft = ForceTable.moldy(p, rmax=5.0)
    t = oracle.Tables(oracle.moldy_tables(oracle.read_moldy(p), 5.0), oracle.EAM, 5.0)
    pos, vel, L_ = lt.cu_config(8, 0.08, 300.0, 12)
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, 5.3, 200)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, 5.3, mxkvois=128, precision=precision)
        e.init_forcetable(ft)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        e.calforce()
        f = e.get_force()
        if precision == "mixed":
            assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
        else:
            assert rel_err(f, ref["f"]) < 1e-10, precision
            assert rel_err(e.get_den(), ref["den"]) < 1e-10, precision
        e.close()
