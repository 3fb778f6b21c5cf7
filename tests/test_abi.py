"""CPU tests of the C ABI: libmsmgb.so loads, exports every entry point include/msmgb.h
declares, and its host-only parts (table generator, argument checks) behave; no kernel is
launched here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from msmpscu_gb300 import _lib as L
from msmpscu_gb300 import ForceTable, lattice as lt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    txt = open(os.path.join(ROOT, "include", "msmgb.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(msmgb_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from msmpscu_gb300 import build
    build.build()
    return L.load()


def test_library_exports_every_declared_symbol(lib):
    declared = _header_functions()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(L.exported_names()) == declared


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = L.Params(0, 1000, 1, 64, 5.07, 0.15, 10, 0, None)
    ctx = C.c_void_p()
    assert lib.msmgb_create(C.byref(ctx), C.byref(p)) == L.ERR_NO_DEVICE


def test_bad_params_rejected(lib):
    p = L.Params(0, 0, 1, 64, 5.07, 0.15, 10, 0, None)
    ctx = C.c_void_p()
    assert lib.msmgb_create(C.byref(ctx), C.byref(p)) in (L.ERR_ARG, L.ERR_NO_DEVICE)


def test_table_generator_matches_oracle(lib, oracle):
    t = ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC)
    o = oracle.make_tables(oracle.POT_CR, [lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")],
                           lt.CU_RC, 10000, 10000, 20.0, want_embed=False)
    for k in ("potr", "fpotr", "potb", "fpotb"):
        np.testing.assert_allclose(getattr(t, k), o[k], rtol=1e-15, atol=0)
    w = ForceTable.marinica_eam2()
    o = oracle.make_tables(oracle.POT_MARINICA2, None, lt.W_RC, 10000, 10000, 20.0)
    for k in ("potr", "fpotr", "potb", "fpotb", "fembd", "dfembd"):
        np.testing.assert_allclose(getattr(w, k), o[k], rtol=1e-15, atol=1e-300)
    assert w.rhod == o["rhod"]
    for sub, pot in (("EAM3", oracle.POT_MARINICA3), ("EAM4", oracle.POT_MARINICA4)):
        w = ForceTable.marinica_eam2(subtype=sub)
        o = oracle.make_tables(pot, None, lt.W_RC, 10000, 10000, 20.0)
        for k in ("potr", "fpotr", "potb", "fpotb", "fembd", "dfembd"):
            np.testing.assert_allclose(getattr(w, k), o[k], rtol=1e-13, atol=1e-13 * np.abs(o[k]).max())
        assert w.rhod == pytest.approx(o["rhod"], rel=1e-15)


def test_table_generator_rejects_unknown_potential(lib):
    z = np.zeros(10)
    d = z.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.msmgb_create_forcetable(99, None, 5.0, 10, 10, 20.0, d, d, d, d, None, None, None) == L.ERR_ARG


@pytest.mark.parametrize("element,a,ecoh", [("Al", 4.05, -3.317), ("Au", 4.079, -3.778)])
def test_cleri_rosato_library_elements(oracle, element, a, ecoh):
    """Al and Au of the reference's Cleri-Rosato library: library tables equal the oracle's
    CR restatement with the same parameters, and the perfect fcc lattice has zero force and
    the Cleri-Rosato cohesive energy at a three-shell cutoff."""
    ft = ForceTable.cleri_rosato_element(element, rc=1.3 * a)
    o = oracle.make_tables(oracle.POT_CR, list(ft.prm), ft.rmax, 10000, 10000, 20.0, want_embed=False)
    for k in ("potr", "fpotr", "potb", "fpotb"):
        np.testing.assert_allclose(getattr(ft, k), o[k], rtol=1e-15, atol=0)
    pos, L_ = lt.fcc(5, 5, 5, a)
    n = len(pos)
    t = oracle.Tables(o, oracle.FS, ft.rmax)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, ft.rmax + 0.3, 128)
    r = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert np.abs(r["f"]).max() < 1e-10
    assert r["epot"].mean() == pytest.approx(ecoh, abs=2e-3)


def test_cleri_rosato_library_ti_single_precision_constants():
    ft = ForceTable.cleri_rosato_element("Ti", rc=5.0)
    assert ft.prm[0] == float(np.float32(0.1519)) and ft.prm[2] == float(np.float32(8.620))
    assert ft.prm[4] == pytest.approx(2.951 * np.sqrt(1 / 3 + 1.5874 ** 2 / 4), rel=1e-6)
    with pytest.raises(ValueError):
        ForceTable.cleri_rosato_element("Cu", rc=5.0)


@pytest.mark.parametrize("pot,a,ecoh", [("POT_AV_CU", 3.615, -3.518), ("POT_AV_AU", 4.078, -3.789),
                                        ("POT_AV_CUAU", None, None)])
def test_ackland_vitek_tables(oracle, pot, a, ecoh):
    """Ackland-Vitek Cu, Au and Cu-Au: the library's CGS evaluation equals the oracle's
    Angstrom/eV restatement; the pure metals have zero force and their cohesive energy on the
    perfect fcc lattice."""
    ft = ForceTable(getattr(L, pot), None, 6.0, 6.0, L.FS_TYPE)
    o = oracle.make_tables(getattr(oracle, pot), None, 6.0, 10000, 10000, 20.0, want_embed=False)
    for k in ("potr", "fpotr", "potb", "fpotb"):
        assert np.max(np.abs(getattr(ft, k) - o[k])) <= 1e-14 * np.max(np.abs(o[k])), k
    if a is None:
        # the cross density's derivative of the reference carries a factor EVERG^2 (CGS)
        assert 0.0 < np.max(np.abs(o["fpotb"])) < 1e-18 < np.max(o["potb"])
        return
    pos, L_ = lt.fcc(5, 5, 5, a)
    n = len(pos)
    t = oracle.Tables(o, oracle.FS, 6.0)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, 6.3, 200)
    r = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert np.abs(r["f"]).max() < 1e-10
    assert r["epot"].mean() == pytest.approx(ecoh, abs=2e-3)


def test_mendelev_zr_tables_and_hcp_energy(oracle):
    """Mendelev-Ackland Zr: library equals oracle (the first F' row is -inf in both, as in the
    reference); the perfect hcp crystal has zero force and E = -6.467 eV/atom."""
    ft = ForceTable.mendelev_zr()
    o = oracle.make_tables(oracle.POT_MENDELEV_ZR, None, 7.6, 10000, 10000, 20.0)
    for k in ("potr", "fpotr", "potb", "fpotb", "fembd", "dfembd"):
        a, b = getattr(ft, k), o[k]
        fin = np.isfinite(b)
        assert np.array_equal(np.isfinite(a), fin), k
        assert np.max(np.abs(a[fin] - b[fin])) <= 1e-12 * np.max(np.abs(b[fin])), k
    assert np.isneginf(ft.dfembd[0]) and ft.rhod == pytest.approx(o["rhod"], rel=1e-14)
    pos, L_ = lt.hcp(6, 4, 4, 3.232, 3.232 * 1.593)
    n = len(pos)
    t = oracle.Tables(o, oracle.EAM, 7.6)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, 7.9, 200)
    r = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert r["nbad"] == 0 and np.abs(r["f"]).max() < 1e-10
    assert r["epot"].mean() == pytest.approx(-6.467, abs=2e-3)


@pytest.mark.parametrize("pot,typ", [("POT_AWB_ZR", "FS"), ("POT_HETI_LJ", "FS")])
def test_awb_and_heti_tables(oracle, pot, typ):
    """AWB Zr and the He-Ti pair: the library's CGS evaluation equals the oracle's Angstrom/eV
    restatement."""
    ft = ForceTable(getattr(L, pot), None, 6.0, 6.0, L.FS_TYPE)
    o = oracle.make_tables(getattr(oracle, pot), None, 6.0, 10000, 10000, 20.0, want_embed=False)
    for k in ("potr", "fpotr", "potb", "fpotb"):
        assert np.max(np.abs(getattr(ft, k) - o[k])) <= 1e-14 * max(np.max(np.abs(o[k])), 1e-300), k


def test_awb_zr_hcp_energy(oracle):
    ft = ForceTable.awb_zr(rmax=6.0)
    t = oracle.Tables(oracle.make_tables(oracle.POT_AWB_ZR, None, 6.0, 10000, 10000, 20.0, want_embed=False),
                      oracle.FS, 6.0)
    pos, L_ = lt.hcp(8, 5, 5, 3.249, 3.249 * 1.593)
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, 6.3, 200)
    r = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert np.abs(r["f"]).max() < 1e-10
    assert r["epot"].mean() == pytest.approx(-6.243, abs=2e-3)
    assert ft.nkind == 1


def test_wangjun_ti_he_kpair():
    ft = ForceTable.wangjun_ti_he(rmax=6.0)
    kp = ft._kpair.reshape(2, 2).T
    assert kp.tolist() == [[1, 4], [3, 2]]
    p = ft.potr.reshape(ft.ntab, 4)
    assert np.array_equal(p[:, 2], p[:, 3]) and not ft.potb.reshape(ft.ntab, 4)[:, 1:].any()
