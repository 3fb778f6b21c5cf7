"""The force-library factory by name: group symbols map to tables as the reference's
Create_Interaction_ForceTable does (PTYPE(I,J) = the table registered for a neighbour of
group J's element at a host of group I's element), only the tables in use are built, and the
result equals the dedicated table builders."""
import numpy as np
import pytest

from msmpscu_gb300 import ForceTable, forcelib
from msmpscu_gb300 import _lib as L


def _cols(ft):
    return {k: getattr(ft, k).reshape(ft.ntab, ft.nkind) for k in ("potr", "fpotr", "potb", "fpotb")}


def test_ackland_vitek_by_symbols_matches_builder():
    f = forcelib.create("EM_TB_Ackland_Vitek_PRB41_10324", ru=5.5, symbols=["Cu", "Au"])
    # a Cu host takes table 3, registered as (Au source, Cu target); an Au host table 4
    assert f.ptype.tolist() == [[1, 3], [4, 2]]
    ref = ForceTable.ackland_vitek(rmax=5.5)
    a, b = _cols(f), _cols(ref)
    kf, kr = f._kpair.reshape(2, 2).T, ref._kpair.reshape(2, 2).T
    for i in range(2):
        for j in range(2):
            for k in a:
                assert np.array_equal(a[k][:, kf[i, j] - 1], b[k][:, kr[i, j] - 1])


def test_only_tables_in_use_are_built():
    f = forcelib.create("EM_TB_Ackland_Vitek_PRB41_10324", ru=5.5, symbols=["Au"])
    assert f.nkind == 1 and f.ptype.tolist() == [[2]] and list(f._kpair) == [1]
    g = forcelib.create("EM_TB_Cleri_Rosato_PRB48_22", ru=4.0, symbols=["Al1"])   # symbol prefix "AL"
    assert g.nkind == 1
    np.testing.assert_array_equal(g.potr, ForceTable.cleri_rosato_element("Al", rc=4.0).potr)
    with pytest.raises(ValueError):
        forcelib.create("EM_TB_Cleri_Rosato_PRB48_22", ru=4.0, symbols=["Al", "Au"])  # no Al-Au table


def test_wangjun_w_he_by_table_numbers_and_eam_variant():
    pt = [[1, 4], [3, 2]]
    f = forcelib.create("EM_TB_WANGJUN_W-HE_2010", ru=6.0, ptype=pt)
    ref = ForceTable.wangjun_w_he(rmax=6.0)
    a, b = _cols(f), _cols(ref)
    kf, kr = f._kpair.reshape(2, 2).T, ref._kpair.reshape(2, 2).T
    assert f.nkind == 4
    for i in range(2):
        for j in range(2):
            for k in a:
                np.testing.assert_array_equal(a[k][:, kf[i, j] - 1], b[k][:, kr[i, j] - 1])
    with pytest.raises(ValueError):
        forcelib.create("EM_TB_WANGJUN_W-HE_2010", ru=6.0, symbols=["W", "He"])   # registered by number
    e = forcelib.create("EM_TB_WANGJUN_W-HE_2010", ru=6.0, ptype=[[5, 4], [3, 2]], pottype="EAM_TYPE")
    assert e.pottype == L.EAM_TYPE and e.nkind1 == 2
    fe = e.fembd.reshape(e.nembd, 2)
    rho = np.arange(e.nembd) * e.rhod
    np.testing.assert_allclose(fe[1:, 0], -np.sqrt(rho[1:]), rtol=1e-15)
    assert e.rhod == pytest.approx(20.0 * e.potb.max() / e.nembd, rel=1e-15)


def test_bonny_and_marinica_by_symbols():
    b = forcelib.create("EAM_WHeH_Bonny_JPCM26_2014", ru=5.4604375, symbols=["W", "H", "He"], subtype="EAM2")
    ref = ForceTable.bonny_wheh("EAM2")
    assert b.ptype.tolist() == [[1, 2, 3], [4, 5, 6], [7, 8, 9]]
    for k in ("potr", "potb"):
        np.testing.assert_array_equal(getattr(b, k).reshape(b.ntab, 9), getattr(ref, k).reshape(ref.ntab, 10)[:, :9])
    np.testing.assert_array_equal(b.fembd.reshape(b.nembd, 3), ref.fembd.reshape(ref.nembd, 3))
    assert list(b._kembd) == [1, 2, 3] and b.rhod == ref.rhod
    m = forcelib.create("EAM_WW_Marinica_JPCM25_2013", ru=5.4604375, symbols=["W"], subtype="EAM4")
    np.testing.assert_array_equal(m.fembd, ForceTable.marinica_eam2(subtype="EAM4").fembd)
    z = forcelib.create("EAM_Zr_Mendelev_Phil_Mag_L87_2007", ru=7.6, symbols=["Zr"])
    np.testing.assert_array_equal(z.potr, ForceTable.mendelev_zr().potr)
    with pytest.raises(ValueError):
        forcelib.create("NO_SUCH_LIB", ru=5.0, symbols=["W"])
