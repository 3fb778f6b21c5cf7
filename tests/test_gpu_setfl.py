"""GPU force parity with tables imported from a setfl file (Mendelev Cu, the reference's own
example potential, and a two-element file derived from it)."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from msmpscu_gb300 import _lib as L
from tests.helpers import rel_err
from tests.setfl_util import cu1, two_elements, write_setfl

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _cu_mendelev(ncell, sigma, seed):
    pos, vel, L_ = lt.cu_config(ncell, sigma, 300.0, seed)
    s = cu1()["alat"] / (L_[0] / ncell)                     # Mendelev lattice constant
    return pos * s, vel, L_ * s


@pytest.mark.parametrize("precision", ["fp64", "ff", "mixed"])
def test_setfl_cu_force_parity(oracle, tmp_path, precision):
    d = cu1()
    path = str(tmp_path / "cu1.setfl")
    write_setfl(d, path)
    ft = ForceTable.setfl(path)
    t = oracle.Tables(oracle.setfl_tables(d), oracle.EAM, d["cutoff"])
    pos, vel, L_ = _cu_mendelev(8, 0.05, 21)
    n = len(pos)
    rc_nl = d["cutoff"] + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 160)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert ref["nbad"] == 0
    e = Engine(n, rc_nl, mxkvois=128, precision=precision)
    e.init_forcetable(ft)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.calforce()
    f = e.get_force()
    if precision == "mixed":
        assert np.linalg.norm(f - ref["f"]) / np.linalg.norm(ref["f"]) < 1e-6
        assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
    else:
        assert rel_err(f, ref["f"]) < TOL
        assert rel_err(e.get_den(), ref["den"]) < TOL
    e.close()


def test_setfl_two_element_force_parity(oracle, tmp_path):
    d = two_elements()
    path = str(tmp_path / "cuxx.setfl")
    write_setfl(d, path)
    ft = ForceTable.setfl(path)
    ntab, ne, nk = ft.ntab, 2, 4
    pos, vel, L_ = _cu_mendelev(8, 0.05, 22)
    n = len(pos)
    ityp = (np.random.default_rng(5).random(n) < 0.35).astype(np.int32) + 1
    kp = ft._kpair.reshape(ne, ne).T
    t = oracle.RawTables(oracle.EAM, ntab, nk, ft.rmax, ft.ru, ft.potr.reshape(ntab, nk),
                         ft.fpotr.reshape(ntab, nk), ft.potb.reshape(ntab, nk), ft.fpotb.reshape(ntab, nk), kp,
                         fembd=ft.fembd.reshape(-1, ne), dfembd=ft.dfembd.reshape(-1, ne), kembd=ft._kembd,
                         rhod=ft.rhod)
    rc_nl = d["cutoff"] + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 160)
    ref = oracle.force(pos, ityp, st, box, kv, ind, t)
    assert ref["nbad"] == 0
    for precision in ("fp64", "ff"):
        e = Engine(n, rc_nl, mxkvois=128, precision=precision)
        e.init_forcetable(ft)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp)
        e.calforce()
        assert rel_err(e.get_force(), ref["f"]) < TOL, precision
        e.close()
