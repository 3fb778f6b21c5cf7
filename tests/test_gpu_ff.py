"""Float-float force passes (MSMGB_PREC_FF): the FP64 parity bar (1e-10 relative, max abs
difference over the max magnitude) against the FP64 oracle, on the FP32 pipe."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from msmpscu_gb300 import _lib as L
from tests.helpers import cu_tables, w_tables, rel_err
from tests.test_gpu_edges import _two_species_tables

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _ref(oracle, pos, L_, t, rc_nl, ityp=None, statu=None, mxk=128):
    n = len(pos)
    st = np.ones(n, np.int32) if statu is None else statu
    ty = np.ones(n, np.int32) if ityp is None else ityp
    box = oracle.make_box([0, 0, 0], L_)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, mxk)
    return oracle.force(pos, ty, st, box, kv, ind, t)


@pytest.mark.parametrize("ncell,sigma,seed", [(10, 0.02, 1), (6, 0.1, 2), (16, 0.05, 3)])
def test_ff_cu_force_parity(oracle, ncell, sigma, seed):
    pos, vel, L_ = lt.cu_config(ncell, sigma, 300.0, seed)
    ref = _ref(oracle, pos, L_, cu_tables(oracle), lt.CU_RC_NL)
    e = Engine(len(pos), lt.CU_RC_NL, mxkvois=64, precision="ff")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.copyin([(len(pos), (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.calforce()
    err_f = rel_err(e.get_force(), ref["f"])
    err_d = rel_err(e.get_den(), ref["den"])
    assert err_f < TOL and err_d < TOL, (err_f, err_d)
    # virial and energies come from the FP64 passes in this mode
    assert rel_err(e.calptensor()[0], ref["vir"]) < TOL
    e.close()


def test_ff_eam_w_force_parity(oracle):
    pos, L_ = lt.w_sia_config(8, 0.02, 3)
    ref = _ref(oracle, pos, L_, w_tables(oracle), lt.W_RC_NL)
    e = Engine(len(pos), lt.W_RC_NL, mxkvois=96, precision="ff")
    e.init_forcetable(ForceTable.marinica_eam2())
    e.copyin([(len(pos), (0, 0, 0), tuple(L_), (1, 1, 1))], pos)
    e.calforce()
    err_f = rel_err(e.get_force(), ref["f"])
    err_d = rel_err(e.get_den(), ref["den"])
    assert err_f < TOL and err_d < TOL, (err_f, err_d)
    e.close()


def test_ff_two_species_and_inactive(oracle):
    pos, vel, L_ = lt.cu_config(8, 0.05, 300.0, 31)
    n = len(pos)
    ityp = (np.random.default_rng(3).random(n) < 0.3).astype(np.int32) + 1
    st = np.ones(n, np.int32)
    st[::9] = 0
    arr, kpair = _two_species_tables(oracle)
    t = oracle.RawTables(oracle.FS, 10000, 4, lt.CU_RC, lt.CU_RC, arr["potr"], arr["fpotr"],
                         arr["potb"], arr["fpotb"], kpair)
    ref = _ref(oracle, pos, L_, t, lt.CU_RC_NL, ityp=ityp, statu=st)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="ff")
    e.init_forcetable_raw(L.FS_TYPE, 10000, 4, lt.CU_RC, lt.CU_RC, arr["potr"], arr["fpotr"],
                          arr["potb"], arr["fpotb"], 2, kpair)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp, statu=st)
    e.calforce()
    f = e.get_force()
    assert np.all(f[::9] == 0.0)
    assert rel_err(f, ref["f"]) < TOL
    e.close()


def test_ff_md_trajectory_parity_cu4000(oracle):
    """100 NVE steps (skin trigger): the float-float step tracks the FP64 oracle like the
    FP64 step does."""
    pos, vel, L_ = lt.cu_config(10, 0.02, 300.0, 1)
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    ox, ov, of, ost, oreb = oracle.md(pos, vel, np.ones(n, np.int32), np.ones(n, np.int32), box,
                                      cu_tables(oracle), np.array([lt.CU_MASS]), 1.0, 100, lt.CU_RC_NL,
                                      skin_trigger=0.15, mxkvois=96)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="ff")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    nreb = e.run_steps(100, 1.0)
    gx, gv, _, _ = e.get_state()
    dx = gx - ox
    dx -= np.round(dx / L_) * L_
    assert np.max(np.abs(dx)) < 1e-8
    assert np.max(np.abs(gv - ov)) < 1e-10
    assert rel_err(e.get_force(), of) < 1e-8
    assert nreb == oreb
    e.close()


def test_ff_full_size_cu_2048000(oracle):
    """2,048,000 atoms (80^3 cells, the benchmark system): float-float forces at the FP64
    parity bar against the OpenMP oracle."""
    pos, vel, L_ = lt.cu_config(80, 0.05, 600.0, 2024)
    n = len(pos)
    ref = _ref(oracle, pos, L_, cu_tables(oracle), lt.CU_RC_NL, mxk=80)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="ff")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.calforce()
    err = rel_err(e.get_force(), ref["f"])
    assert err < TOL, err
    e.close()
