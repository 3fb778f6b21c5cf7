"""GPU parity on the reference's own tables.

The tables here are not generated by this library: they are the rows the reference itself
exported (tests/golden/ref_*.xz, byte copies of its Export_ForceTable output), read back and
re-gridded as the reference runs them (Register_Imported_ForceTable,
MDLIB/sor/Common/MD_TypeDef_ForceTable.F90:1612-1855; the route of every NIST potential,
MDLIB/sor/Appshell/MD_ForceLib_Register.F90:405-420).  The library imports them with its own
spline, the oracle with its restatement of the reference's SPLID1/SPLID2; each side then runs
its own passes on its own import.  So everything upstream of the force arithmetic is the
reference's bytes, and the parity bars are those of the other GPU tests: FP64 and
float-float forces, F'(rho), energies and virial within 1e-10 relative, a 100-step FP64
trajectory within 1e-8 A, mixed forces within 1e-6."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from tests.helpers import reference_export, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-10
CU_RU = 5.5                      # below the setfl file's 6 A range
CU_RC_NL = CU_RU + 0.3
W_RU = 6.0
MASSES_WHE = np.array([183.84, 4.0026]) * lt.AMU


def _oracle_tables(oracle, d, ru):
    return oracle.RawTables(d["pottype"], d["ntab"], d["potr"].shape[1], d["rmax"], ru, d["potr"], d["fpotr"],
                            d["potb"], d["fpotb"], d["kpair"], fembd=d["fembd"], dfembd=d["dfembd"],
                            kembd=d["kembd"], rhod=d["rhod"])


def _cu_state(seed, ncell=10, sigma=0.05, temp=600.0):
    return lt.cu_config(ncell, sigma, temp, seed)


def test_imported_cu_setfl_force_parity(oracle, tmp_path):
    """fcc Cu on the reference's Cu1 setfl export (EAM), every precision."""
    stem = reference_export(tmp_path, "cu1_setfl")
    od = oracle.import_tables(stem, [[1]], CU_RU, 10000, 10000)
    t = _oracle_tables(oracle, od, CU_RU)
    ft = ForceTable.imported(stem, [[1]], CU_RU, 10000, 10000)
    pos, vel, L_ = _cu_state(3)
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, CU_RC_NL, 128)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    assert np.abs(ref["f"]).max() > 0.1
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, CU_RC_NL, mxkvois=96, precision=precision)
        e.init_forcetable(ft)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        if precision == "mixed":
            e.calforce()
            f = e.get_force()
            assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
        else:
            vir = e.calptensor()[0]
            assert rel_err(e.get_force(), ref["f"]) < TOL, precision
            assert rel_err(vir, ref["vir"]) < TOL, precision
            assert rel_err(e.get_den(), ref["den"]) < TOL, precision
            e.calepot()
            assert rel_err(e.get_epot(), ref["epot"]) < TOL, precision
        e.close()


def test_imported_cu_setfl_md_100_steps(oracle, tmp_path):
    """100 NVE steps of 1 fs (600 K, skin trigger) on the imported Cu tables: FP64 trajectory
    within 1e-8 A of the oracle's on its own import, same rebuild count."""
    stem = reference_export(tmp_path, "cu1_setfl")
    od = oracle.import_tables(stem, [[1]], CU_RU, 10000, 10000)
    t = _oracle_tables(oracle, od, CU_RU)
    ft = ForceTable.imported(stem, [[1]], CU_RU, 10000, 10000)
    pos, vel, L_ = _cu_state(4)
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    one = np.ones(n, np.int32)
    ox, ov, of, _, oreb = oracle.md(pos, vel, one, one, box, t, np.array([lt.CU_MASS]), 1.0, 100, CU_RC_NL,
                                    skin_trigger=0.15, mxkvois=128)
    e = Engine(n, CU_RC_NL, mxkvois=96, skin_trigger=0.15)
    e.init_forcetable(ft)
    e.set_masses([lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    nreb = e.run_steps(100, 1.0)
    x, v, _, _ = e.get_state()
    dx = x - ox
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < 1e-8
    assert np.abs(v - ov).max() < 1e-10
    assert rel_err(e.get_force(), of) < 1e-8
    assert nreb == oreb and nreb > 0
    e.close()


def _w_he(seed):
    rng = np.random.default_rng(seed)
    pos, L_ = lt.bcc(8, 8, 8, lt.W_A)
    a = lt.W_A
    cells = rng.choice(512, 15, replace=False)
    he = [a * np.array([c % 8, (c // 8) % 8, c // 64], float) + a * np.array([0.25, 0.5, 0.0]) for c in cells]
    pos = np.vstack([pos, np.array(he)]) + rng.normal(scale=0.03, size=(len(pos) + len(he), 3))
    pos -= np.floor(pos / L_) * L_
    ityp = np.concatenate([np.ones(len(pos) - len(he), np.int32), np.full(len(he), 2, np.int32)])
    return pos, ityp, L_


@pytest.mark.parametrize("ww", [1, 5])
def test_imported_w_he_fs_parity(oracle, tmp_path, ww):
    """bcc W with He interstitials on the reference's W-He export (FS, four of its five tables:
    W-W #1 Ackland or #5 Derlet, W-He #4, He-W #3, He-He #2), FP64 / float-float / mixed, and
    10 FP64 MD steps."""
    stem = reference_export(tmp_path, "wangjun_w_he")
    ptype = [[ww, 4], [3, 2]]
    od = oracle.import_tables(stem, ptype, W_RU, 10000, 10000)
    t = _oracle_tables(oracle, od, W_RU)
    ft = ForceTable.imported(stem, ptype, W_RU, 10000, 10000)
    pos, ityp, L_ = _w_he(11)
    n = len(pos)
    rc_nl = W_RU + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 200)
    ref = oracle.force(pos, ityp, st, box, kv, ind, t)
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, rc_nl, mxkvois=160, precision=precision)
        e.init_forcetable(ft)
        e.set_masses(MASSES_WHE)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, ityp=ityp)
        e.calforce()
        f = e.get_force()
        if precision == "mixed":
            assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
        else:
            assert rel_err(f, ref["f"]) < TOL, precision
            e.calepot()
            assert rel_err(e.get_epot(), ref["epot"]) < TOL, precision
        e.close()
    rng = np.random.default_rng(5)
    vel = rng.normal(size=(n, 3)) * np.sqrt(600.0 * 8.617333e-5 / MASSES_WHE[ityp - 1])[:, None]
    ox, ov, _, _, _ = oracle.md(pos, vel, ityp, st, box, t, MASSES_WHE, 1.0, 10, rc_nl, skin_trigger=0.15,
                                mxkvois=200)
    e = Engine(n, rc_nl, mxkvois=160, skin_trigger=0.15)
    e.init_forcetable(ft)
    e.set_masses(MASSES_WHE)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp)
    e.run_steps(10, 1.0)
    x, v, _, _ = e.get_state()
    dx = x - ox
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < 1e-9
    e.close()
