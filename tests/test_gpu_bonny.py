"""GPU parity with the reference's Bonny W-H-He EAM (EAM1: H and He pair-only; EAM2: H
embedded in the W density, an asymmetric KPAIR density) on bcc W with tetrahedral H and He
interstitials and substitutional He.  The oracle tabulates the functions independently."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

RC = 5.4604375
MASSES = np.array([183.84, 1.008, 4.0026]) * lt.AMU


def _w_h_he(seed):
    rng = np.random.default_rng(seed)
    pos, L_ = lt.bcc(8, 8, 8, lt.W_A)
    n0 = len(pos)
    ityp = np.ones(n0, np.int32)
    ityp[rng.choice(n0, 10, replace=False)] = 3                       # substitutional He
    a = lt.W_A
    cells = rng.choice(512, 24, replace=False)
    extra = [a * np.array([c % 8, (c // 8) % 8, c // 64], float) + a * np.array([0.25, 0.5, 0.0]) for c in cells]
    etyp = [2] * 16 + [3] * 8                                          # tetrahedral H and He
    pos = np.vstack([pos, np.array(extra)]) + rng.normal(scale=0.03, size=(n0 + len(extra), 3))
    pos -= np.floor(pos / L_) * L_
    return pos, np.concatenate([ityp, np.array(etyp, np.int32)]), L_


def _oracle_tables(oracle, sub):
    t = oracle.bonny_tables(sub)
    return oracle.RawTables(oracle.EAM, 10000, t["nkind"], RC, RC, t["potr"], t["fpotr"], t["potb"], t["fpotb"],
                            t["kpair"], fembd=t["fembd"], dfembd=t["dfembd"], kembd=t["kembd"], rhod=t["rhod"])


@pytest.mark.parametrize("sub", ["EAM1", "EAM2"])
def test_bonny_force_parity(oracle, sub):
    ft = ForceTable.bonny_wheh(sub, rmax=RC)
    t = _oracle_tables(oracle, 1 if sub == "EAM1" else 2)
    pos, ityp, L_ = _w_h_he(11)
    n = len(pos)
    rc_nl = RC + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 200)
    ref = oracle.force(pos, ityp, st, box, kv, ind, t)
    assert ref["nbad"] == 0
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, rc_nl, mxkvois=128, precision=precision)
        e.init_forcetable(ft)
        e.set_masses(MASSES)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, ityp=ityp)
        e.calforce()
        f = e.get_force()
        if precision == "mixed":
            assert np.abs(f - ref["f"]).max() / np.abs(ref["f"]).max() < 1e-6
        else:
            assert rel_err(f, ref["f"]) < 1e-10, precision
            assert rel_err(e.get_den(), ref["den"]) < 1e-10, precision
            e.calepot()
            assert rel_err(e.get_epot(), ref["epot"]) < 1e-10, precision
        e.close()


def test_bonny_eam2_md_parity(oracle):
    ft = ForceTable.bonny_wheh("EAM2", rmax=RC)
    t = _oracle_tables(oracle, 2)
    pos, ityp, L_ = _w_h_he(12)
    n = len(pos)
    rng = np.random.default_rng(5)
    vel = rng.normal(size=(n, 3)) * np.sqrt(300.0 * 8.617333e-5 / MASSES[ityp - 1])[:, None]
    rc_nl = RC + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    ox, ov, _, _, _ = oracle.md(pos, vel, ityp, st, box, t, MASSES, 0.5, 10, rc_nl, skin_trigger=0.15,
                                mxkvois=200)
    e = Engine(n, rc_nl, mxkvois=128, skin_trigger=0.15)
    e.init_forcetable(ft)
    e.set_masses(MASSES)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp)
    e.run_steps(10, 0.5)
    x, v, _, _ = e.get_state()
    dx = x - ox
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < 1e-10
    assert rel_err(v, ov) < 1e-9
    e.close()
