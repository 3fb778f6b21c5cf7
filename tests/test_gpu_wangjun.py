"""GPU parity with the reference's W-He FS library (EM_TB_WangJun_W-HE_2010: five tables,
KPAIR for W and He groups) on bcc W with tetrahedral He interstitials and a He pair; He hosts
have zero density (the FS F'(rho) guard), He-W pairs sit in the ab-initio cubic pieces.  The
oracle tabulates the same functions independently (Angstrom/eV restatement)."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from tests.helpers import rel_err

pytestmark = pytest.mark.gpu

RU = 6.0
MASSES = np.array([183.84, 4.0026]) * lt.AMU


def _w_he(seed):
    rng = np.random.default_rng(seed)
    pos, L_ = lt.bcc(8, 8, 8, lt.W_A)
    a = lt.W_A
    cells = rng.choice(512, 15, replace=False)
    he = [a * np.array([c % 8, (c // 8) % 8, c // 64], float) + a * np.array([0.25, 0.5, 0.0]) for c in cells]
    he.append(he[0] + np.array([1.5, 0.0, 0.0]))          # a He-He pair 1.5 A apart
    pos = np.vstack([pos, np.array(he)]) + rng.normal(scale=0.03, size=(len(pos) + len(he), 3))
    pos -= np.floor(pos / L_) * L_
    ityp = np.concatenate([np.ones(len(pos) - len(he), np.int32), np.full(len(he), 2, np.int32)])
    return pos, ityp, L_


def _oracle_tables(oracle, ww):
    pots = [oracle.POT_ACKLAND_WW, oracle.POT_HEHE_EXP6, oracle.POT_HEW_ZBL, oracle.POT_HEW_ZBL,
            oracle.POT_DERLET_WW]
    ts = [oracle.make_tables(p, None, RU, 10000, 10000, 20.0, want_embed=False) for p in pots]
    arr = {k: np.stack([t[k] for t in ts], 1) for k in ("potr", "fpotr", "potb", "fpotb")}
    kpair = np.array([[1 if ww == "ackland" else 5, 4], [3, 2]])
    return oracle.RawTables(oracle.FS, 10000, 5, RU, RU, arr["potr"], arr["fpotr"], arr["potb"],
                            arr["fpotb"], kpair)


@pytest.mark.parametrize("ww", ["ackland", "derlet"])
def test_wangjun_w_he_force_parity(oracle, ww):
    ft = ForceTable.wangjun_w_he(rmax=RU, ww=ww)
    t = _oracle_tables(oracle, ww)
    pos, ityp, L_ = _w_he(7)
    n = len(pos)
    rc_nl = RU + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 200)
    ref = oracle.force(pos, ityp, st, box, kv, ind, t)
    assert np.abs(ref["f"][ityp == 2]).max() > 1.0          # the He atoms are pushed
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, rc_nl, mxkvois=160, precision=precision)
        e.init_forcetable(ft)
        e.set_masses(MASSES)
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


def test_wangjun_w_he_md_parity(oracle):
    ft = ForceTable.wangjun_w_he(rmax=RU)
    t = _oracle_tables(oracle, "ackland")
    pos, ityp, L_ = _w_he(8)
    n = len(pos)
    rng = np.random.default_rng(3)
    vel = rng.normal(size=(n, 3)) * np.sqrt(600.0 * 8.617333e-5 / MASSES[ityp - 1])[:, None]
    rc_nl = RU + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    ox, ov, _, _, _ = oracle.md(pos, vel, ityp, st, box, t, MASSES, 1.0, 10, rc_nl, skin_trigger=0.15,
                                mxkvois=200)
    e = Engine(n, rc_nl, mxkvois=160, skin_trigger=0.15)
    e.init_forcetable(ft)
    e.set_masses(MASSES)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp)
    e.run_steps(10, 1.0)
    x, v, _, _ = e.get_state()
    dx = x - ox
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < 1e-10
    assert rel_err(v, ov) < 1e-9
    e.close()
