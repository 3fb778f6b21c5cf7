"""GPU parity with tables imported from an lspt potential: the reference's own W-H-He example
(W embedding, H and He without one, nine pair/density tables), on a bcc W box holding
substitutional and interstitial H and He.  The oracle tabulates independently from the same
files."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from tests.helpers import rel_err
from tests.lspt_util import whhe

pytestmark = pytest.mark.gpu

TOL = 1e-10
MASSES = np.array([183.84, 1.008, 4.0026]) * lt.AMU


def _w_h_he(seed):
    rng = np.random.default_rng(seed)
    pos, L_ = lt.bcc(8, 8, 8, lt.W_A)
    n0 = len(pos)
    ityp = np.ones(n0, np.int32)
    sub = rng.choice(n0, 40, replace=False)
    ityp[sub[:24]] = 2                                   # substitutional H
    ityp[sub[24:]] = 3                                   # substitutional He
    cells = rng.choice(512, 12, replace=False)
    a = lt.W_A
    extra, etyp = [], []
    for c, cell in enumerate(cells):
        o = a * np.array([cell % 8, (cell // 8) % 8, cell // 64], float)
        if c < 8:
            extra.append(o + a * np.array([0.25, 0.5, 0.0]))   # tetrahedral H
            etyp.append(2)
        else:
            extra.append(o + a * np.array([0.5, 0.5, 0.0]))    # octahedral He
            etyp.append(3)
    pos = np.vstack([pos, np.array(extra)]) + rng.normal(scale=0.03, size=(n0 + len(extra), 3))
    pos -= np.floor(pos / L_) * L_
    return pos, np.concatenate([ityp, np.array(etyp, np.int32)]), L_


def _oracle_tables(oracle, path, ntab=10000):
    t = oracle.lspt_tables(oracle.read_lspt(path), ntab=ntab)
    return oracle.RawTables(oracle.EAM, ntab, 9, t["rmax"], t["rmax"], t["potr"], t["fpotr"], t["potb"],
                            t["fpotb"], t["kpair"], fembd=t["fembd"], dfembd=t["dfembd"], kembd=t["kembd"],
                            rhod=t["rhod"]), t["rmax"]


def test_lspt_whhe_force_parity(oracle, tmp_path):
    path = whhe(str(tmp_path))
    ft = ForceTable.lspt(path)
    t, rmax = _oracle_tables(oracle, path)
    pos, ityp, L_ = _w_h_he(3)
    n = len(pos)
    rc_nl = rmax + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 160)
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
            assert rel_err(f, ref["f"]) < TOL, precision
            assert rel_err(e.get_den(), ref["den"]) < TOL, precision
            e.calepot()
            assert rel_err(e.get_epot(), ref["epot"]) < TOL, precision
        e.close()


def test_lspt_whhe_md_parity(oracle, tmp_path):
    """Ten FP64 velocity-Verlet steps at dt = 0.5 fs with the light atoms moving."""
    path = whhe(str(tmp_path))
    ft = ForceTable.lspt(path)
    t, rmax = _oracle_tables(oracle, path)
    pos, ityp, L_ = _w_h_he(4)
    n = len(pos)
    rng = np.random.default_rng(9)
    vel = rng.normal(size=(n, 3)) * np.sqrt(300.0 * 8.617333e-5 / MASSES[ityp - 1])[:, None]
    rc_nl = rmax + 0.3
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    ox, ov, of, _, _ = oracle.md(pos, vel, ityp, st, box, t, MASSES, 0.5, 10, rc_nl, skin_trigger=0.15,
                                 mxkvois=160)
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
