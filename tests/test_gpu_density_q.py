"""The table-assisted mixed density pass (k_density32q: exact FP32 sum of squares on hi parts
rounded to a power-of-two quantum, sqrt(r) index from one table row holding r2_k) against the
oracle and against the Newton-index pass it replaces: the same pair codes for the force pass
up to the last quantum of DK, F'(rho) within FP32 rounding, forces within the mixed bar of
1e-6 of the FP64 oracle, in FS and EAM, with several boxes, open faces and inactive atoms."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from tests.helpers import cu_tables, w_tables

pytestmark = pytest.mark.gpu

Q_VARIANTS = [258, 259, 260, 261, 274, 275, 276, 277, 386, 387, 388, 389, 402, 403, 404, 405]
NEWTON = 2          # the Newton-index density pass, 2 neighbours in flight
FORCE = 20          # a fixed force-pass variant


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _forces(e, dens):
    e.set_tuning(density=dens, force=FORCE, fused=-1)
    e.calforce()
    return e.get_force(), e.get_den()


@pytest.mark.parametrize("dens", Q_VARIANTS)
def test_density_q_fs_matches_oracle(oracle, dens):
    pos, vel, L_ = lt.cu_config(14, 0.08, 900.0, 31)          # 10,976 atoms
    n = len(pos)
    st = np.ones(n, np.int32)
    st[::97] = 0                                             # some inactive atoms
    box = oracle.make_box([0, 0, 0], L_)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, cu_tables(oracle))
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="mixed")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, statu=st)
    f_new, d_new = _forces(e, dens)
    f_old, d_old = _forces(e, NEWTON)
    e.close()
    assert _rel(f_new, ref["f"]) < 1e-6
    assert np.all(f_new[::97] == 0.0)
    assert _rel(f_new, f_old) < 2e-7
    act = st == 1
    assert _rel(d_new[act], ref["den"][act]) < 2e-7


def test_density_q_eam_and_several_boxes(oracle):
    """Marinica W with a dumbbell next to a second, open-faced box: EAM F'(rho) interpolation,
    per-box image shifts and a box without periodicity in one direction."""
    p1, L1 = lt.w_sia_config(7, 0.05, 2)
    p2, L2 = lt.bcc(6, 6, 6, lt.W_A)
    p2 = p2 + np.random.default_rng(4).normal(scale=0.05, size=p2.shape)
    p2 -= np.floor(p2 / L2) * L2
    pos = np.vstack([p1, p2])
    boxes = [(len(p1), (0, 0, 0), tuple(L1), (1, 1, 1)), (len(p2), (0, 0, 0), tuple(L2), (1, 1, 0))]
    t = w_tables(oracle)
    refs = []
    for p, L_, pd in ((p1, L1, (1, 1, 1)), (p2, L2, (1, 1, 0))):
        box = oracle.make_box([0, 0, 0], L_, ifpd=pd)
        st = np.ones(len(p), np.int32)
        kv, ind = oracle.nlist(p, st, box, lt.W_RC_NL, 128)
        refs.append(oracle.force(p, st, st, box, kv, ind, t)["f"])
    ref = np.vstack(refs)
    e = Engine(len(pos), lt.W_RC_NL, max_boxes=2, mxkvois=96, precision="mixed")
    e.init_forcetable(ForceTable.marinica_eam2())
    e.copyin(boxes, pos)
    for dens in (258, 277, 386, 405):
        f, _ = _forces(e, dens)
        assert _rel(f, ref) < 1e-6, dens
    e.close()


def test_density_q_md_steps(oracle):
    """Mixed MD with the table-assisted density pass in the step graph: forces after 20 steps
    against the oracle's FP64 forces at the same positions."""
    pos, vel, L_ = lt.cu_config(10, 0.05, 600.0, 9)
    n = len(pos)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="mixed", skin_trigger=0.15)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.set_tuning(density=274, force=FORCE, fused=14)
    e.run_steps(20, 1.0)
    x, _, _, _ = e.get_state()
    f = e.get_force()
    assert e.tuning()["density_variant"] == 274
    e.close()
    st = np.ones(n, np.int32)
    box = oracle.make_box([0, 0, 0], L_)
    kv, ind = oracle.nlist(x, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(x, st, st, box, kv, ind, cu_tables(oracle))["f"]
    assert _rel(f, ref) < 1e-6


@pytest.mark.parametrize("dens,fused,dens_sb,fused_sb", [(275, 14, 787, 78), (403, 46, 915, 110),
                                                        (261, 16, 773, 80)])
def test_single_box_parameter_variants_bitwise(dens, fused, dens_sb, fused_sb):
    """One box: the density and fused step kernels with the box constants as kernel
    parameters against the same kernels reading them from the box array per thread: the
    same arithmetic, bitwise the same forces and trajectory."""
    pos, vel, L_ = lt.cu_config(12, 0.08, 1200.0, 17)
    n = len(pos)
    out = []
    for d, f in ((dens, fused), (dens_sb, fused_sb)):
        e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="mixed", skin_trigger=0.15)
        e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
        e.set_masses([lt.CU_MASS])
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        e.set_tuning(density=d, force=FORCE, fused=f)
        reb = e.run_steps(30, 1.0)
        x, v, _, _ = e.get_state()
        out.append((x, v, e.get_force(), reb))
        t = e.tuning()
        assert (t["density_variant"], t["fused_variant"]) == (d, f)
        e.close()
    (xa, va, fa, ra), (xb, vb, fb, rb) = out
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa, fb)
    assert ra == rb and ra > 0


def test_density_q_long_box(oracle):
    """A box of 20,000 A along x (open faces there): the hi parts of the positions take a
    coarser quantum (2^-6 A instead of 2^-7 A, so that every shifted coordinate rounds to a
    multiple of it), and the exact sums of squares, the list and the forces still hold."""
    p, L_ = lt.fcc(8, 8, 8, lt.CU_A)
    p = p + np.random.default_rng(12).normal(scale=0.06, size=p.shape)
    p -= np.floor(p / L_) * L_
    p[:, 0] += 15000.0
    L = (20000.0, float(L_[1]), float(L_[2]))
    n = len(p)
    box = oracle.make_box([0, 0, 0], L, ifpd=(0, 1, 1))
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(p, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(p, st, st, box, kv, ind, cu_tables(oracle))
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="mixed")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.copyin([(n, (0, 0, 0), L, (0, 1, 1))], p)
    for dens in (258, 277, 386, 405):
        f, d = _forces(e, dens)
        assert e.tuning()["density_variant"] == dens
        assert _rel(f, ref["f"]) < 1e-6, dens
        assert _rel(d, ref["den"]) < 2e-7, dens
    e.close()
