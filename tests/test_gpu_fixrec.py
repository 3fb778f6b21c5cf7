"""The mixed force variants on the 16 B fixed-point records (coordinates as 32-bit fractions of
the box, F'(rho) in the fourth word; the table index still the density pass's exact one):
forces within the mixed bar of 1e-6 of the FP64 oracle and within 5e-7 of the variants on
the 32 B float-float records, in FS and EAM, with inactive atoms, open faces and several
boxes; MD with the fused step kernel on them, bitwise equal to the unfused step; the
fall-back to the 32 B records when an edge exceeds the records' span, and of the one-box
variants when the state has several boxes."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt
from msmpscu_gb300 import _lib as L
from tests.helpers import cu_tables, w_tables

pytestmark = pytest.mark.gpu

FORCE_FIX = [128 + 50, 128 + 51, 128 + 52, 128 + 53]
FUSED_FIX = [128 + 12, 128 + 14, 128 + 16, 128 + 32 + 16, 128 + 64 + 14, 128 + 64 + 32 + 16, 128 + 64 + 13]


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _cu_engine(n, **kw):
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="mixed", **kw)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


@pytest.mark.parametrize("force", FORCE_FIX)
def test_fix_force_pass_vs_oracle(oracle, force):
    pos, vel, L_ = lt.cu_config(14, 0.08, 900.0, 41)          # 10,976 atoms
    n = len(pos)
    st = np.ones(n, np.int32)
    st[::89] = 0
    box = oracle.make_box([0, 0, 0], L_)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, cu_tables(oracle))["f"]
    e = _cu_engine(n)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, statu=st)
    e.set_tuning(density=275, force=50, fused=-1)
    e.calforce()
    f32 = e.get_force()
    e.set_tuning(density=275, force=force, fused=-1)
    assert e.tuning()["force_variant"] == force
    e.calforce()
    ffix = e.get_force()
    e.close()
    assert _rel(ffix, ref) < 1e-6
    assert _rel(ffix, f32) < 5e-7
    assert np.all(ffix[::89] == 0.0)


def test_fix_eam_open_face_and_boxes(oracle):
    """Marinica W with a dumbbell next to a box open along z: per-box units, the open edge's
    doubled span (no wrap-around image) and the per-thread box lookup."""
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
    for force in FORCE_FIX:
        e.set_tuning(density=258, force=force, fused=-1)
        e.calforce()
        assert _rel(e.get_force(), ref) < 1e-6, force
    # one-box fused codes are refused with two boxes
    with pytest.raises(MSMError) as ei:
        e.set_tuning(density=-1, force=-1, fused=128 + 64 + 14)
    assert ei.value.code == L.ERR_ARG
    e.close()


@pytest.mark.parametrize("fused", FUSED_FIX)
def test_fix_fused_md_vs_float_float_records(oracle, fused):
    """30 MD steps with the fused step kernel on the fixed-point records against the same run
    on the 32 B records: the trajectories agree to well below the mixed force error's effect,
    and the forces at the end are within 1e-6 of the oracle's at the same positions."""
    pos, vel, L_ = lt.cu_config(12, 0.08, 1200.0, 17)
    n = len(pos)
    out = []
    for f in (14, fused):
        e = _cu_engine(n, skin_trigger=0.15)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        e.set_tuning(density=275, force=50, fused=f)
        reb = e.run_steps(30, 1.0)
        assert e.tuning()["fused_variant"] == f
        x, v, _, _ = e.get_state()
        out.append((x, v, e.get_force(), reb))
        e.close()
    (xa, va, fa, ra), (xb, vb, fb, rb) = out
    dx = xb - xa
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < 1e-6
    assert ra == rb
    st = np.ones(n, np.int32)
    box = oracle.make_box([0, 0, 0], L_)
    kv, ind = oracle.nlist(xb, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(xb, st, st, box, kv, ind, cu_tables(oracle))["f"]
    assert _rel(fb, ref) < 1e-6


def test_fix_records_off_beyond_their_span(oracle):
    """A box of 20,000 A along x: the fixed-point records are off, their codes are refused and
    the autotuner picks a 32 B-record variant; the forces stay within the mixed bar."""
    p, L_ = lt.fcc(8, 8, 8, lt.CU_A)
    p = p + np.random.default_rng(12).normal(scale=0.06, size=p.shape)
    p -= np.floor(p / L_) * L_
    p[:, 0] += 15000.0
    Lb = (20000.0, float(L_[1]), float(L_[2]))
    n = len(p)
    box = oracle.make_box([0, 0, 0], Lb, ifpd=(0, 1, 1))
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(p, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(p, st, st, box, kv, ind, cu_tables(oracle))["f"]
    e = _cu_engine(n)
    e.copyin([(n, (0, 0, 0), Lb, (0, 1, 1))], p)
    for code in (dict(force=128 + 50, fused=-1), dict(force=-1, fused=128 + 16)):
        with pytest.raises(MSMError) as ei:
            e.set_tuning(density=-1, **code)
        assert ei.value.code == L.ERR_ARG
    e.calforce()                     # autotuned
    t = e.tuning()
    assert t["force_variant"] < 128
    assert _rel(e.get_force(), ref) < 1e-6
    e.close()


def test_one_box_variants_fall_back_with_several_boxes(oracle):
    """Variants tuned on a one-box state keep working after a copy-in of the same atom count in
    two boxes: the one-box codes run the per-thread-box loop instead."""
    pos, vel, L_ = lt.cu_config(10, 0.05, 600.0, 9)          # 4,000 atoms
    n = len(pos)
    e = _cu_engine(n, max_boxes=2, skin_trigger=0.15)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.set_tuning(density=915, force=128 + 50, fused=128 + 64 + 32 + 16)
    e.run_steps(5, 1.0)
    # the same atoms as two boxes: the halves of the box along x, open there
    half = L_[0] / 2.0
    sel = pos[:, 0] < half
    p2 = np.vstack([pos[sel], pos[~sel]])
    v2 = np.vstack([vel[sel], vel[~sel]])
    b2 = [(int(sel.sum()), (0, 0, 0), (half, L_[1], L_[2]), (0, 1, 1)),
          (int((~sel).sum()), (half, 0, 0), (half, L_[1], L_[2]), (0, 1, 1))]
    e.copyin(b2, p2, v2)
    e.calforce()
    f = e.get_force()
    x, _, _, _ = e.get_state()
    refs = []
    off = 0
    for (cnt, lo, ln, pd) in b2:
        xs = x[off:off + cnt]
        box = oracle.make_box(list(lo), list(ln), ifpd=pd)
        st = np.ones(cnt, np.int32)
        kv, ind = oracle.nlist(xs, st, box, lt.CU_RC_NL, 96)
        refs.append(oracle.force(xs, st, st, box, kv, ind, cu_tables(oracle))["f"])
        off += cnt
    assert _rel(f, np.vstack(refs)) < 1e-6
    e.run_steps(5, 1.0)
    e.close()


@pytest.mark.parametrize("fused", [128 + 64 + 32 + 15, 128 + 32 + 15])
def test_fused_step_equals_unfused_step_bitwise(fused):
    """The fused step kernel on the fixed-point records against the unfused step (the
    integrator kernel, the density pass and the fixed-point force pass, forced by a zero
    external field): the same forces, corrector and predictor arithmetic, so bitwise the same
    trajectory, forces and list rebuilds."""
    pos, vel, L_ = lt.cu_config(12, 0.08, 1200.0, 29)
    n = len(pos)
    out = []
    for zero_field in (False, True):
        e = _cu_engine(n, skin_trigger=0.15)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        e.set_tuning(density=275, force=128 + 52, fused=fused)
        if zero_field:
            e.set_extforce_field(np.zeros((n, 3)))
        reb = e.run_steps(40, 1.0)
        x, v, _, dis = e.get_state()
        out.append((x, v, dis, e.get_force(), reb))
        e.close()
    for u, w in zip(out[0][:4], out[1][:4]):
        assert np.array_equal(u, w)
    assert out[0][4] == out[1][4] and out[0][4] > 0
