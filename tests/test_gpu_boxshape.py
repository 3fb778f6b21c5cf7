"""Non-cubic boxes (BOXSHAPE): separations in length units are BOXSHAPE . SEP after the minimum
image (MD_FS_ForceTable.F90:235,333, MD_NeighborsList.F90:362-364).  The FP64 calls against the
oracle's restatement of the reference's CPU path: neighbour sets, forces, virial, energies and
per-atom stress; MD and the reduced precisions refuse such a state."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt
from helpers import cu_tables, rel_err, sorted_sets

pytestmark = pytest.mark.gpu

TOL = 1e-10

SHEAR = np.array([[1.0, 0.04, 0.0], [0.0, 0.98, 0.03], [0.02, 0.0, 1.01]])
STRONG = np.array([[1.0, 0.30, 0.0], [0.0, 1.0, 0.0], [0.0, -0.25, 1.0]])


def _engine(n, nbox=1, prec="fp64"):
    e = Engine(n, lt.CU_RC_NL, max_boxes=nbox, mxkvois=96, precision=prec)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


@pytest.mark.parametrize("shape", [SHEAR, STRONG])
def test_shaped_box_fp64_parity(oracle, shape):
    pos, vel, L_ = lt.cu_config(7, 0.04, 300.0, 19)
    n = len(pos)
    st = np.ones(n, np.int32)
    box = oracle.make_box([0, 0, 0], L_, shape=shape)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 128)
    t = cu_tables(oracle)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    e = _engine(n)
    e.set_boxshape(0, shape)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.cal_neighborelist()
    gkv, gind = e.get_neighborelist()
    assert sorted_sets(gkv, gind) == sorted_sets(kv, ind)
    vir = e.calptensor()[0]
    assert rel_err(e.get_force(), ref["f"]) < TOL
    assert rel_err(vir, ref["vir"]) < TOL
    e.calepot()
    assert rel_err(e.get_epot(), ref["epot"]) < TOL
    ap = e.atomic_stress()
    ap_ref = oracle.atomic_stress(pos, np.ones(n, np.int32), st, box, kv, ind, t, ref["den"])
    assert rel_err(ap, ap_ref) < TOL
    # the shape changes the result: the cubic box gives other forces
    cub = oracle.force(pos, np.ones(n, np.int32), st, oracle.make_box([0, 0, 0], L_),
                       *oracle.nlist(pos, st, oracle.make_box([0, 0, 0], L_), lt.CU_RC_NL, 128), t)
    assert rel_err(cub["f"], ref["f"]) > 1e-3
    e.close()


def test_shaped_and_cubic_boxes_in_one_state(oracle):
    p1, v1, L1 = lt.cu_config(6, 0.04, 300.0, 3)
    p2, v2, L2 = lt.cu_config(5, 0.04, 300.0, 4)
    pos, vel = np.vstack([p1, p2]), np.vstack([v1, v2])
    e = _engine(len(pos), nbox=2)
    e.set_boxshape(1, SHEAR)
    e.copyin([(len(p1), (0, 0, 0), tuple(L1), (1, 1, 1)), (len(p2), (0, 0, 0), tuple(L2), (1, 1, 1))], pos, vel)
    e.calforce()
    f = e.get_force()
    t = cu_tables(oracle)
    for (p, L_, shape, sl) in ((p1, L1, None, slice(0, len(p1))), (p2, L2, SHEAR, slice(len(p1), len(pos)))):
        n = len(p)
        st = np.ones(n, np.int32)
        box = oracle.make_box([0, 0, 0], L_, shape=shape)
        kv, ind = oracle.nlist(p, st, box, lt.CU_RC_NL, 128)
        ref = oracle.force(p, np.ones(n, np.int32), st, box, kv, ind, t)
        assert rel_err(f[sl], ref["f"]) < TOL
    e.close()


def test_shaped_state_refuses_md_and_reduced_precision():
    pos, vel, L_ = lt.cu_config(5, 0.04, 300.0, 5)
    n = len(pos)
    e = _engine(n, prec="mixed")
    e.set_boxshape(0, SHEAR)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    with pytest.raises(MSMError):
        e.calforce()
    with pytest.raises(MSMError):
        e.run_steps(2, 1.0)
    e.set_precision("fp64")
    e.calforce()                                  # the FP64 call works on the same state
    assert np.isfinite(e.get_force()).all()
    with pytest.raises(MSMError):
        e.run_steps(2, 1.0)
    e.close()


def test_identity_shape_is_the_cubic_box():
    pos, vel, L_ = lt.cu_config(6, 0.04, 600.0, 6)
    n = len(pos)
    out = []
    for shape in (None, np.eye(3)):
        e = _engine(n, prec="mixed")
        if shape is not None:
            e.set_boxshape(0, shape)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        e.set_tuning(density=275, force=128 + 50, fused=128 + 32 + 15)   # the same variants in both
        e.run_steps(10, 1.0)
        out.append(e.get_state()[0])
        e.close()
    assert np.array_equal(out[0], out[1])
