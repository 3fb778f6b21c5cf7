"""The batched-box benchmark configuration at full size: 512 periodic Cu boxes with edges of
4..12 fcc cells (253..6,912 atoms, 1,365,955 in total), 0..3 vacancies, 300..1200 K, in one
context.  Per box: FP64 and float-float forces against the oracle at 1e-10, mixed forces
below 1e-6, and MD of the whole batch bit-identical to MD of single boxes on their own."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from tests.helpers import cu_tables, rel_err

pytestmark = pytest.mark.gpu


def _batch():
    boxes = lt.uneven_batch(512, seed=512)
    pos = np.vstack([b[0] for b in boxes])
    vel = np.vstack([b[1] for b in boxes])
    desc = [(len(b[0]), (0, 0, 0), tuple(b[2]), (1, 1, 1)) for b in boxes]
    return boxes, pos, vel, desc


def _engine(n, nbox, precision, skin=0.15):
    e = Engine(n, lt.CU_RC_NL, max_boxes=nbox, mxkvois=64, skin_trigger=skin, precision=precision)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


def test_512_uneven_boxes_forces_all_precisions(oracle):
    boxes, pos, vel, desc = _batch()
    assert len(pos) == 1365955
    t = cu_tables(oracle)
    refs = []
    for p, v, L_ in boxes:
        n = len(p)
        box = oracle.make_box([0, 0, 0], L_)
        st = np.ones(n, np.int32)
        kv, ind = oracle.nlist(p, st, box, lt.CU_RC_NL, 96)
        refs.append(oracle.force(p, st, st, box, kv, ind, t, want_virial=False, want_epot=False)["f"])
    for precision, tol in (("fp64", 1e-10), ("ff", 1e-10), ("mixed", 1e-6)):
        e = _engine(len(pos), len(boxes), precision)
        e.copyin(desc, pos, vel)
        e.calforce()
        f = e.get_force()
        off, worst = 0, 0.0
        for k, ((p, v, L_), ref) in enumerate(zip(boxes, refs)):
            sl = slice(off, off + len(p))
            worst = max(worst, rel_err(f[sl], ref))
            # momentum: FP64-class passes to rounding, the mixed passes to FP32 rounding
            mtol = (1e-6 if precision == "mixed" else 1e-9) * len(p) * np.abs(ref).max()
            assert np.abs(f[sl].sum(0)).max() < mtol, (precision, k)
            off += len(p)
        assert worst < tol, (precision, worst)
        e.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_512_boxes_md_equals_single_box_md(precision):
    """10 NVE steps of the batch against the same boxes run in contexts of their own.  The
    rebuild trigger is a maximum over a whole context, so it is set out of reach here: with
    the initial lists kept, the FP64 batch is bit-identical to the single boxes (the passes and
    the list order of a box do not depend on the other boxes); the mixed passes are tuned per
    atom count and may pick another kernel variant, so they agree to FP32 rounding."""
    boxes, pos, vel, desc = _batch()
    e = _engine(len(pos), len(boxes), precision, skin=10.0)
    e.copyin(desc, pos, vel)
    e.run_steps(10, 1.0)
    gx, gv, _, _ = e.get_state()
    e.close()
    offs = np.concatenate([[0], np.cumsum([len(b[0]) for b in boxes])])
    rng = np.random.default_rng(3)
    for k in rng.choice(len(boxes), 6, replace=False):
        p, v, L_ = boxes[k]
        s = _engine(len(p), 1, precision, skin=10.0)
        s.copyin([desc[k]], p, v)
        s.run_steps(10, 1.0)
        x1, v1, _, _ = s.get_state()
        s.close()
        if precision == "fp64":
            assert np.array_equal(gx[offs[k]:offs[k + 1]], x1), k
            assert np.array_equal(gv[offs[k]:offs[k + 1]], v1), k
        else:
            assert np.abs(gx[offs[k]:offs[k + 1]] - x1).max() < 1e-8, k
