"""External forces between the force pass and the corrector (AddExtForce_ForceClass0 and
Cumulate_ExtForce0, MDLIB/sor/CommonGPU/MD_ForceClass_Register_GPU.F90:584-606, 636-656,
982-1180): a constant per-atom field (msmgb_set_extforce_field) and registered routines
(msmgb_add_extforce).  The trajectory with a field must match the oracle's, which adds the
same field after each force evaluation: FP64 and float-float within 1e-8 A over 50 steps;
mixed forces within 1e-6 of the oracle's at the same positions."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt
from msmpscu_gb300 import _lib as L
from tests.helpers import cu_tables, rel_err

pytestmark = pytest.mark.gpu


def _state(seed=3):
    pos, vel, L_ = lt.cu_config(10, 0.05, 600.0, seed)        # 4,000 atoms
    n = len(pos)
    rng = np.random.default_rng(seed)
    # a uniform field plus a per-atom random part (e.g. a boost or a coupling term)
    fext = np.array([0.05, -0.02, 0.01]) + 0.02 * rng.normal(size=(n, 3))
    return pos, vel, L_, fext


def _engine(n, prec):
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision=prec, skin_trigger=0.15)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


@pytest.mark.parametrize("prec", ["fp64", "ff"])
def test_extfield_trajectory_matches_oracle(oracle, prec):
    pos, vel, L_, fext = _state()
    n = len(pos)
    st = np.ones(n, np.int32)
    st[::211] = 0                                          # inactive atoms get no field
    box = oracle.make_box([0, 0, 0], L_)
    ox, ov, of, _, oreb = oracle.md(pos, vel, np.ones(n, np.int32), st, box, cu_tables(oracle),
                                    np.array([lt.CU_MASS]), 1.0, 50, lt.CU_RC_NL, skin_trigger=0.15,
                                    mxkvois=96, fext=fext)
    e = _engine(n, prec)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, statu=st)
    e.set_extforce_field(fext)
    nreb = e.run_steps(50, 1.0)
    x, v, _, _ = e.get_state()
    dx = x - ox
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < 1e-8
    assert rel_err(e.get_force(), of) < 1e-8
    assert nreb == oreb
    # the field changed the run: it is not the field-free one
    oxf, _, _, _, _ = oracle.md(pos, vel, np.ones(n, np.int32), st, box, cu_tables(oracle),
                                np.array([lt.CU_MASS]), 1.0, 50, lt.CU_RC_NL, skin_trigger=0.15, mxkvois=96)
    d0 = oxf - ox
    d0 -= np.round(d0 / L_) * L_
    assert np.abs(d0).max() > 1e-5
    e.close()


def test_extfield_mixed_forces_and_clear(oracle):
    pos, vel, L_, fext = _state(5)
    n = len(pos)
    e = _engine(n, "mixed")
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.set_extforce_field(fext)
    e.run_steps(30, 1.0)
    x, _, _, _ = e.get_state()
    f = e.get_force()
    st = np.ones(n, np.int32)
    box = oracle.make_box([0, 0, 0], L_)
    kv, ind = oracle.nlist(x, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(x, st, st, box, kv, ind, cu_tables(oracle))["f"]
    assert np.abs(f - (ref + fext)).max() / np.abs(ref + fext).max() < 1e-6
    # removing the field restores the plain forces (and the fused step)
    e.set_extforce_field(None)
    e.calforce()
    assert np.abs(e.get_force() - ref).max() / np.abs(ref).max() < 1e-6
    e.run_steps(5, 1.0)
    e.close()


def test_extforce_routine_called_and_errors():
    """A registered routine sees the context's stream and device arrays after every force
    pass; inside MD it is called while the step graph is built (its device work is replayed),
    not once per step; a nonzero return fails the call with its tag in the message."""
    pos, vel, L_, _ = _state(7)
    n = len(pos)
    e = _engine(n, "mixed")
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    seen = []

    def routine(view):
        seen.append((view.n, view.nbox, view.stream,
                     bool(view.fx and view.fy and view.fz and view.pos and view.gid)))
        return 0

    e.add_extforce("probe", routine)
    e.calforce()
    assert seen == [(n, 1, e.stream, True)]
    e.run_steps(20, 1.0)
    calls_md = len(seen) - 1
    assert 1 <= calls_md <= 3                 # capture of the step graph, not 20 calls
    e.run_steps(20, 1.0)
    assert len(seen) - 1 == calls_md          # the graph is reused
    e.clear_extforce()
    e.add_extforce("failing", lambda view: 3)
    with pytest.raises(MSMError) as ei:
        e.calforce()
    assert ei.value.code == L.ERR_ARG and "failing" in str(ei.value)
    e.clear_extforce()
    e.calforce()
    e.close()
