"""The TMA-streamed variants of the mixed MD step kernel (list tiles moved into shared memory
by cp.async.bulk.tensor behind mbarriers) against the variants that load the list slots
directly with the same arithmetic in the same order: identical trajectories.  Also the
failure path of the bounded waits."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt
from msmpscu_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _run(pos, vel, L_, fused, steps=20):
    n = len(pos)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="mixed")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    e.set_tuning(density=3, force=20, fused=fused)
    e.run_steps(steps, 1.0)
    x, v, _, _ = e.get_state()
    f = e.get_force()
    assert e.tuning()["fused_variant"] == fused
    e.close()
    return x, v, f


@pytest.mark.parametrize("ncell", [7, 40])        # 1,372 atoms (a partial last block), 256,000
@pytest.mark.parametrize("tma,direct", [(18, 12), (19, 13)])
def test_tma_step_kernel_matches_direct_loads(ncell, tma, direct):
    pos, vel, L_ = lt.cu_config(ncell, 0.05, 600.0, 77)
    xa, va, fa = _run(pos, vel, L_, direct)
    xb, vb, fb = _run(pos, vel, L_, tma)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa, fb)


def test_bounded_wait_reports_timeout_and_context_survives():
    pos, vel, L_ = lt.cu_config(6, 0.05, 300.0, 3)
    n = len(pos)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision="mixed")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    with pytest.raises(MSMError) as ei:
        e._ck(e.lib.msmgb_selftest_wait(e.ctx))
    assert ei.value.code == L.ERR_TIMEOUT
    e.calforce()                                        # the context is still usable
    assert np.isfinite(e.get_force()).all()
    e.close()
