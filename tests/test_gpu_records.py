"""The float-float position records (hi on the positions' quantum q, lo the rest) that the list
prefilter, the list's band decision and the reduced-precision passes read, checked on the
device against the FP64 positions after MD (msmgb_check_records): hi a multiple of q,
|lo| <= q/2 and hi + lo within q (2^-26 + 2^-33) of x - lo_box + L, the bound of the split
through the fixed-point form of the coordinate, in every precision, for the smallest quantum
(2^-7 A) and a coarser one (a 20,000 A edge: 2^-6 A), with open faces."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt
from msmpscu_gb300 import _lib as L

pytestmark = pytest.mark.gpu

BOUND = 2.0 ** -26 + 2.0 ** -33


def _engine(n, precision, **kw):
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision=precision, skin_trigger=0.15, **kw)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


@pytest.mark.parametrize("precision", ["mixed", "ff", "fp64"])
def test_records_after_md(precision):
    pos, vel, L_ = lt.cu_config(12, 0.08, 1200.0, 5)        # 6,912 atoms
    n = len(pos)
    e = _engine(n, precision)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    err0, bad0 = e.check_records()
    reb = e.run_steps(60, 1.0)
    err, bad = e.check_records()
    e.close()
    assert reb > 0
    assert bad0 == 0 and bad == 0
    assert 0.0 < err <= BOUND and err0 <= BOUND


def test_records_coarse_quantum_open_faces():
    """A box of 20,000 A along x, open there and along z, shifted away from the origin: the
    positions' quantum is 2^-6 A (3 L / 2^22 above 2^-7) and the frame offset L - lo_box is not
    a round number."""
    p, L_ = lt.fcc(8, 8, 8, lt.CU_A)
    p = p + np.random.default_rng(12).normal(scale=0.06, size=p.shape)
    p -= np.floor(p / L_) * L_
    lo = (-7321.25, 13.5, 2.0)
    Lb = (20000.0, float(L_[1]), float(L_[2]) + 6.0)
    p = p + np.array([15000.0 + lo[0], lo[1], lo[2] + 3.0])
    n = len(p)
    vel = np.random.default_rng(3).normal(scale=0.01, size=p.shape)
    e = _engine(n, "mixed")
    e.copyin([(n, lo, Lb, (0, 1, 0))], p, vel)
    e.run_steps(40, 1.0)
    err, bad = e.check_records()
    e.close()
    assert bad == 0
    assert 0.0 < err <= BOUND


def test_check_records_needs_a_state():
    e = _engine(100, "mixed")
    with pytest.raises(MSMError) as ei:
        e.check_records()
    assert ei.value.code == L.ERR_ARG
    e.close()
