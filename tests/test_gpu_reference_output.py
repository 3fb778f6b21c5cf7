"""The library against forces and energies the reference itself computed (the 2,001-atom W + H
box of the reference's NEB example at step 0, Bonny EAM1; tests/test_reference_output.py
states the configuration and the bars).  The FP64 and float-float passes reproduce every
printed force component and per-atom energy to its last digit (float-float: within FF_SLACK
more, its own error of ~5e-13 of the force, for components the FP64 value sits at the
rounding edge of) and match the oracle to 1e-10; the mixed passes give the energies (FP64
passes) to the last digit and the forces within their FP32 pair terms' error, MIXED_F."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, forcelib, lattice as lt
from tests.helpers import NEB_PTYPE, neb_reference_configs, rel_err
from tests.test_reference_output import _evaluate, digit_ratios

pytestmark = pytest.mark.gpu

MIXED_F = 1e-6      # eV/A, largest |F - F_ref| of the mixed force passes (FP32 pair terms)
FF_SLACK = 1e-12    # eV/A on top of the printed digits' tolerance, float-float forces


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("precision", ["fp64", "ff", "mixed"])
def test_library_reproduces_reference_output(oracle, k, precision):
    c = neb_reference_configs()[k]
    n = len(c["typ"])
    ft = forcelib.create("EAM_WHeH_Bonny_JPCM26_2014", ru=c["ru"], rmax=c["rmax"], ptype=NEB_PTYPE,
                         subtype="EAM1")
    e = Engine(n, c["rc_nl"], mxkvois=160, precision=precision)
    e.init_forcetable(ft)
    e.set_masses(np.array([183.84, 1.008]) * lt.AMU)
    e.copyin([(n, tuple(c["lo"]), tuple(c["length"]), (1, 1, 1))], c["pos"], ityp=c["typ"])
    e.calforce()
    f = e.get_force()
    e.calepot()
    ep = e.get_epot()
    e.close()
    rf, re = digit_ratios(c, f, ep)
    assert re <= 1.0, precision
    df = np.abs(f - c["force"])
    if precision == "mixed":
        assert df.max() < MIXED_F
    else:
        assert np.all(df <= c["force_tol"] + (FF_SLACK if precision == "ff" else 0.0)), precision
        r = _evaluate(oracle, c)
        assert rel_err(f, r["f"]) < 1e-10
        assert rel_err(ep, r["epot"]) < 1e-10
