"""The library against forces and energies the reference itself computed (the 2,001-atom W + H
box of the reference's NEB example at step 0, Bonny EAM1; tests/test_reference_output.py
states the configuration and the bars): the FP64 and float-float passes within the bars the
oracle meets and within 1e-10 of the oracle, the mixed passes within the same bars."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, forcelib, lattice as lt
from tests.helpers import NEB_PTYPE, neb_far_from_h, neb_reference_configs, rel_err
from tests.test_reference_output import E_ATOM, E_TOTAL, F_ALL, F_FAR, _evaluate

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [0, 1])
@pytest.mark.parametrize("precision", ["fp64", "ff", "mixed"])
def test_library_matches_reference_output(oracle, k, precision):
    c = neb_reference_configs()[k]
    n = len(c["typ"])
    ft = forcelib.create("EAM_WHeH_Bonny_JPCM26_2014", ru=c["ru"], ptype=NEB_PTYPE, subtype="EAM1")
    e = Engine(n, c["rc_nl"], mxkvois=160, precision=precision)
    e.init_forcetable(ft)
    e.set_masses(np.array([183.84, 1.008]) * lt.AMU)
    e.copyin([(n, tuple(c["lo"]), tuple(c["length"]), (1, 1, 1))], c["pos"], ityp=c["typ"])
    e.calforce()
    f = e.get_force()
    e.calepot()
    ep = e.get_epot()
    e.close()
    far = neb_far_from_h(c)
    df = np.abs(f - c["force"])
    assert df[far].max() < F_FAR, precision
    assert df.max() < F_ALL, precision
    assert np.abs(ep - c["epot"]).max() < E_ATOM, precision
    assert abs(ep.sum() - c["epot"].sum()) < E_TOTAL, precision
    if precision != "mixed":
        r = _evaluate(oracle, c, c["typ"])
        assert rel_err(f, r["f"]) < 1e-10
        assert rel_err(ep, r["epot"]) < 1e-10
