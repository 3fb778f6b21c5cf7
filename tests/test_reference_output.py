"""The oracle against forces and energies the reference itself computed: the 2,001-atom W + H
box (Bonny W-H-He EAM, subtype EAM1) at step 0 of the reference's GMD run in examples/NEB_Test
(tests/golden/make_golden_neb.py), evaluated with that run's parameters (RU = 1.9 LU, neighbour
cutoff NB_RM = 1.2 RU, tables of 10,000 points up to NB_RM as the version that wrote the
records had them, periodic box of 10 LU).

Every per-atom energy and every force component must reproduce its printed value to half a
unit in the ninth significant digit (forces: or to 1e-11 eV/LU, FP64 summation-order noise,
where that digit lies below it).  Planted mistakes, each on the CPU, must break the bars: the
H atom evaluated as W, and the tables gridded up to RU (the current source's RMAX) instead of
NB_RM."""
import numpy as np
import pytest

from tests.helpers import NEB_PTYPE, neb_reference_configs


def _oracle_tables(oracle, rmax, ru):
    t = oracle.bonny_tables(1, rmax=rmax)
    return oracle.RawTables(oracle.EAM, 10000, t["nkind"], rmax, ru, t["potr"], t["fpotr"], t["potb"],
                            t["fpotb"], NEB_PTYPE, fembd=t["fembd"], dfembd=t["dfembd"],
                            kembd=np.array([1, 2], np.int32), rhod=t["rhod"])


def _evaluate(oracle, c, typ=None, rmax=None):
    tab = _oracle_tables(oracle, c["rmax"] if rmax is None else rmax, c["ru"])
    box = oracle.make_box(c["lo"], c["length"])
    typ = c["typ"] if typ is None else typ
    st = np.ones(len(typ), np.int32)
    kv, ind = oracle.nlist(c["pos"], st, box, c["rc_nl"], 256)
    r = oracle.force(c["pos"], typ, st, box, kv, ind, tab)
    assert r["nbad"] == 0
    return r


def digit_ratios(c, f, epot):
    """Largest |difference| over the tolerance of the printed digits, for forces and energies."""
    return (float(np.max(np.abs(f - c["force"]) / c["force_tol"])),
            float(np.max(np.abs(epot - c["epot"]) / c["epot_tol"])))


@pytest.fixture(scope="module")
def configs():
    return neb_reference_configs()


@pytest.mark.parametrize("k", [0, 1])
def test_oracle_reproduces_reference_output_digits(oracle, configs, k):
    c = configs[k]
    r = _evaluate(oracle, c)
    rf, re = digit_ratios(c, r["f"], r["epot"])
    assert rf <= 1.0 and re <= 1.0


def test_planted_mistakes_break_the_bars(oracle, configs):
    c = configs[0]
    r = _evaluate(oracle, c, typ=np.ones_like(c["typ"]))        # the H atom as W
    rf, re = digit_ratios(c, r["f"], r["epot"])
    assert rf > 1e3 and re > 1e3
    r = _evaluate(oracle, c, rmax=c["ru"])                      # tables gridded up to RU
    rf, re = digit_ratios(c, r["f"], r["epot"])
    assert rf > 10.0 and re > 10.0
