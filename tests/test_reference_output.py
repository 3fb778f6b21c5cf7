"""The oracle against forces and energies the reference itself computed: the 2,001-atom W + H
box (Bonny W-H-He EAM, subtype EAM1) at step 0 of the reference's GMD run in examples/NEB_Test
(tests/golden/make_golden_neb.py), evaluated with that run's parameters (RU = 1.9 LU, tables of
10,000 points up to RU, neighbour cutoff 1.2 RU, periodic box of 10 LU).

The file prints 9 digits and was written by the reference of 2019: per-atom energies agree to
1e-6 eV (1e-7 of the W cohesive energy), forces on W atoms farther than 8 A from the H atom to
4e-6 eV/A, and forces next to the H atom to ~8e-5 eV/A: the residual sits at the W-H terms,
which that version may evaluate slightly differently from the current reference (the oracle's
source, pinned to its table exports).  The bars below sit a few times above those figures; a planted mistake (the H atom
evaluated as W) must break them."""
import numpy as np
import pytest

from tests.helpers import NEB_PTYPE, neb_far_from_h, neb_reference_configs

E_ATOM = 2e-6       # eV, per-atom energy
E_TOTAL = 1e-3      # eV, total over 2,001 atoms (~17,800 eV)
F_FAR = 1e-5        # eV/A, W atoms farther than 8 A from H
F_ALL = 2e-4        # eV/A, every atom


def _oracle_tables(oracle, ru):
    t = oracle.bonny_tables(1, rmax=ru)
    return oracle.RawTables(oracle.EAM, 10000, t["nkind"], ru, ru, t["potr"], t["fpotr"], t["potb"], t["fpotb"],
                            NEB_PTYPE, fembd=t["fembd"], dfembd=t["dfembd"], kembd=np.array([1, 2], np.int32),
                            rhod=t["rhod"])


def _evaluate(oracle, c, typ):
    tab = _oracle_tables(oracle, c["ru"])
    box = oracle.make_box(c["lo"], c["length"])
    st = np.ones(len(typ), np.int32)
    kv, ind = oracle.nlist(c["pos"], st, box, c["rc_nl"], 256)
    r = oracle.force(c["pos"], typ, st, box, kv, ind, tab)
    assert r["nbad"] == 0
    return r


@pytest.fixture(scope="module")
def configs():
    return neb_reference_configs()


@pytest.mark.parametrize("k", [0, 1])
def test_oracle_matches_reference_output(oracle, configs, k):
    c = configs[k]
    r = _evaluate(oracle, c, c["typ"])
    far = neb_far_from_h(c)
    df = np.abs(r["f"] - c["force"])
    assert np.abs(r["epot"] - c["epot"]).max() < E_ATOM
    assert abs(r["epot"].sum() - c["epot"].sum()) < E_TOTAL
    assert df[far].max() < F_FAR
    assert df.max() < F_ALL


def test_planted_mistake_breaks_the_bars(oracle, configs):
    c = configs[0]
    r = _evaluate(oracle, c, np.ones_like(c["typ"]))        # the H atom as W
    df = np.abs(r["f"] - c["force"])
    assert df.max() > 10 * F_ALL
    assert np.abs(r["epot"] - c["epot"]).max() > 10 * E_ATOM
