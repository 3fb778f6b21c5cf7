"""Bonny W-H-He EAM (EAM_WHeH_Bonny_JPCM26_2014): the oracle's tables are pinned against the
embedding table the reference exported for subtype EAM1 (which also fixes RHOD, i.e. the
gauge-transformed W density maximum), and the library's table builder reproduces the oracle's
tables for both subtypes."""
import os

import numpy as np
import pytest

from msmpscu_gb300 import ForceTable

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bonny_embd_rows.txt")
EVERG = 1.60219e-12


def test_oracle_bonny_embedding_matches_reference_export(oracle):
    te = oracle.bonny_tables(1, ntab=2000, nembd=10000)     # NEMBD = 10000 as in the export
    rows = {}
    for line in open(GOLDEN):
        f = line.split()
        if f and f[0] == "E":
            rows[int(f[1])] = [float(x) for x in f[2:]]
    assert len(rows) > 380
    rhod = te["rhod"]
    for i, (rho, f, df) in rows.items():
        assert rho == pytest.approx((i - 1) * rhod, rel=1e-8, abs=1e-15), i
        assert te["fembd"][i - 1, 0] == pytest.approx(f, rel=6e-9, abs=1e-12), i
        assert te["dfembd"][i - 1, 0] * EVERG == pytest.approx(df, rel=6e-9, abs=1e-20), i
    assert not te["fembd"][:, 1:].any()


@pytest.mark.parametrize("sub", ["EAM1", "EAM2"])
def test_library_bonny_tables_match_oracle(oracle, sub):
    s = 1 if sub == "EAM1" else 2
    ft = ForceTable.bonny_wheh(sub, ntab=4000, nembd=4000)
    t = oracle.bonny_tables(s, ntab=4000, nembd=4000)
    assert ft.nkind == t["nkind"] and ft.rhod == pytest.approx(t["rhod"], rel=1e-15)
    for k in ("potr", "fpotr", "potb", "fpotb"):
        a = getattr(ft, k).reshape(4000, ft.nkind)
        assert np.max(np.abs(a - t[k])) <= 1e-13 * max(np.max(np.abs(t[k])), 1e-300), k
    for k in ("fembd", "dfembd"):
        a = getattr(ft, k).reshape(4000, 3)
        assert np.max(np.abs(a - t[k])) <= 1e-13 * np.max(np.abs(t[k])), k
    assert np.array_equal(ft._kpair.reshape(3, 3).T, t["kpair"])
    # EAM2 only: an H host takes the W density from a W neighbour (KPAIR(H, W) = 4), not the reverse
    potb = ft.potb.reshape(4000, ft.nkind)
    if sub == "EAM2":
        assert potb[:, 3].any() and not potb[:, 1].any() and ft.fembd.reshape(-1, 3)[1:, 1].any()
    else:
        assert not potb[:, 1:].any()
