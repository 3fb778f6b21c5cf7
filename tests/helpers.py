"""Shared builders for the tests: the same seeded inputs go to the oracle and the library."""
import numpy as np

from msmpscu_gb300 import lattice as lt

CR_PRM = [lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")]


def cu_tables(oracle, rc=lt.CU_RC, ntab=10000):
    tabs = oracle.make_tables(oracle.POT_CR, CR_PRM, rc, ntab, ntab, 20.0, want_embed=False)
    return oracle.Tables(tabs, oracle.FS, rc)


def w_tables(oracle, rc=lt.W_RC, ntab=10000):
    tabs = oracle.make_tables(oracle.POT_MARINICA2, None, rc, ntab, ntab, 20.0, want_embed=True)
    return oracle.Tables(tabs, oracle.EAM, rc)


def sorted_sets(kvois, indi):
    return [tuple(sorted(indi[:kvois[i], i].tolist())) for i in range(len(kvois))]


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def reference_export(tmp_dir, name):
    """Writes the reference's exported table files tests/golden/ref_<name>.{pair,embd}.xz
    (byte copies of its Export_ForceTable output, see tests/golden/make_golden_import.py) into
    tmp_dir and returns their common stem."""
    import lzma
    import os
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    stem = os.path.join(str(tmp_dir), name)
    for ext in ("pair", "embd"):
        with open(os.path.join(here, "ref_%s.%s.xz" % (name, ext)), "rb") as fh:
            data = lzma.decompress(fh.read())
        with open(stem + "." + ext, "wb") as fh:
            fh.write(data)
    return stem
