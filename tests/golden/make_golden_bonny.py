"""Fixture that pins the Bonny W-H-He EAM tables against the reference's own export.

Source in the reference tree: examples/use_ForceTableGen/EAM_WHeH_Bonny_JPCM26_2014.embd, the
embedding tables the reference generated for subtype EAM1 (Export_ForceTable,
MD_TypeDef_ForceTable.F90:1315-1459): NEMBD = 10000 rows of rho, then F [eV] and dF/drho times
the eV->erg constant 1.60219e-12 for each of the 9 tables.  Only the W-W table has an embedding
function; the script checks that the other 8 columns are zero in every row.  Its rho grid
carries RHOD = 20 * max POTB / NEMBD, so it also pins the gauge-transformed W density.

Writes bonny_embd_rows.txt (selected rows of the W column).  Run once in a container that has
the reference mounted; the output is committed.
"""
import os
import sys

import numpy as np

# root of the reference tree: $MSMPSCU_REFERENCE, else where this container mounts it;
# the first command-line argument overrides the whole path
REF_ROOT = os.environ.get("MSMPSCU_REFERENCE", "/root/reference")
REF = os.path.join(REF_ROOT, "examples/use_ForceTableGen/EAM_WHeH_Bonny_JPCM26_2014.embd")
HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    src = sys.argv[1] if len(sys.argv) > 1 else REF
    rows = [ln.split() for ln in open(src) if ln.split() and ln.split()[0].isdigit()]
    assert len(rows) == 10000
    vals = np.array([[float(x) for x in r[2:]] for r in rows])
    assert np.all(vals[:, 2:] == 0.0)
    # both branches of the W embedding: rho_I = 1.359141225 sits near row 2551
    keep = sorted(set(list(range(1, 120)) + list(range(120, 10001, 40)) + list(range(2540, 2565)) + [10000]))
    with open(os.path.join(HERE, "bonny_embd_rows.txt"), "w") as fh:
        fh.write("# EAM_WHeH_Bonny_JPCM26_2014.embd (subtype EAM1) of the reference: NEMBD = 10000, 9 tables; "
                 "columns of tables 2-9 are zero in all rows\n")
        fh.write("# E index rho F1_eV dF1drho_times_1.60219e-12\n")
        for i in keep:
            r = rows[i - 1]
            fh.write("E %d %s %s %s\n" % (i, r[1], r[2], r[3]))
    print("wrote", len(keep), "rows")


if __name__ == "__main__":
    main()
