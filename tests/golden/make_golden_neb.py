"""Fixture of forces and energies the reference itself computed, for a 2,001-atom W + H box.

Source in the reference tree: examples/NEB_Test/GMD/ReactP0000_0001.0000 and
ProductP0000_0001.0000, the step-0 configurations that the reference's GMD application wrote
(&BOXCFG18 format, 2019-01-03) for the NEB example Setup_test1.dat: box file
W_2000_H1_EAM1_box.dat (2,000 W + 1 H, potential library EAM_WHeH_Bonny_JPCM26_2014 subtype
EAM1, tables W: 1 2, H: 4 5), control file CtrlFile0K.dat (cutoff RU = 1.9 lattice units,
TABLESIZE 10000, neighbour cutoff NB_RM = 1.2 RU, periodic).  At step 0 the forces and
energies in the file are the reference's evaluation at the positions it prints, which are
the initial configuration's 5-digit decimals (in lattice units, LATT = 3.14 A).  The version
that wrote them gridded the tables up to max NB_RM (the form left commented at
MD_TypeDef_ForceTable.F90:591); with that grid they are reproduced to their printed digits.
The later records (.0001) print the quenched positions with forces of another iteration, so
they are not used.

Per atom the file holds TYPE, POS (LU), VEL, STATU, FOR (eV/LU), POT (eV, printed as -EPOT),
K.E., DISPLACE.  Writes neb_w2000h1_bonny_eam1.npz with, per configuration, the types, the
positions in LU, the forces in eV/LU, the printed POT column and the box (LATT, BOXLOW and
BOXSIZE in LU).  Run once in a container that has the reference mounted; the output is
committed.
"""
import os
import sys

import numpy as np

# root of the reference tree: $MSMPSCU_REFERENCE, else where this container mounts it;
# a first command-line argument overrides it
REF_ROOT = os.environ.get("MSMPSCU_REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
FILES = ("ReactP0000_0001.0000", "ProductP0000_0001.0000")


def read_boxcfg(path):
    """&BOXCFG18 record: header keys, then one row of 16 numbers per atom."""
    rows, latt, low, size = [], None, None, None
    for ln in open(path):
        s = ln.split()
        if ln.startswith("&LATT"):
            latt = float(s[-1])
        elif ln.startswith("&BOXLOW"):
            low = [float(v) for v in s[-3:]]
        elif ln.startswith("&BOXSIZE"):
            size = [float(v) for v in s[-3:]]
        elif len(s) == 16 and s[0].isdigit():
            rows.append([float(v) for v in s])
    a = np.array(rows)
    return dict(typ=a[:, 0].astype(np.int32), pos=a[:, 1:4], statu=a[:, 7].astype(np.int32),
                force=a[:, 8:11], pot=a[:, 11], latt=latt, boxlow=np.array(low), boxsize=np.array(size))


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else REF_ROOT
    out = {}
    for k, name in enumerate(FILES):
        d = read_boxcfg(os.path.join(root, "examples/NEB_Test/GMD", name))
        assert len(d["typ"]) == 2001 and (d["typ"] == 2).sum() == 1 and np.all(d["statu"] == 1)
        for key, v in d.items():
            out["c%d_%s" % (k, key)] = np.asarray(v)
    np.savez_compressed(os.path.join(HERE, "neb_w2000h1_bonny_eam1.npz"), **out)
    print("wrote", len(FILES), "configurations")


if __name__ == "__main__":
    main()
