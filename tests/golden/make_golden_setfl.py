"""Fixtures that pin the setfl import (tabulated EAM) against the reference's own export.

Sources in the reference tree:
  examples/NIST_Potentials/Cu_EAM/Cu1.eam.fs.setfl       input: Mendelev et al. Cu (setfl layout)
  examples/NIST_Potentials/Cu_EAM/Cu1.eam.fs.setfl.pair  pair tables the reference generated
  examples/NIST_Potentials/Cu_EAM/Cu1.eam.fs.setfl.embd  embedding table it generated
(written by Export_ForceTable, MD_TypeDef_ForceTable.F90:1315-1459: columns r [A],
r*phi [eV*A] (= 2 POTR), -r*dphi/dr [eV], rho, -drho/dr [1/A]; embedding rho, F [eV] and
dF/drho multiplied by the reference's eV->erg constant 1.60219e-12).

Writes:
  cu1_setfl_data.npz  the file's grids and its F(rho), rho(r), r*phi(r) arrays (the spline
                      input), so the tests need no reference tree
  cu1_setfl_rows.txt  selected pair rows (r >= 0.24 A: below 0.1 A the file holds 1e12
                      placeholders) and embedding rows

Run once in a container that has the reference mounted; the outputs are committed.
"""
import os
import sys

import numpy as np

# root of the reference tree: $MSMPSCU_REFERENCE, else where this container mounts it;
# the first command-line argument overrides the whole path
REF_ROOT = os.environ.get("MSMPSCU_REFERENCE", "/root/reference")
REF = os.path.join(REF_ROOT, "examples/NIST_Potentials/Cu_EAM")
HERE = os.path.dirname(os.path.abspath(__file__))


def read_setfl_arrays(path):
    lines = open(path).read().split("\n")
    g = lines[4].split()
    toks = " ".join(lines[5:]).split()
    nrho, drho, nr, dr, cutoff = int(g[0]), float(g[1]), int(g[2]), float(g[3]), float(g[4])
    head = toks[:4]
    vals = np.array([float(x) for x in toks[4:4 + nrho + 2 * nr]])
    return dict(nrho=nrho, drho=drho, nr=nr, dr=dr, cutoff=cutoff, z=int(float(head[0])),
                mass=float(head[1]), alat=float(head[2]), lattice=head[3],
                frho=vals[:nrho], rhor=vals[nrho:nrho + nr], rphi=vals[nrho + nr:nrho + 2 * nr],
                header=lines[:5])


def rows(path, ncol):
    out = {}
    for line in open(path):
        p = line.split()
        if p and p[0].isdigit() and len(p) >= ncol + 1:
            out[int(p[0])] = p[1:ncol + 1]
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else REF
    d = read_setfl_arrays(os.path.join(ref, "Cu1.eam.fs.setfl"))
    np.savez_compressed(os.path.join(HERE, "cu1_setfl_data.npz"), frho=d["frho"], rhor=d["rhor"],
                        rphi=d["rphi"], grid=np.array([d["nrho"], d["drho"], d["nr"], d["dr"], d["cutoff"]]),
                        atom=np.array([d["z"], d["mass"], d["alat"]]))
    pr = rows(os.path.join(ref, "Cu1.eam.fs.setfl.pair"), 5)
    er = rows(os.path.join(ref, "Cu1.eam.fs.setfl.embd"), 3)
    keep_p = sorted(set(list(range(2000, 10001, 20)) + list(range(6440, 6470)) + [9999, 10000]))
    keep_e = sorted(set(list(range(1, 200)) + list(range(200, 10001, 50)) + [10000]))
    with open(os.path.join(HERE, "cu1_setfl_rows.txt"), "w") as fh:
        fh.write("# Cu1.eam.fs.setfl exports of the reference (NTAB = 10000, Rmax = 6 A; NEMBD = 10000, RHOD = 0.03)\n")
        fh.write("# P index r_A rphi_eVA mrdphidr_eV rho mdrhodr_perA\n")
        for i in keep_p:
            fh.write("P %d %s\n" % (i, " ".join(pr[i])))
        fh.write("# E index rho F_eV dFdrho_times_1.60219e-12\n")
        for i in keep_e:
            fh.write("E %d %s\n" % (i, " ".join(er[i])))
    print("wrote", len(keep_p), "pair rows,", len(keep_e), "embedding rows")


if __name__ == "__main__":
    main()
