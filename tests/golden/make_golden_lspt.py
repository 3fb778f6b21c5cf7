"""Fixtures that pin the lspt import (tabulated EAM from ".spt" files) against the
reference's own export.

Sources in the reference tree (examples/NIST_Potentials/WHHe_EAM1_LSPT):
  WHHe_EAM1.lspt        control file: elements W, H, He; F(rho) and rho(r) of W only ("NA"
                        for H and He); pair lines "pWW" / "pWH", "pHH" / "pWHe", "pHHe", "pHeHe"
  *.spt                 the data files: 5000 "x f(x)" rows each on a uniform grid
  WHHe_EAM1.lspt.embd   the embedding tables the reference generated from them
                        (Export_ForceTable, MD_TypeDef_ForceTable.F90:1315-1459): NEMBD = 10000
                        rows of rho, then F [eV] and dF/drho times the eV->erg constant
                        1.60219e-12 for each of the 9 tables

Writes:
  whhe_lspt_data.npz    the element symbols, the file named in each slot of the control
                        file, and per data file its f(x) column with (n, x_last) of its grid
                        (x_i = i x_last/(n-1); the files' x column matches that to 6e-15)
  whhe_lspt_embd_rows.txt  selected rows of the W embedding table (table 1); the script
                        checks that the other 8 columns are zero in every row

Run once in a container that has the reference mounted; the outputs are committed.
"""
import os
import sys

import numpy as np

# root of the reference tree: $MSMPSCU_REFERENCE, else where this container mounts it;
# the first command-line argument overrides the whole path
REF_ROOT = os.environ.get("MSMPSCU_REFERENCE", "/root/reference")
REF = os.path.join(REF_ROOT, "examples/NIST_Potentials/WHHe_EAM1_LSPT")
HERE = os.path.dirname(os.path.abspath(__file__))


def quoted(s):
    out, i = [], 0
    while i < len(s):
        if s[i] in "\"'":
            e = s.find(s[i], i + 1)
            out.append(s[i + 1:e])
            i = e + 1
        else:
            i += 1
    return out


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else REF
    lines = [ln.strip() for ln in open(os.path.join(ref, "WHHe_EAM1.lspt"))]
    lines = [ln for ln in lines if ln and not ln.startswith("!")]
    elements = [q.strip() for q in quoted(lines[2])]
    ne = len(elements)
    slots = {}
    k = 3
    for e in range(ne):
        slots["frho_%d" % e] = quoted(lines[k])[0].strip()
        slots["rhor_%d" % e] = quoted(lines[k + 1])[0].strip()
        k += 2
    for i in range(ne):
        for j, q in enumerate(quoted(lines[k])):
            slots["vr_%d_%d" % (i, j)] = q.strip()
        k += 1
    arrays = {}
    for name in sorted(set(v for v in slots.values() if v.upper() != "NA")):
        a = np.loadtxt(os.path.join(ref, name))
        n, xl = len(a), a[-1, 0]
        assert np.abs(a[:, 0] - np.arange(n) * (xl / (n - 1))).max() < 1e-14, name
        arrays["y:" + name] = a[:, 1]
        arrays["g:" + name] = np.array([n, xl])
    np.savez_compressed(os.path.join(HERE, "whhe_lspt_data.npz"), elements=np.array(elements),
                        slot_keys=np.array(list(slots.keys())), slot_files=np.array(list(slots.values())),
                        **arrays)
    rows = []
    for line in open(os.path.join(ref, "WHHe_EAM1.lspt.embd")):
        p = line.split()
        if p and p[0].isdigit():
            rows.append(p)
    assert len(rows) == 10000
    vals = np.array([[float(x) for x in r[2:]] for r in rows])
    assert np.all(vals[:, 2:] == 0.0)
    keep = sorted(set(list(range(1, 200)) + list(range(200, 10001, 50)) + [9999, 10000]))
    with open(os.path.join(HERE, "whhe_lspt_embd_rows.txt"), "w") as fh:
        fh.write("# WHHe_EAM1.lspt embedding export of the reference (NEMBD = 10000, 9 tables; "
                 "columns of tables 2-9 are zero in all rows)\n")
        fh.write("# E index rho F1_eV dF1drho_times_1.60219e-12\n")
        for i in keep:
            r = rows[i - 1]
            fh.write("E %d %s %s %s\n" % (i, r[1], r[2], r[3]))
    print("wrote", len(arrays) // 2, "data files,", len(keep), "embedding rows")


if __name__ == "__main__":
    main()
