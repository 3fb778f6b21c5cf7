"""Setfl fixtures for the tests: the committed Cu1 arrays as read_setfl-style dicts, and a
writer of setfl files (LAMMPS layout) so the library's own file reader is exercised."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cu1():
    z = np.load(os.path.join(GOLDEN, "cu1_setfl_data.npz"))
    nrho, drho, nr, dr, cutoff = z["grid"]
    return dict(elements=["Cu"], nrho=int(nrho), drho=float(drho), nr=int(nr), dr=float(dr),
                cutoff=float(cutoff), mass=[float(z["atom"][1])], alat=float(z["atom"][2]),
                frho=[z["frho"]], rhor=[z["rhor"]], rphi={(0, 0): z["rphi"]})


def two_elements():
    """Cu1 plus a second element derived from it (F x1.1, rho x0.9, phi x1.2; cross pair the
    mean), for the multi-element tables."""
    d = cu1()
    f, rho, rp = d["frho"][0], d["rhor"][0], d["rphi"][(0, 0)]
    d["elements"] = ["Cu", "Xx"]
    d["mass"] = [d["mass"][0], 1.5 * d["mass"][0]]
    d["frho"] = [f, 1.1 * f]
    d["rhor"] = [rho, 0.9 * rho]
    d["rphi"] = {(0, 0): rp, (1, 1): 1.2 * rp, (1, 0): 1.1 * rp}
    return d


def write_setfl(d, path):
    ne = len(d["elements"])
    with open(path, "w") as fh:
        fh.write("test setfl\n\n\n")
        fh.write("%d %s\n" % (ne, " ".join(d["elements"])))
        fh.write("%d %.17g %d %.17g %.17g\n" % (d["nrho"], d["drho"], d["nr"], d["dr"], d["cutoff"]))

        def block(v):
            for k in range(0, len(v), 5):
                fh.write(" ".join("%.17g" % x for x in v[k:k + 5]) + "\n")

        for e in range(ne):
            fh.write("29 %.17g %.17g fcc\n" % (d["mass"][e], d.get("alat", 3.6)))
            block(d["frho"][e])
            block(d["rhor"][e])
        for i in range(ne):
            for j in range(i + 1):
                block(d["rphi"][(i, j)])
