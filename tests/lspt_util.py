"""lspt fixtures for the tests: writes the W-H-He potential of the committed arrays as an lspt
control file with its ".spt" data files (the layout Filedatas_Func_Lspt.F90:118-301 reads),
so the library's own reader is exercised."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def whhe_data():
    z = np.load(os.path.join(GOLDEN, "whhe_lspt_data.npz"))
    slots = dict(zip([str(k) for k in z["slot_keys"]], [str(v) for v in z["slot_files"]]))
    files = {}
    for key in z.files:
        if key.startswith("y:"):
            name = key[2:]
            n, xl = z["g:" + name]
            files[name] = (np.arange(int(n)) * (xl / (int(n) - 1)), z[key])
    return [str(e) for e in z["elements"]], slots, files


def write_spt(path, x, y):
    with open(path, "w") as fh:
        fh.write("# x f(x)\n")
        for a, b in zip(x, y):
            fh.write("%.17g %.17g\n" % (a, b))


def write_lspt(folder, elements, slots, files, name="pot.lspt"):
    """Control file + data files into `folder`; returns the control file's path."""
    os.makedirs(folder, exist_ok=True)
    for fname, (x, y) in files.items():
        write_spt(os.path.join(folder, fname), x, y)
    ne = len(elements)
    q = lambda s: '"%s"' % s
    with open(os.path.join(folder, name), "w") as fh:
        fh.write("! test potential\n!\n&LSPT ----\n")
        fh.write("   NGROUP  number of groups = %d  (elements)\n" % ne)
        fh.write("   ATOMSYMBOL " + ", ".join("group#%d = %s" % (e + 1, q(s)) for e, s in enumerate(elements)) + "\n")
        for e in range(ne):
            fh.write("      F_RHO #%d filename = %s\n" % (e + 1, q(slots["frho_%d" % e])))
            fh.write("      RHO_R #%d filename = %s\n" % (e + 1, q(slots["rhor_%d" % e])))
        for i in range(ne):
            fh.write("   VR  line %d  filenames = %s\n" % (i + 1, ", ".join(q(slots["vr_%d_%d" % (i, j)])
                                                                         for j in range(i + 1))))
    return os.path.join(folder, name)


def whhe(folder):
    el, slots, files = whhe_data()
    return write_lspt(folder, el, slots, files)
