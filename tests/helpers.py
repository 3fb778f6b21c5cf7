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


# The reference's GMD run of examples/NEB_Test (tests/golden/make_golden_neb.py): RU = 1.9
# lattice units, neighbour cutoff NB_RM = 1.2 RU (MD_SimBoxArray_ToolShell_14_CPU.F90:669-674),
# tables of 10,000 points, Bonny EAM1 with the box file's tables W: 1 2, H: 4 5.  The version
# that wrote the records gridded the tables up to the largest neighbour cutoff, RMAX = max
# NB_RM (the form left commented at MD_TypeDef_ForceTable.F90:591, where the current source
# takes max RU): with it the records are reproduced to their printed digits.
NEB_RU_LU = 1.9
NEB_NB_FACTOR = 1.2
NEB_PTYPE = np.array([[1, 2], [4, 5]], np.int32)
# absolute floor of the force check (eV/LU): FP64 summation-order noise on components whose
# ninth printed digit lies below it
NEB_F_FLOOR_LU = 1e-11


def half_printed_unit(v):
    """Half a unit in the last printed digit of values written as E15.8 (9 significant
    digits), with a 0.1 % allowance for the decimal-binary conversion."""
    a = np.abs(np.asarray(v, float))
    e = np.floor(np.log10(np.where(a > 0.0, a, 1.0)))
    return 0.5005 * 10.0 ** (e - 8)


def neb_reference_configs():
    """The two step-0 configurations in A and eV: types, positions, box low corner and edges,
    the reference's forces (eV/A) and per-atom energies (eV, the file prints -EPOT), RU, the
    table range RMAX, rc_nl, and per value the tolerance of its printed digits (force
    components in eV/A with the absolute floor, energies in eV)."""
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "neb_w2000h1_bonny_eam1.npz"))
    out = []
    for k in range(2):
        latt = float(d["c%d_latt" % k])
        ru = NEB_RU_LU * latt
        f_lu, pot = d["c%d_force" % k], d["c%d_pot" % k]
        out.append(dict(typ=d["c%d_typ" % k], pos=d["c%d_pos" % k] * latt, lo=d["c%d_boxlow" % k] * latt,
                        length=d["c%d_boxsize" % k] * latt, force=f_lu / latt, epot=-pot, ru=ru,
                        rmax=NEB_NB_FACTOR * ru, rc_nl=NEB_NB_FACTOR * ru,
                        force_tol=np.maximum(half_printed_unit(f_lu), NEB_F_FLOOR_LU) / latt,
                        epot_tol=half_printed_unit(pot)))
    return out


def neb_far_from_h(c, dist=8.0):
    """Atoms farther than dist A (minimum image) from the H atom."""
    h = c["pos"][c["typ"] == 2][0]
    dx = c["pos"] - h
    dx -= np.round(dx / c["length"]) * c["length"]
    return np.linalg.norm(dx, axis=1) > dist
