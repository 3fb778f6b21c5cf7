"""The reference's force-library factory, by library name.

Mirrors Register_ForceLib (MDLIB/sor/Appshell/MD_ForceLib_Register.F90:63-360) and
Create_Interaction_ForceTable (MDLIB/sor/Common/MD_TypeDef_ForceTable.F90:1151-1230):
- A library registers its pair tables in a fixed order.  Most register them by
  (source, target) element symbols; EM_TB_WangJun_W-HE_2010 registers them by number.
- The table used for a host of group I and a neighbour of group J is
  PTYPE(I, J) = the table registered as (symbol of J, symbol of I) (:1168-1178),
  unless the caller gives PTYPE itself.
- Only the tables PTYPE names are built.  They are numbered by first appearance (I outer,
  J inner), which gives KPAIR.  For EAM, the embedding of group I is that of table
  PTYPE(I, I), numbered the same way, which gives KEMBD (:1191-1219).
- The sqrt(r) grid runs to Rmax = the cutoff RU (:591).

The tables themselves come from the library's generators (msmgb_create_forcetable,
msmgb_bonny_wheh_tables).
"""
from types import SimpleNamespace

import numpy as np

from . import _lib as L
from .engine import ForceTable, _cr_element_prm

FS, EAM = L.FS_TYPE, L.EAM_TYPE


def _single(pot, prm=None):
    return ("single", pot, prm)


# name -> (default pottype, registered tables in order: (source, target) or None, generator)
LIBRARIES = {
    "EM_TB_CLERI_ROSATO_PRB48_22": (FS, [(("AL", "AL"), _single(L.POT_CR, "Al")),
                                         (("AU", "AU"), _single(L.POT_CR, "Au")),
                                         (("TI", "TI"), _single(L.POT_CR, "Ti"))]),
    "EM_TB_ACKLAND_VITEK_PRB41_10324": (FS, [(("CU", "CU"), _single(L.POT_AV_CU)),
                                             (("AU", "AU"), _single(L.POT_AV_AU)),
                                             (("AU", "CU"), _single(L.POT_AV_CUAU)),
                                             (("CU", "AU"), _single(L.POT_AV_CUAU))]),
    "EM_TB_WANGJUN_TI-HE_2007": (FS, [(("TI", "TI"), _single(L.POT_CR, "Ti")),
                                      (("HE", "HE"), _single(L.POT_HEHE_EXP6)),
                                      (("TI", "HE"), _single(L.POT_HETI_LJ)),
                                      (("HE", "TI"), _single(L.POT_HETI_LJ))]),
    "EM_TB_AWB_PHIL_MAG_A71_1995_553": (FS, [(("ZR", "ZR"), _single(L.POT_AWB_ZR))]),
    "EM_TB_WANGJUN_W-HE_2010": (FS, [(None, _single(L.POT_ACKLAND_WW)),
                                     (None, _single(L.POT_HEHE_EXP6)),
                                     (None, _single(L.POT_HEW_ZBL)),
                                     (None, _single(L.POT_HEW_ZBL)),
                                     (None, _single(L.POT_DERLET_WW))]),
    "EAM_WW_MARINICA_JPCM25_2013": (EAM, [(("W", "W"), ("marinica",))]),
    "EAM_ZR_MENDELEV_PHIL_MAG_L87_2007": (EAM, [(("ZR", "ZR"), _single(L.POT_MENDELEV_ZR))]),
    "EAM_WHEH_BONNY_JPCM26_2014": (EAM, [((s, t), ("bonny", k)) for k, (s, t) in enumerate(
        [("W", "W"), ("H", "W"), ("HE", "W"), ("W", "H"), ("H", "H"), ("HE", "H"), ("W", "HE"), ("H", "HE"),
         ("HE", "HE")])]),
}


def _symbol(s):
    """Leading letters of a group symbol, upper case (Extract_SubSymb, EXSUBSTR.F)."""
    out = ""
    for ch in s.strip():
        if not ch.isalpha():
            break
        out += ch
    return out.upper()


def ptype_from_symbols(libname, symbols):
    """PTYPE(I, J) (1-based table numbers, host I) from the group symbols; raises when a pair
    has no registered table (the reference stops there)."""
    _, reg = LIBRARIES[libname.upper()]
    ids = {}
    for k, (st, _g) in enumerate(reg):
        if st is not None:
            ids.setdefault(st, k + 1)
    sym = [_symbol(s) for s in symbols]
    ng = len(sym)
    pt = np.zeros((ng, ng), np.int32)
    for i in range(ng):
        for j in range(ng):
            key = (sym[j], sym[i])
            if key not in ids:
                raise ValueError("no force table registered in %s for a %s neighbour of a %s host"
                                 % (libname, sym[j], sym[i]))
            pt[i, j] = ids[key]
    return pt


def nist(path, ru, ntab=10000, nembd=10000, export_dir=None):
    """A NIST potential file (.setfl or .lspt) the way the reference runs one
    (Register_Internal_ForceLib, MDLIB/sor/Appshell/MD_ForceLib_Register.F90:405-420):
    - if path.pair and path.embd exist, they are imported as they are;
    - otherwise the file's tables are generated on its own r and rho ranges
      (NIST_ForceTable.F90:140-175, 379-413: every element pair, groups in the file's element
      order, table id (I-1)*NE + J for an I host with a J neighbour), exported in the
      reference's format (to export_dir, default a temporary directory; the reference writes
      them next to the file) and imported;
    - the import re-grids them onto the sqrt(r) grid up to the cutoff ru (ntab points) and
      the embedding functions onto nembd points (Register_Imported_ForceTable), so the
      tables carry the export's 10-digit rounding exactly as the reference's do."""
    import os
    import tempfile
    ext = path.rsplit(".", 1)[-1].upper()
    masses = None
    stem = path
    if not (os.path.exists(path + ".pair") and os.path.exists(path + ".embd")):
        if ext == "SETFL":
            gen = ForceTable.setfl(path, ntab=ntab)
            masses = gen.masses
        else:
            gen = ForceTable.lspt(path, ntab=ntab, nembd=nembd)
        ne = gen.ngroup
        out_dir = export_dir or tempfile.mkdtemp(prefix="msmgb_nist_")
        stem = os.path.join(out_dir, os.path.basename(path))
        gen.export(stem, ids=np.arange(1, ne * ne + 1), emb_ids=[i * ne + i + 1 for i in range(ne)])
    import ctypes as C
    nt = C.c_int()
    rc = L.load().msmgb_import_info(os.fsencode(stem), None, C.byref(nt), None, None, None, None, None)
    if rc != L.OK:
        raise ValueError("cannot read the tables %s.pair / .embd" % stem)
    ne = int(round(np.sqrt(nt.value)))
    ptype = np.array([[i * ne + j + 1 for j in range(ne)] for i in range(ne)], np.int32)
    out = ForceTable.imported(stem, ptype, ru, ntab=ntab, nembd=nembd)
    out.masses = masses
    out.library = path
    return out


def create(libname, ru, symbols=None, ptype=None, subtype=None, pottype=None, ntab=10000, nembd=10000,
           rhoscal=20.0, rmax=None):
    """ForceTable of library `libname` for groups given by `symbols` (element symbols) or by
    `ptype` (NGROUP x NGROUP table numbers, host first), on the sqrt(r) grid up to `rmax`
    (default the cutoff `ru`: the reference's Rmax = max RU, MD_TypeDef_ForceTable.F90:591;
    versions of the reference took the largest neighbour cutoff, max NB_RM, instead).  `subtype` selects EAM2/EAM3/EAM4 (Marinica) or EAM1/EAM2 (Bonny); `pottype`
    "EAM_TYPE" gives EM_TB_WangJun_W-HE_2010 its EAM variant (every table embedded with
    F = -sqrt(rho), FS_EMEDMENTFUN, MD_TypeDef_ForceTable.F90:1859-1882)."""
    key = libname.upper()
    ext = key.rsplit(".", 1)[-1] if "." in key else ""
    if ext == "MOLDY":
        return ForceTable.moldy(libname, rmax=ru, ntab=ntab, nembd=nembd, rhoscal=rhoscal)
    if ext in ("SETFL", "LSPT"):
        return nist(libname, ru, ntab=ntab, nembd=nembd)
    if key not in LIBRARIES:
        raise ValueError("unknown force library %s" % libname)
    deftype, reg = LIBRARIES[key]
    ptyp = deftype
    if pottype is not None:
        ptyp = EAM if str(pottype).upper() in ("EAM", "EAM_TYPE", str(EAM)) else FS
    if ptyp != deftype and key != "EM_TB_WANGJUN_W-HE_2010":
        raise ValueError("%s has no %s variant" % (libname, pottype))
    if ptype is None:
        if symbols is None:
            raise ValueError("give the group symbols or PTYPE")
        ptype = ptype_from_symbols(key, symbols)
    ptype = np.asarray(ptype, np.int32)
    ng = ptype.shape[0]
    if ptype.min() < 1 or ptype.max() > len(reg):
        raise ValueError("PTYPE names a table %s does not register" % libname)
    order = []
    for i in range(ng):
        for j in range(ng):
            if ptype[i, j] not in order:
                order.append(int(ptype[i, j]))
    kpair = np.array([[order.index(int(ptype[i, j])) + 1 for j in range(ng)] for i in range(ng)], np.int32)
    emb_ids = []
    for i in range(ng):
        if ptype[i, i] not in emb_ids:
            emb_ids.append(int(ptype[i, i]))
    kembd = np.array([emb_ids.index(int(ptype[i, i])) + 1 for i in range(ng)], np.int32)

    rm = float(ru if rmax is None else rmax)
    cols, emb = [], {}
    bonny = None
    for tid in order:
        gen = reg[tid - 1][1]
        if gen[0] == "single":
            prm = _cr_element_prm(gen[2]) if isinstance(gen[2], str) else gen[2]
            t = ForceTable(gen[1], prm, rm, ru, deftype, ntab=ntab, nembd=nembd, rhoscal=rhoscal)
            cols.append(t)
            if t.pottype == EAM:
                emb[tid] = (t.fembd, t.dfembd, t.rhod)
        elif gen[0] == "marinica":
            t = ForceTable.marinica_eam2(rc=ru, ntab=ntab, nembd=nembd, rhoscal=rhoscal, subtype=subtype or "EAM2",
                                         rmax=rm)
            cols.append(t)
            emb[tid] = (t.fembd, t.dfembd, t.rhod)
        else:
            if bonny is None:
                bonny = ForceTable.bonny_wheh(subtype or "EAM1", rmax=rm, ntab=ntab, nembd=nembd, rhoscal=rhoscal,
                                              ru=ru)
            k = gen[1]
            cols.append(SimpleNamespace(**{name: getattr(bonny, name).reshape(ntab, bonny.nkind)[:, k].copy()
                                           for name in ("potr", "fpotr", "potb", "fpotb")}))
            g = {0: 0, 4: 1, 8: 2}.get(k)
            if g is not None:
                emb[tid] = (bonny.fembd.reshape(nembd, 3)[:, g].copy(), bonny.dfembd.reshape(nembd, 3)[:, g].copy(),
                            bonny.rhod)

    out = ForceTable.__new__(ForceTable)
    out.pot, out.prm = None, np.zeros(5)
    out.pottype = ptyp
    out.rmax, out.ru = rm, float(ru)
    out.ntab, out.nembd = int(ntab), int(nembd)
    nk = len(order)
    out.nkind, out.ngroup, out.nkind1 = nk, ng, len(emb_ids)
    for name in ("potr", "fpotr", "potb", "fpotb"):
        setattr(out, name, np.stack([getattr(c, name) for c in cols], 1).reshape(-1).copy())
    out._kpair = np.ascontiguousarray(kpair.T).reshape(-1)
    out._kembd = kembd
    out.masses = None
    out.library, out.ptype = key, ptype
    if ptyp == EAM:
        if key == "EM_TB_WANGJUN_W-HE_2010":
            rhomx = rhoscal * max(0.0, out.potb.max())
            rhod = rhomx / nembd if rhomx > 1e-64 * nembd else 1.0
            rho = np.arange(nembd) * rhod
            f = np.where(rho > 0.0, -np.sqrt(np.maximum(rho, 0.0)), 0.0)
            df = np.where(rho > 0.0, -0.5 / np.sqrt(np.where(rho > 0.0, rho, 1.0)), 0.0)
            fe = np.stack([f] * len(emb_ids), 1)
            dfe = np.stack([df] * len(emb_ids), 1)
        else:
            rhods = {v[2] for v in emb.values()}
            rhod = max(rhods) if rhods else 1.0
            z = np.zeros(nembd)
            fe = np.stack([emb[t][0] if t in emb else z for t in emb_ids], 1)
            dfe = np.stack([emb[t][1] if t in emb else z for t in emb_ids], 1)
        out.rhod = float(rhod)
        out.fembd = np.ascontiguousarray(fe).reshape(-1)
        out.dfembd = np.ascontiguousarray(dfe).reshape(-1)
    else:
        out.rhod = 1.0
        out.fembd = out.dfembd = None
    return out
