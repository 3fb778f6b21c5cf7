"""Host-side mirror of msmpscu's GPU force class, neighbour list and integrator.

``ForceTable`` mirrors Register_Interaction_Table + Create_Interaction_ForceTable
(MD_TypeDef_ForceTable.F90:1151-1230) for the potentials of the benchmark configurations;
``Engine`` mirrors the MDForceClassGPU procedure pointers (MD_ForceClass_Register_GPU.F90:
248-259), Cal_NeighBoreList_DEV and Predictor_DEV / Correction_DEV.  Every call goes through
the C ABI of libmsmgb.so; there is no CPU path.

Units: Angstrom, eV, fs, masses in eV*fs^2/A^2 (``lattice.AMU`` per amu).
"""
import ctypes as C
import os

import numpy as np

from . import _lib as L


class MSMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("msmgb error %d: %s" % (code, msg))
        self.code = code


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def _tptr(t):
    """double* of a contiguous float64 torch tensor (host or device memory)."""
    if str(t.dtype) != "torch.float64" or not t.is_contiguous():
        raise ValueError("expected a contiguous float64 tensor")
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))


def _torch_ready(t):
    """Orders the library's work after pending torch work on a CUDA tensor: the library runs
    on its own stream and synchronises it before returning."""
    if getattr(t, "is_cuda", False):
        import torch
        torch.cuda.current_stream(t.device).synchronize()


def _cr_element_prm(element):
    """A, xi, p, q, r0 of the reference's Cleri-Rosato library (TB_CR_AlAl/AuAu/TiTi.F90) as it
    holds them: Al's lattice constant 4.050 and all Ti constants are single-precision literals,
    and Ti's r0 = 2.951 A * sqrt(1/3 + beta^2/4) is evaluated in single precision."""
    f32 = np.float32
    halfrsq2 = 0.707106781187                                  # CP_HALFRSQ2
    if element == "Al":
        return [0.1221, 1.316, 8.612, 2.516, float(f32(4.050)) * halfrsq2]
    if element == "Au":
        return [0.2061, 1.790, 10.229, 4.036, 4.079 * halfrsq2]
    if element == "Ti":
        beta = f32(1.5874)
        fac = np.sqrt(f32(1.0) / f32(3.0) + beta * beta / f32(4.0), dtype=np.float32)
        return [float(f32(0.1519)), float(f32(1.8112)), float(f32(8.620)), float(f32(2.390)), 2.951 * float(fac)]
    raise ValueError("the Cleri-Rosato library holds Al, Au and Ti")


class ForceTable:
    """Single-species force table in the reference's conventions (NKIND = NGROUP = 1)."""

    def __init__(self, pot, prm, rmax, ru, pottype, ntab=10000, nembd=10000, rhoscal=20.0):
        lib = L.load()
        self.pot, self.pottype = pot, pottype
        self.prm = np.ascontiguousarray(prm if prm is not None else np.zeros(5), dtype=np.float64)
        self.rmax, self.ru, self.ntab, self.nembd = float(rmax), float(ru), int(ntab), int(nembd)
        self.potr, self.fpotr, self.potb, self.fpotb = (np.zeros(self.ntab) for _ in range(4))
        eam = pottype == L.EAM_TYPE
        self.fembd = np.zeros(self.nembd) if eam else None
        self.dfembd = np.zeros(self.nembd) if eam else None
        rhod = C.c_double()
        rc = lib.msmgb_create_forcetable(pot, _d(self.prm), self.rmax, self.ntab, self.nembd,
                                         float(rhoscal), _d(self.potr), _d(self.fpotr),
                                         _d(self.potb), _d(self.fpotb), _d(self.fembd),
                                         _d(self.dfembd), C.byref(rhod))
        if rc != L.OK:
            raise MSMError(rc, "table generation failed")
        self.rhod = rhod.value
        self._kpair = np.array([1], np.int32)
        self._kembd = np.array([1], np.int32)
        self.nkind = self.nkind1 = self.ngroup = 1
        self.masses = None

    @classmethod
    def setfl(cls, path, ntab=10000):
        """Tabulated EAM potential from a setfl file (Register_ForceTableProc_Setfl): NE^2
        pair tables on the sqrt(r) grid up to the file's cutoff, NE embedding tables on the
        file's rho grid; masses (amu) from the file."""
        lib = L.load()
        ne, nrho, nr, cut = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        bpath = os.fsencode(path)
        rc = lib.msmgb_setfl_info(bpath, C.byref(ne), C.byref(nrho), C.byref(nr), C.byref(cut))
        if rc != L.OK:
            raise MSMError(rc, "cannot read setfl file %s" % path)
        self = cls.__new__(cls)
        ne, nrho = ne.value, nrho.value
        self.pot, self.pottype, self.prm = None, L.EAM_TYPE, np.zeros(5)
        self.rmax = self.ru = cut.value
        self.ntab, self.nembd = int(ntab), nrho
        self.nkind, self.nkind1, self.ngroup = ne * ne, ne, ne
        self.potr, self.fpotr, self.potb, self.fpotb = (np.zeros(self.ntab * self.nkind) for _ in range(4))
        self.fembd, self.dfembd = np.zeros(nrho * ne), np.zeros(nrho * ne)
        self._kpair = np.zeros(ne * ne, np.int32)
        self._kembd = np.zeros(ne, np.int32)
        self.masses = np.zeros(ne)
        rhod = C.c_double()
        rc = lib.msmgb_setfl_tables(bpath, self.ntab, _d(self.potr), _d(self.fpotr), _d(self.potb),
                                    _d(self.fpotb), _d(self.fembd), _d(self.dfembd), _i(self._kpair),
                                    _i(self._kembd), C.byref(rhod), _d(self.masses))
        if rc != L.OK:
            raise MSMError(rc, "setfl table generation failed")
        self.rhod = rhod.value
        return self

    @classmethod
    def lspt(cls, path, ntab=10000, nembd=10000, rmax=None, each_vr_file=False):
        """Tabulated EAM potential from an lspt control file and the ".spt" files it names
        (Register_ForceTableProc_SPT): NE^2 pair tables on the sqrt(r) grid up to the largest
        pair-file r (or rmax), NE embedding tables of nembd points up to the largest F(rho)
        knot.  each_vr_file=False reads, like the reference, the first file named on each pair
        line for all pairs of that line.  The files carry no masses: set them with
        Engine.set_masses."""
        lib = L.load()
        flags = L.LSPT_EACH_VR_FILE if each_vr_file else 0
        bpath = os.fsencode(path)
        ne, rfile, rhofile = C.c_int(), C.c_double(), C.c_double()
        rc = lib.msmgb_lspt_info(bpath, flags, C.byref(ne), C.byref(rfile), C.byref(rhofile))
        if rc != L.OK:
            raise MSMError(rc, "cannot read lspt potential %s" % path)
        self = cls.__new__(cls)
        ne = ne.value
        self.pot, self.pottype, self.prm = None, L.EAM_TYPE, np.zeros(5)
        self.rmax = self.ru = float(rmax) if rmax else rfile.value
        self.ntab, self.nembd = int(ntab), int(nembd)
        self.nkind, self.nkind1, self.ngroup = ne * ne, ne, ne
        self.potr, self.fpotr, self.potb, self.fpotb = (np.zeros(self.ntab * self.nkind) for _ in range(4))
        self.fembd, self.dfembd = np.zeros(self.nembd * ne), np.zeros(self.nembd * ne)
        self._kpair = np.zeros(ne * ne, np.int32)
        self._kembd = np.zeros(ne, np.int32)
        self.masses = None
        rhod = C.c_double()
        rc = lib.msmgb_lspt_tables(bpath, flags, self.ntab, self.nembd, self.rmax, _d(self.potr), _d(self.fpotr), _d(self.potb), _d(self.fpotb),
                                   _d(self.fembd), _d(self.dfembd), _i(self._kpair), _i(self._kembd),
                                   C.byref(rhod))
        if rc != L.OK:
            raise MSMError(rc, "lspt table generation failed")
        self.rhod = rhod.value
        return self

    @classmethod
    def imported(cls, stem, ptype, rmax, ntab=10000, nembd=10000, units=L.UNITS_EV_A):
        """Tables read back from a pair of files stem.pair / stem.embd that the reference (or
        export()) wrote (Register_Imported_ForceTable): the file tables PTYPE names (NGROUP x
        NGROUP, host first, ids as in the files), re-gridded by the reference's spline onto the
        sqrt(r) grid of ntab points up to rmax and, for EAM, onto nembd embedding points."""
        lib = L.load()
        ptype = np.asarray(ptype, np.int32)
        ng = ptype.shape[0]
        self = cls.__new__(cls)
        self.pot, self.prm = None, np.zeros(5)
        self.rmax = self.ru = float(rmax)
        self.ntab, self.nembd = int(ntab), int(nembd)
        self.potr, self.fpotr, self.potb, self.fpotb = (np.zeros(self.ntab * ng * ng) for _ in range(4))
        fe, dfe = np.zeros(self.nembd * ng), np.zeros(self.nembd * ng)
        self._kpair = np.zeros(ng * ng, np.int32)
        self._kembd = np.ones(ng, np.int32)
        nk, nk1, rhod, pt = C.c_int(), C.c_int(), C.c_double(), C.c_int()
        pcol = np.ascontiguousarray(ptype.T).reshape(-1)
        rc = lib.msmgb_import_forcetable(os.fsencode(stem), int(units), ng, _i(pcol), self.rmax, self.ntab,
                                         self.nembd, _d(self.potr), _d(self.fpotr), _d(self.potb),
                                         _d(self.fpotb), _d(fe), _d(dfe), _i(self._kpair), _i(self._kembd),
                                         C.byref(nk), C.byref(nk1), C.byref(rhod), C.byref(pt))
        if rc != L.OK:
            raise MSMError(rc, "cannot import force tables %s.pair / .embd" % stem)
        self.pottype = pt.value
        self.nkind, self.nkind1, self.ngroup = nk.value, max(nk1.value, 1), ng
        n = self.nkind * self.ntab
        self.potr, self.fpotr, self.potb, self.fpotb = (a[:n].copy() for a in
                                                        (self.potr, self.fpotr, self.potb, self.fpotb))
        if self.pottype == L.EAM_TYPE:
            self.fembd, self.dfembd = fe[:nk1.value * self.nembd].copy(), dfe[:nk1.value * self.nembd].copy()
        else:
            self.fembd = self.dfembd = None
        self.rhod = rhod.value
        self.masses = None
        self.ptype = ptype
        return self

    def export(self, stem, ids=None, emb_ids=None, units=L.UNITS_EV_A):
        """Writes stem.pair / stem.embd in the reference's layout (Export_ForceTable); ids and
        emb_ids name the tables (default 1, 2, ...)."""
        lib = L.load()
        t = self.struct()
        ia = None if ids is None else np.asarray(ids, np.int32)
        ea = None if emb_ids is None else np.asarray(emb_ids, np.int32)
        rc = lib.msmgb_export_forcetable(os.fsencode(stem), int(units), C.byref(t),
                                         _i(ia) if ia is not None else None,
                                         _i(ea) if ea is not None else None)
        if rc != L.OK:
            raise MSMError(rc, "cannot export force tables to %s" % stem)

    @classmethod
    def moldy(cls, path, rmax, ntab=10000, nembd=10000, rhoscal=20.0):
        """One-element EAM potential (F = -sqrt(rho)) from a Moldy file
        (Register_ForceTableProc_Moldy), on the sqrt(r) grid up to the cutoff rmax."""
        lib = L.load()
        self = cls.__new__(cls)
        self.pot, self.pottype, self.prm = None, L.EAM_TYPE, np.zeros(5)
        self.rmax = self.ru = float(rmax)
        self.ntab, self.nembd = int(ntab), int(nembd)
        self.potr, self.fpotr, self.potb, self.fpotb = (np.zeros(self.ntab) for _ in range(4))
        self.fembd, self.dfembd = np.zeros(self.nembd), np.zeros(self.nembd)
        rhod = C.c_double()
        rc = lib.msmgb_moldy_tables(os.fsencode(path), self.rmax, self.ntab, self.nembd, float(rhoscal),
                                    _d(self.potr), _d(self.fpotr), _d(self.potb), _d(self.fpotb),
                                    _d(self.fembd), _d(self.dfembd), C.byref(rhod))
        if rc != L.OK:
            raise MSMError(rc, "cannot read Moldy potential %s" % path)
        self.rhod = rhod.value
        self._kpair = np.array([1], np.int32)
        self._kembd = np.array([1], np.int32)
        self.nkind = self.nkind1 = self.ngroup = 1
        self.masses = None
        return self

    @classmethod
    def cleri_rosato(cls, A, xi, p, q, r0, rc, ntab=10000):
        """Cleri-Rosato TB-SMA (FS type) with a hard cutoff rc (Rmax = RU = rc)."""
        return cls(L.POT_CR, [A, xi, p, q, r0], rc, rc, L.FS_TYPE, ntab=ntab, nembd=ntab)

    @classmethod
    def awb_zr(cls, rmax=5.6, ru=None, ntab=10000):
        """Ackland-Wooding-Bacon Zr (FS type), the reference's EM_TB_AWB_Phil_Mag_A71_1995_553."""
        return cls(L.POT_AWB_ZR, None, rmax, ru if ru else rmax, L.FS_TYPE, ntab=ntab)

    @classmethod
    def wangjun_ti_he(cls, rmax, ru=None, ntab=10000):
        """The reference's Ti-He FS library EM_TB_WangJun_Ti-HE_2007
        (EM_TB_ForcetTable_WangJun_Ti_He_2007.F90): #1 Ti-Ti (Cleri-Rosato Ti), #2 He-He
        (ZBL/EXP6, the W-He library's), #3 (Ti neighbour of a He host) and #4 (He neighbour of a
        Ti host), both He-Ti.  Groups Ti = 1, He = 2: KPAIR(1,1) = 1, KPAIR(2,2) = 2,
        KPAIR(2,1) = 3, KPAIR(1,2) = 4."""
        ru = ru if ru else rmax
        parts = [cls(L.POT_CR, _cr_element_prm("Ti"), rmax, ru, L.FS_TYPE, ntab=ntab, nembd=ntab),
                 cls(L.POT_HEHE_EXP6, None, rmax, ru, L.FS_TYPE, ntab=ntab),
                 cls(L.POT_HETI_LJ, None, rmax, ru, L.FS_TYPE, ntab=ntab),
                 cls(L.POT_HETI_LJ, None, rmax, ru, L.FS_TYPE, ntab=ntab)]
        self = parts[0]
        for key in ("potr", "fpotr", "potb", "fpotb"):
            setattr(self, key, np.stack([getattr(t, key) for t in parts], 1).reshape(-1).copy())
        self.pot = None
        self.nkind, self.ngroup, self.nkind1 = 4, 2, 1
        kp = np.array([[1, 4], [3, 2]], np.int32)           # KPAIR(I, J) at kp[I-1, J-1]
        self._kpair = np.ascontiguousarray(kp.T).reshape(-1)
        self._kembd = np.ones(2, np.int32)
        return self

    @classmethod
    def cleri_rosato_element(cls, element, rc, ntab=10000):
        """The reference's Cleri-Rosato library EM_TB_Cleri_Rosato_PRB48_22 (Al, Au, Ti;
        EM_TB_ForcetTable_CR_2014.F90:31-36), FS type with a hard cutoff rc.  Parameters as
        the reference holds them: Al's lattice constant 4.050 (TB_CR_AlAl.F90:13) and all of
        Ti's constants (TB_CR_TiTi.F90:10-16) are single-precision literals, and Ti's
        r0 = 2.951 A * sqrt(1/3 + beta^2/4) is evaluated in single precision."""
        prm = _cr_element_prm(element)
        return cls(L.POT_CR, prm, rc, rc, L.FS_TYPE, ntab=ntab, nembd=ntab)

    @classmethod
    def marinica_eam2(cls, rc=5.4604375, ntab=10000, nembd=10000, rhoscal=20.0, subtype="EAM2", rmax=None):
        """Marinica W (EAM type), subtype EAM2 (the reference's default), EAM3 or EAM4
        (EAM_ForceTable_Marinica_JPCM25_2013.F90:31-44); tables up to rmax (default rc)."""
        pot = {"EAM2": L.POT_MARINICA2, "EAM3": L.POT_MARINICA3, "EAM4": L.POT_MARINICA4}[subtype.upper()]
        return cls(pot, None, rc if rmax is None else rmax, rc, L.EAM_TYPE, ntab=ntab, nembd=nembd,
                   rhoscal=rhoscal)

    @classmethod
    def ackland_ww(cls, rmax, ru=None, ntab=10000):
        return cls(L.POT_ACKLAND_WW, None, rmax, ru if ru else rmax, L.FS_TYPE, ntab=ntab)

    @classmethod
    def wangjun_w_he(cls, rmax=10.0, ru=None, ww="ackland", ntab=10000):
        """The reference's W-He FS library EM_TB_WangJun_W-HE_2010
        (EM_TB_ForceTable_WangJun_W_HE_2010.F90:68-121): tables #1 W-W (Ackland-Thetford),
        #2 He-He (ZBL/EXP6), #3 He-W and #4 W-He (ZBL/ab-initio/EXP6), #5 W-W (Derlet et al.).
        Groups W = 1, He = 2: KPAIR(1,1) = 1 (ww="ackland") or 5 (ww="derlet"),
        KPAIR(2,2) = 2, KPAIR(2,1) = 3, KPAIR(1,2) = 4."""
        pots = [L.POT_ACKLAND_WW, L.POT_HEHE_EXP6, L.POT_HEW_ZBL, L.POT_HEW_ZBL, L.POT_DERLET_WW]
        parts = [cls(p, None, rmax, ru if ru else rmax, L.FS_TYPE, ntab=ntab) for p in pots]
        self = parts[0]
        nk = len(pots)
        for key in ("potr", "fpotr", "potb", "fpotb"):
            setattr(self, key, np.stack([getattr(t, key) for t in parts], 1).reshape(-1).copy())
        self.pot = None
        self.nkind, self.ngroup, self.nkind1 = nk, 2, 1
        ww_id = {"ackland": 1, "derlet": 5}[ww]
        kp = np.array([[ww_id, 4], [3, 2]], np.int32)       # KPAIR(I, J) at kp[I-1, J-1]
        self._kpair = np.ascontiguousarray(kp.T).reshape(-1)
        self._kembd = np.ones(2, np.int32)
        return self

    @classmethod
    def mendelev_zr(cls, rc=7.6, ntab=10000, nembd=10000, rhoscal=20.0):
        """Mendelev-Ackland Zr (EAM type), the reference's EAM_Zr_Mendelev_Phil_Mag_L87_2007;
        its pair knots end at 7.6 A."""
        return cls(L.POT_MENDELEV_ZR, None, rc, rc, L.EAM_TYPE, ntab=ntab, nembd=nembd, rhoscal=rhoscal)

    @classmethod
    def ackland_vitek(cls, rmax, ru=None, ntab=10000):
        """The reference's Cu-Au FS library EM_TB_Ackland_Vitek_PRB41_10324
        (EM_TB_ForceTable_Ackland_Vitek_PRB41_10324.F90): tables #1 Cu-Cu, #2 Au-Au,
        #3 (Au neighbour of a Cu host) and #4 (Cu neighbour of an Au host), both the Cu-Au
        cross functions.  Groups Cu = 1, Au = 2: KPAIR(1,1) = 1, KPAIR(2,2) = 2,
        KPAIR(1,2) = 3, KPAIR(2,1) = 4."""
        pots = [L.POT_AV_CU, L.POT_AV_AU, L.POT_AV_CUAU, L.POT_AV_CUAU]
        parts = [cls(p, None, rmax, ru if ru else rmax, L.FS_TYPE, ntab=ntab) for p in pots]
        self = parts[0]
        for key in ("potr", "fpotr", "potb", "fpotb"):
            setattr(self, key, np.stack([getattr(t, key) for t in parts], 1).reshape(-1).copy())
        self.pot = None
        self.nkind, self.ngroup, self.nkind1 = 4, 2, 1
        kp = np.array([[1, 3], [4, 2]], np.int32)           # KPAIR(I, J) at kp[I-1, J-1]
        self._kpair = np.ascontiguousarray(kp.T).reshape(-1)
        self._kembd = np.ones(2, np.int32)
        return self

    @classmethod
    def bonny_wheh(cls, subtype="EAM1", rmax=5.4604375, ntab=10000, nembd=10000, rhoscal=20.0, ru=None):
        """The reference's W-H-He EAM of Bonny, Grigorev, Terentyev (EAM_WHeH_Bonny_JPCM26_2014),
        subtype "EAM1" (H, He pair-only) or "EAM2" (H embedded in the W density); groups
        W = 1, H = 2, He = 3.  Tables up to rmax, cutoff ru (default rmax)."""
        lib = L.load()
        sub = {"EAM1": 1, "EAM2": 2}[subtype.upper()]
        self = cls.__new__(cls)
        self.pot, self.pottype, self.prm = None, L.EAM_TYPE, np.zeros(5)
        self.rmax = float(rmax)
        self.ru = float(rmax if ru is None else ru)
        self.ntab, self.nembd = int(ntab), int(nembd)
        arrs = [np.zeros(10 * self.ntab) for _ in range(4)]
        self.fembd, self.dfembd = np.zeros(3 * self.nembd), np.zeros(3 * self.nembd)
        self._kpair = np.zeros(9, np.int32)
        self._kembd = np.zeros(3, np.int32)
        nk, rhod = C.c_int(), C.c_double()
        rc = lib.msmgb_bonny_wheh_tables(sub, self.rmax, self.ntab, self.nembd, float(rhoscal),
                                         *[_d(a) for a in arrs], _d(self.fembd), _d(self.dfembd),
                                         _i(self._kpair), _i(self._kembd), C.byref(nk), C.byref(rhod))
        if rc != L.OK:
            raise MSMError(rc, "Bonny W-H-He table generation failed")
        self.nkind, self.nkind1, self.ngroup = nk.value, 3, 3
        self.potr, self.fpotr, self.potb, self.fpotb = (a[:self.nkind * self.ntab].copy() for a in arrs)
        self.rhod = rhod.value
        self.masses = None
        return self

    def struct(self):
        t = L.ForceTable()
        t.pottype, t.ntab, t.nkind, t.rmax = self.pottype, self.ntab, self.nkind, self.rmax
        t.potr, t.fpotr, t.potb, t.fpotb = (_d(a) for a in (self.potr, self.fpotr, self.potb, self.fpotb))
        eam = self.pottype == L.EAM_TYPE
        t.nembd = self.nembd if eam else 0
        t.nkind1 = self.nkind1 if eam else 0
        t.rhod = self.rhod
        t.fembd, t.dfembd = (_d(self.fembd), _d(self.dfembd)) if eam else (None, None)
        t.ngroup = self.ngroup
        t.kpair = _i(self._kpair)
        t.kembd = _i(self._kembd)
        t.ru = self.ru
        return t

    @property
    def csi(self):
        return float(self.ntab) / np.sqrt(self.rmax)


class Engine:
    """One device context: tables, a batch of boxes, neighbour list, force passes, MD steps."""

    def __init__(self, max_atoms, rc_nl, max_boxes=1, mxkvois=64, skin_trigger=0.15,
                 nb_uptab=10, precision="fp64", device=0, stream=None, outer_skin=None):
        self.lib = L.load()
        p = L.Params()
        p.device, p.max_atoms, p.max_boxes, p.mxkvois = device, int(max_atoms), int(max_boxes), int(mxkvois)
        p.rc_nl, p.skin_trigger, p.nb_uptab = float(rc_nl), float(skin_trigger), int(nb_uptab)
        p.precision = L.PRECISIONS[precision]
        self.precision = precision
        p.stream = stream
        self.ctx = C.c_void_p()
        rc = self.lib.msmgb_create(C.byref(self.ctx), C.byref(p))
        if rc != L.OK:
            raise MSMError(rc, "context creation failed (device %d)" % device)
        self.params = p
        self.n = 0
        self.nbox = 0
        self._table = None
        if outer_skin is not None:
            self.set_outer_skin(outer_skin)

    # ---- plumbing --------------------------------------------------------------------------
    def _ck(self, rc):
        if rc != L.OK:
            msg = self.lib.msmgb_last_error(self.ctx)
            raise MSMError(rc, msg.decode() if msg else "")
        return rc

    def close(self):
        if self.ctx:
            self.lib.msmgb_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self.lib.msmgb_stream(self.ctx)

    @property
    def launches(self):
        return int(self.lib.msmgb_launch_count(self.ctx))

    def synchronize(self):
        self._ck(self.lib.msmgb_synchronize(self.ctx))

    def set_precision(self, precision):
        self._ck(self.lib.msmgb_set_precision(self.ctx, L.PRECISIONS[precision]))
        self.precision = precision

    # ---- force class ---------------------------------------------------------------------------
    def init_forcetable(self, table: ForceTable):
        self._table = table
        s = table.struct()
        self._ck(self.lib.msmgb_init_forcetable(self.ctx, C.byref(s)))

    def init_forcetable_raw(self, pottype, ntab, nkind, rmax, ru, potr, fpotr, potb, fpotb, ngroup,
                            kpair, nembd=0, nkind1=0, rhod=1.0, fembd=None, dfembd=None, kembd=None):
        """Tables already in the reference layout (NKIND, NTAB) column-major, i.e. numpy
        arrays of shape (NTAB, NKIND) in C order; kpair (NGROUP, NGROUP) 1-based ids with
        KPAIR(i, j) at kpair[i-1, j-1]."""
        keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (potr, fpotr, potb, fpotb)]
        kp = np.ascontiguousarray(np.asarray(kpair, np.int32).T)      # column-major (i fastest)
        t = L.ForceTable()
        t.pottype, t.ntab, t.nkind, t.rmax, t.ru = pottype, int(ntab), int(nkind), float(rmax), float(ru)
        t.potr, t.fpotr, t.potb, t.fpotb = (_d(a) for a in keep)
        t.ngroup = int(ngroup)
        t.kpair = _i(kp)
        if pottype == L.EAM_TYPE:
            ke = np.ascontiguousarray(kembd, np.int32)
            fe = np.ascontiguousarray(fembd, np.float64)
            dfe = np.ascontiguousarray(dfembd, np.float64)
            keep += [ke, fe, dfe]
            t.nembd, t.nkind1, t.rhod = int(nembd), int(nkind1), float(rhod)
            t.fembd, t.dfembd, t.kembd = _d(fe), _d(dfe), _i(ke)
        self._raw_keep = (keep, kp)
        self._ck(self.lib.msmgb_init_forcetable(self.ctx, C.byref(t)))

    def clear_forcetable(self):
        self._ck(self.lib.msmgb_clear_forcetable(self.ctx))

    def calforce(self):
        self._ck(self.lib.msmgb_calforce(self.ctx))

    def calptensor(self):
        v = np.zeros(9 * max(self.nbox, 1))
        self._ck(self.lib.msmgb_calptensor(self.ctx, _d(v)))
        return v.reshape(-1, 3, 3)

    def calepot(self):
        self._ck(self.lib.msmgb_calepot(self.ctx))

    def calden(self):
        self._ck(self.lib.msmgb_calden(self.ctx))

    def atomic_stress(self, order=L.ORDER_ORIGINAL):
        """Per-atom virial tensors sum_j FORTOT s_a s_b, shape (N, 3, 3) (pCalAVStress)."""
        ap = np.zeros(9 * self.n)
        self._ck(self.lib.msmgb_cal_atomic_stress(self.ctx, _d(ap), order))
        return ap.reshape(9, self.n).T.reshape(self.n, 3, 3).copy()

    # ---- state ---------------------------------------------------------------------------------
    def copyin(self, boxes, pos, vel=None, ityp=None, statu=None):
        """boxes: list of (natom, lo[3], len[3], ifpd[3]); pos/vel: (N,3) arrays."""
        n = int(pos.shape[0])
        arr = (L.Box * len(boxes))()
        tot = 0
        for k, (na, lo, ln, pd) in enumerate(boxes):
            arr[k].natom = int(na)
            for d in range(3):
                arr[k].lo[d], arr[k].len[d], arr[k].ifpd[d] = float(lo[d]), float(ln[d]), int(pd[d])
            tot += int(na)
        if tot != n:
            raise ValueError("box atom counts (%d) do not add up to N (%d)" % (tot, n))
        xp = np.ascontiguousarray(np.asarray(pos, np.float64).T).reshape(-1)
        xp1 = np.ascontiguousarray(np.asarray(vel, np.float64).T).reshape(-1) if vel is not None else None
        ty = np.ascontiguousarray(ityp if ityp is not None else np.ones(n), dtype=np.int32)
        st = np.ascontiguousarray(statu if statu is not None else np.full(n, L.STATU_ACTIVE), dtype=np.int32)
        self._ck(self.lib.msmgb_copyin_simbox(self.ctx, len(boxes), arr, _i(ty), _i(st), _d(xp), _d(xp1)))
        self.n, self.nbox = n, len(boxes)

    @staticmethod
    def pack_boxes(boxes):
        arr = (L.Box * len(boxes))()
        for k, (na, lo, ln, pd) in enumerate(boxes):
            arr[k].natom = int(na)
            for d in range(3):
                arr[k].lo[d], arr[k].len[d], arr[k].ifpd[d] = float(lo[d]), float(ln[d]), int(pd[d])
        return arr

    def copyin_raw(self, box_arr, nbox, ityp, statu, xp, xp1):
        """Upload from caller-prepared arrays already in the ABI layout (XP(N,3) column-major
        float64, int32 types/status), e.g. pinned host buffers; no host-side conversion."""
        self._ck(self.lib.msmgb_copyin_simbox(self.ctx, nbox, box_arr, _i(ityp), _i(statu), _d(xp), _d(xp1)))
        self.n, self.nbox = int(ityp.size), nbox

    def copyout_raw(self, xp=None, xp1=None, fp=None, order=L.ORDER_ORIGINAL):
        """Download into caller-provided XP-layout float64 arrays (any may be None)."""
        if xp is not None or xp1 is not None:
            self._ck(self.lib.msmgb_copyout_simbox(self.ctx, _d(xp), _d(xp1), None, None, order))
        if fp is not None:
            self._ck(self.lib.msmgb_copyout_force(self.ctx, _d(fp), order))

    def update_positions(self, x):
        """New positions (N,3) of the loaded atoms: a numpy array, or a float64 torch tensor in
        the XP layout (shape (3, N) contiguous: x block, then y, then z) whose memory, host or
        device, is read directly."""
        if hasattr(x, "data_ptr"):
            _torch_ready(x)
            self._ck(self.lib.msmgb_update_positions(self.ctx, C.c_void_p(x.data_ptr())))
        else:
            xp = np.ascontiguousarray(np.asarray(x, np.float64).T).reshape(-1)
            self._ck(self.lib.msmgb_update_positions(self.ctx, xp.ctypes.data_as(C.c_void_p)))

    def set_steps_per_graph(self, k):
        """MD steps captured into one CUDA graph launch (1..64)."""
        self._ck(self.lib.msmgb_set_steps_per_graph(self.ctx, int(k)))

    @property
    def graph_launches(self):
        n = C.c_int64()
        self._ck(self.lib.msmgb_graph_launch_count(self.ctx, C.byref(n)))
        return n.value

    def set_extforce_field(self, fext):
        """Constant external force per atom ((N, 3), caller order), added after every force
        pass (None removes it); MD steps then run unfused."""
        if fext is None:
            self._ck(self.lib.msmgb_set_extforce_field(self.ctx, None))
            return
        f = np.ascontiguousarray(np.asarray(fext, np.float64).T).reshape(-1)
        self._ck(self.lib.msmgb_set_extforce_field(self.ctx, f.ctypes.data_as(C.c_void_p)))

    def add_extforce(self, tag, fn):
        """Registers fn(view) -> int, called after every force pass with an ExtForceView of
        device pointers (msmgb.h); the ctypes callback is kept alive by the engine."""
        cb = L.EXTFORCE_FN(lambda user, view: int(fn(view.contents)))
        self._ext_cbs = getattr(self, "_ext_cbs", []) + [cb]
        self._ck(self.lib.msmgb_add_extforce(self.ctx, tag.encode(), cb, None))

    def clear_extforce(self):
        self._ck(self.lib.msmgb_clear_extforce(self.ctx))
        self._ext_cbs = []

    def set_masses(self, cm):
        cm = np.ascontiguousarray(np.atleast_1d(cm), dtype=np.float64)
        self._ck(self.lib.msmgb_set_masses(self.ctx, int(cm.size), _d(cm)))

    def _xp(self, fn, order):
        out = np.zeros(3 * self.n)
        self._ck(fn(self.ctx, _d(out), order))
        return out.reshape(3, self.n).T.copy()

    def get_force(self, order=L.ORDER_ORIGINAL):
        return self._xp(self.lib.msmgb_copyout_force, order)

    def force_into(self, out):
        """Forces of the last force call into a float64 torch tensor of shape (3, N) (XP
        layout, caller order), on the host or the device, with no staging through numpy."""
        _torch_ready(out)
        self._ck(self.lib.msmgb_copyout_force(self.ctx, _tptr(out), L.ORDER_ORIGINAL))
        return out

    def hvp_into(self, v, out):
        """Hessian-vector product on float64 torch tensors of shape (3, N) (XP layout), host or
        device memory."""
        _torch_ready(v)
        self._ck(self.lib.msmgb_hvp(self.ctx, _tptr(v), _tptr(out)))
        return out

    def get_epot(self, order=L.ORDER_ORIGINAL):
        out = np.zeros(self.n)
        self._ck(self.lib.msmgb_copyout_epot(self.ctx, _d(out), order))
        return out

    def get_ekin(self, order=L.ORDER_ORIGINAL):
        """Per-atom kinetic energy 0.5 m v^2 (-1e32 for inactive or position-fixed atoms)."""
        out = np.zeros(self.n)
        self._ck(self.lib.msmgb_calekin(self.ctx, _d(out), order))
        return out

    def get_den(self, order=L.ORDER_ORIGINAL):
        out = np.zeros(self.n)
        self._ck(self.lib.msmgb_copyout_den(self.ctx, _d(out), order))
        return out

    def get_state(self, order=L.ORDER_ORIGINAL):
        xp, xp1, dis = np.zeros(3 * self.n), np.zeros(3 * self.n), np.zeros(3 * self.n)
        st = np.zeros(self.n, np.int32)
        self._ck(self.lib.msmgb_copyout_simbox(self.ctx, _d(xp), _d(xp1), _i(st), _d(dis), order))
        f = lambda a: a.reshape(3, self.n).T.copy()
        return f(xp), f(xp1), st, f(dis)

    def get_gid(self):
        g = np.zeros(self.n, np.int32)
        self._ck(self.lib.msmgb_copyout_gid(self.ctx, _i(g)))
        return g

    # ---- neighbour list --------------------------------------------------------------------------
    def cal_neighborelist(self):
        self._ck(self.lib.msmgb_cal_neighborelist(self.ctx))

    def get_neighborelist(self, order=L.ORDER_ORIGINAL):
        mxk = self.params.mxkvois
        kv = np.zeros(self.n, np.int32)
        ind = np.zeros(mxk * self.n, np.int32)
        self._ck(self.lib.msmgb_copyout_neighborelist(self.ctx, _i(kv), _i(ind), self.n, order))
        return kv, ind.reshape(mxk, self.n)

    # ---- integrator ------------------------------------------------------------------------------
    def predictor(self, h):
        self._ck(self.lib.msmgb_predictor(self.ctx, float(h)))

    def correction(self, h):
        self._ck(self.lib.msmgb_correction(self.ctx, float(h)))

    def run_steps(self, nsteps, h):
        nr = C.c_int()
        self._ck(self.lib.msmgb_run_steps(self.ctx, int(nsteps), float(h), C.byref(nr)))
        return nr.value

    def enqueue_steps(self, nsteps, h):
        self._ck(self.lib.msmgb_enqueue_steps(self.ctx, int(nsteps), float(h)))

    def finish_steps(self, h):
        nr = C.c_int()
        self._ck(self.lib.msmgb_finish_steps(self.ctx, float(h), C.byref(nr)))
        return nr.value

    def time_steps(self, nsteps, h):
        ms = C.c_float()
        nr = C.c_int()
        self._ck(self.lib.msmgb_time_steps(self.ctx, int(nsteps), float(h), C.byref(ms), C.byref(nr)))
        return float(ms.value), nr.value

    def time_passes(self, reps=5):
        out = (C.c_float * 5)()
        self._ck(self.lib.msmgb_time_passes(self.ctx, int(reps), out))
        return dict(density=out[0], force=out[1], nlist=out[2], vv=out[3], fused=out[4])

    def tuning(self):
        out = (C.c_int * 3)()
        ms = (C.c_float * 3)()
        self._ck(self.lib.msmgb_get_tuning(self.ctx, out, ms))
        return {"density_variant": out[0], "force_variant": out[1], "fused_variant": out[2],
                "density_ms": ms[0], "force_ms": ms[1], "fused_ms": ms[2]}

    def set_tuning(self, density=-1, force=-1, fused=-1):
        """Pins kernel variants of the mixed passes (-1 leaves a choice to the tuner)."""
        codes = (C.c_int * 3)(density, force, fused)
        self._ck(self.lib.msmgb_set_tuning(self.ctx, codes))

    def set_boxshape(self, ibox, shape):
        """BOXSHAPE (3x3, row K maps SEP to the K-th length component) of box ibox; applies
        from the next copyin.  Non-cubic states support the FP64 static calls only."""
        bs = np.ascontiguousarray(np.asarray(shape, np.float64).reshape(9))
        self._ck(self.lib.msmgb_set_boxshape(self.ctx, int(ibox), _d(bs)))

    def set_outer_skin(self, skin):
        """Outer skin of the two-level list (0: off); applies from the next copyin."""
        self._ck(self.lib.msmgb_set_outer_skin(self.ctx, float(skin)))

    def rebuild_counts(self):
        """(rebuilds, full rebuilds) done inside MD steps since the context was created."""
        r, f = C.c_int64(), C.c_int64()
        self._ck(self.lib.msmgb_rebuild_counts(self.ctx, C.byref(r), C.byref(f)))
        return r.value, f.value

    def time_rebuilds(self, reps=3):
        """Device time (ms) of a full list rebuild and of a re-selection from the candidates."""
        full, inner = C.c_float(), C.c_float()
        self._ck(self.lib.msmgb_time_rebuilds(self.ctx, int(reps), C.byref(full), C.byref(inner)))
        return dict(full=full.value, inner=inner.value)

    def tile_stats(self):
        """Cell tiles of the mixed passes: blocks, blocks with a tile, mean and largest halo."""
        nb, nt, mx = C.c_int(), C.c_int(), C.c_int()
        mean = C.c_double()
        self._ck(self.lib.msmgb_tile_stats(self.ctx, C.byref(nb), C.byref(nt), C.byref(mean), C.byref(mx)))
        return dict(blocks=nb.value, tiled=nt.value, mean_halo=mean.value, max_halo=mx.value)

    def check_records(self):
        """Largest |hi + lo - u| of the float-float position records in units of the positions'
        quantum, and the number of atoms whose hi is off the quantum or |lo| > quantum / 2."""
        err = C.c_double()
        bad = C.c_int()
        self._ck(self.lib.msmgb_check_records(self.ctx, C.byref(err), C.byref(bad)))
        return err.value, bad.value

    def list_stats(self):
        mk = C.c_int()
        mean = C.c_double()
        self._ck(self.lib.msmgb_list_stats(self.ctx, C.byref(mk), C.byref(mean)))
        return mk.value, mean.value

    # ---- differentiation ---------------------------------------------------------------------------
    def param_adjoint(self, prm, ft, pot=L.POT_CR):
        """Force-matching loss sum|F - Ft|^2 and its gradient with respect to the potential
        parameters (Cleri-Rosato: A, xi, p, q, r0) of the loaded tables."""
        prm = np.ascontiguousarray(prm, dtype=np.float64)
        ft = np.ascontiguousarray(np.asarray(ft, np.float64).T).reshape(-1)
        loss = C.c_double()
        grad = np.zeros(5)
        self._ck(self.lib.msmgb_param_adjoint(self.ctx, pot, _d(prm), _d(ft), C.byref(loss), _d(grad)))
        return loss.value, grad

    def time_hvp(self, v, reps=10):
        """(ms per Hessian-vector product, ms per FP64 force call) on the device."""
        v = np.ascontiguousarray(np.asarray(v, np.float64).T).reshape(-1)
        a, b = C.c_float(), C.c_float()
        self._ck(self.lib.msmgb_time_hvp(self.ctx, _d(v), int(reps), C.byref(a), C.byref(b)))
        return float(a.value), float(b.value)

    def hvp(self, v):
        v = np.ascontiguousarray(np.asarray(v, np.float64).T).reshape(-1)
        out = np.zeros(3 * self.n)
        self._ck(self.lib.msmgb_hvp(self.ctx, _d(v), _d(out)))
        return out.reshape(3, self.n).T.copy()
