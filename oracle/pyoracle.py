"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py import this
module, and only as the checker.  The product (``msmpscu_gb300``) never imports it.
"""
import ctypes as C
import os
import re

import numpy as np

from . import build as _build

POT_CR, POT_MARINICA2, POT_ACKLAND_WW = 1, 2, 3
POT_DERLET_WW, POT_HEHE_EXP6, POT_HEW_ZBL = 4, 5, 6
POT_MARINICA3, POT_MARINICA4 = 7, 8
POT_AV_CU, POT_AV_AU, POT_AV_CUAU = 9, 10, 11
POT_MENDELEV_ZR = 12
POT_AWB_ZR = 13
POT_HETI_LJ = 14
FS, EAM = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class OrcTables(C.Structure):
    _fields_ = [("pottype", C.c_int), ("ntab", C.c_int), ("nkind", C.c_int),
                ("csi", C.c_double), ("ru2", C.c_double),
                ("potr", _dp), ("fpotr", _dp), ("potb", _dp), ("fpotb", _dp),
                ("nembd", C.c_int), ("nkind1", C.c_int), ("rhod", C.c_double),
                ("fembd", _dp), ("dfembd", _dp),
                ("ngroup", C.c_int), ("kpair", _ip), ("kembd", _ip)]


class OrcBox(C.Structure):
    _fields_ = [("lo", C.c_double * 3), ("len", C.c_double * 3), ("ifpd", C.c_int * 3),
                ("shaped", C.c_int), ("bs", C.c_double * 9)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        _lib.orc_make_tables.restype = C.c_int
        _lib.orc_nlist.restype = C.c_int
        _lib.orc_nlist_brute.restype = C.c_int
        _lib.orc_force.restype = C.c_int
        _lib.orc_md.restype = C.c_int
        _lib.orc_md_ext.restype = C.c_int
        _lib.orc_hvp.restype = C.c_int
        _lib.orc_adjoint_cr.restype = C.c_int
        _lib.orc_atomic_stress.restype = None
        _lib.orc_spline_eval.restype = C.c_double
        _lib.orc_setfl_tables.restype = C.c_int
        _lib.orc_spline_knots.restype = None
        _lib.orc_bonny_pair.restype = C.c_int
        _lib.orc_bonny_embed.restype = C.c_int
        _lib.orc_spline_knots_eval.restype = None
        _lib.orc_pot_eval.restype = C.c_int
        _lib.orc_embed_eval.restype = C.c_int
        _lib.orc_splid2.restype = C.c_double
        _lib.orc_import_regrid_pair.restype = None
        _lib.orc_import_regrid_embd.restype = None
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def pot_eval(pot, prm, r):
    prm = f64(prm if prm is not None else np.zeros(5))
    out = np.zeros(4)
    v = [C.c_double() for _ in range(4)]
    lib().orc_pot_eval(pot, _d(prm), C.c_double(r), *[C.byref(x) for x in v])
    out[:] = [x.value for x in v]
    return out


def make_tables(pot, prm, rmax, ntab=10000, nembd=10000, rhoscal=20.0, want_embed=True):
    prm = f64(prm if prm is not None else np.zeros(5))
    potr, fpotr, potb, fpotb = (np.zeros(ntab) for _ in range(4))
    fembd = np.zeros(nembd) if want_embed else None
    dfembd = np.zeros(nembd) if want_embed else None
    rhod = C.c_double()
    rc = lib().orc_make_tables(pot, _d(prm), C.c_double(rmax), ntab, nembd, C.c_double(rhoscal),
                               _d(potr), _d(fpotr), _d(potb), _d(fpotb),
                               _d(fembd) if want_embed else None,
                               _d(dfembd) if want_embed else None, C.byref(rhod))
    if rc != 0:
        raise ValueError("unknown potential id %d" % pot)
    return dict(potr=potr, fpotr=fpotr, potb=potb, fpotb=fpotb, fembd=fembd, dfembd=dfembd,
                rhod=rhod.value, ntab=ntab, nembd=nembd, rmax=rmax)


class Tables:
    """Single-species tables in the reference's (NKIND=1, NTAB) layout."""

    def __init__(self, tabs, pottype, ru):
        self.t = tabs
        self.keep = [f64(tabs[k]) for k in ("potr", "fpotr", "potb", "fpotb")]
        emb = [f64(tabs["fembd"]), f64(tabs["dfembd"])] if tabs.get("fembd") is not None \
            else [np.zeros(1), np.zeros(1)]
        self.keep += emb
        self.kpair = i32([1])
        self.kembd = i32([1])
        ntab = tabs["ntab"]
        s = OrcTables()
        s.pottype = pottype
        s.ntab = ntab
        s.nkind = 1
        s.csi = float(ntab) / np.sqrt(tabs["rmax"])
        s.ru2 = ru * ru
        s.potr, s.fpotr, s.potb, s.fpotb = (_d(a) for a in self.keep[:4])
        s.nembd = tabs["nembd"] if tabs.get("fembd") is not None else 1
        s.nkind1 = 1
        s.rhod = tabs["rhod"]
        s.fembd, s.dfembd = _d(self.keep[4]), _d(self.keep[5])
        s.ngroup = 1
        s.kpair = _i(self.kpair)
        s.kembd = _i(self.kembd)
        self.s = s


class RawTables:
    """Multi-kind tables in the reference layout: arrays (NTAB, NKIND) C-order = Fortran
    (NKIND, NTAB); kpair (NGROUP, NGROUP) with KPAIR(i, j) at kpair[i-1, j-1]."""

    def __init__(self, pottype, ntab, nkind, rmax, ru, potr, fpotr, potb, fpotb, kpair, fembd=None,
                 dfembd=None, kembd=None, rhod=1.0):
        """EAM: fembd/dfembd (NEMBD, NKIND1) C-order = Fortran (NKIND1, NEMBD), kembd 1-based."""
        emb = [f64(fembd), f64(dfembd)] if fembd is not None else [np.zeros(1), np.zeros(1)]
        self.keep = [f64(a) for a in (potr, fpotr, potb, fpotb)] + emb
        ng = np.asarray(kpair).shape[0]
        self.kpair = i32(np.asarray(kpair, np.int32).T)
        self.kembd = i32(kembd if kembd is not None else np.ones(ng))
        s = OrcTables()
        s.pottype, s.ntab, s.nkind = pottype, ntab, nkind
        s.csi = float(ntab) / np.sqrt(rmax)
        s.ru2 = ru * ru
        s.potr, s.fpotr, s.potb, s.fpotb = (_d(a) for a in self.keep[:4])
        if fembd is not None:
            fe = np.asarray(fembd)
            s.nembd, s.nkind1, s.rhod = fe.shape[0], (fe.shape[1] if fe.ndim == 2 else 1), float(rhod)
        else:
            s.nembd, s.nkind1, s.rhod = 1, 1, 1.0
        s.fembd, s.dfembd = _d(self.keep[4]), _d(self.keep[5])
        s.ngroup = ng
        s.kpair = _i(self.kpair)
        s.kembd = _i(self.kembd)
        self.s = s


def read_setfl(path):
    """Setfl file (Filedatas_Func_Setfl.F90:119-253): elements, grids, and per element F(rho)
    and rho(r), then r*phi(r) for every pair i >= j.  'INF' / 'NAN' as the first value of a
    rho / r*phi block stand for the r = 0 entry, which takes the next value."""
    lines = open(path).read().split("\n")
    el = lines[3].split()
    ne = int(float(el[0]))
    g = lines[4].split()
    nrho, drho, nr, dr, cutoff = int(g[0]), float(g[1]), int(g[2]), float(g[3]), float(g[4])
    toks = " ".join(lines[5:]).split()
    pos = 0
    out = dict(elements=el[1:1 + ne], nrho=nrho, drho=drho, nr=nr, dr=dr, cutoff=cutoff,
               mass=[], frho=[], rhor=[], rphi={})

    def block(n):
        nonlocal pos
        v = toks[pos:pos + n]
        pos += n
        vals = np.array([np.nan if x.upper() in ("INF", "NAN") else float(x) for x in v])
        if np.isnan(vals[0]):
            vals[0] = vals[1]
        return vals

    for _ in range(ne):
        out["mass"].append(float(toks[pos + 1]))
        pos += 4
        out["frho"].append(block(nrho))
        out["rhor"].append(block(nr))
    for i in range(ne):
        for j in range(i + 1):
            out["rphi"][(i, j)] = block(nr)
    return out


def setfl_tables(d, ntab=10000, i=0, j=None):
    """Tables of an element-i atom with an element-j neighbour (default j = i) from
    read_setfl output: pair phi_ij, density of element j, embedding of element i; RHOD = drho."""
    j = i if j is None else j
    potr, fpotr, potb, fpotb = (np.zeros(ntab) for _ in range(4))
    fe, dfe = np.zeros(d["nrho"]), np.zeros(d["nrho"])
    rc = lib().orc_setfl_tables(d["nrho"], C.c_double(d["drho"]), d["nr"], C.c_double(d["cutoff"]),
                                _d(f64(d["frho"][i])), _d(f64(d["rhor"][j])),
                                _d(f64(d["rphi"][(max(i, j), min(i, j))])),
                                ntab, _d(potr), _d(fpotr), _d(potb), _d(fpotb), _d(fe), _d(dfe))
    if rc != 0:
        raise RuntimeError("oracle setfl tables failed")
    return dict(potr=potr, fpotr=fpotr, potb=potb, fpotb=fpotb, fembd=fe, dfembd=dfe, rhod=d["drho"],
                ntab=ntab, nembd=d["nrho"], rmax=d["cutoff"])


def _ctl_lines(path, skip):
    """Non-comment lines as GETINPUTSTRLINE returns them (LIB/sor/f/MiniUtilities/
    GETINPUTSTRLINE.F): printable characters (codes 20..126), left-adjusted, blank lines and
    lines starting with a character of `skip` dropped."""
    out = []
    for raw in open(path, "rb").read().split(b"\n"):
        s = "".join(chr(c) for c in raw if 20 <= c <= 126).lstrip(" ")
        if s and s[0] not in skip:
            out.append(s)
    return out


def _quoted(s):
    """Substrings between matching quotes (LIB/sor/f/MiniUtilities/EXSUBSTR.F)."""
    out, i = [], 0
    while i < len(s):
        if s[i] in "\"'":
            e = s.find(s[i], i + 1)
            if e < 0:
                break
            out.append(s[i + 1:e])
            i = e + 1
        else:
            i += 1
    return out


def _read_spt(path):
    rows = [ln.split() for ln in _ctl_lines(path, "#")]
    a = np.array([[float(r[0]), float(r[1])] for r in rows])
    return a[:, 0].copy(), a[:, 1].copy()


def read_lspt(path, each_vr_file=False):
    """lspt control file and its ".spt" files (get_filedatas_lspt, Filedatas_Func_Lspt.F90:
    118-301).  Pair line I quotes I files; the reference opens the first of them for every
    pair of the line (:263), which each_vr_file=False reproduces."""
    folder = os.path.dirname(path)
    ln = _ctl_lines(path, "!")
    if not ln[0].split()[0].upper().startswith("&LSPT"):
        raise ValueError("no &LSPT block")
    ne = int(re.search(r"\d+", ln[1]).group(0))
    el = [q.strip() for q in _quoted(ln[2])]
    assert len(el) == ne
    d = dict(elements=el, frho=[], rhor=[], vr={})
    k = 3
    for e in range(ne):
        for key in ("frho", "rhor"):
            name = _quoted(ln[k])[0].strip()
            k += 1
            d[key].append(None if name.upper() == "NA" else _read_spt(os.path.join(folder, name)))
    for i in range(ne):
        q = _quoted(ln[k])
        k += 1
        assert len(q) == i + 1
        for j in range(i + 1):
            d["vr"][(i, j)] = _read_spt(os.path.join(folder, (q[j] if each_vr_file else q[0]).strip()))
    d["rmax"] = max(v[0][-1] for v in d["vr"].values())
    d["rhomax"] = max([0.0] + [f[0][-1] for f in d["frho"] if f is not None])
    return d


def _spt_eval(xy, t, keep_above):
    """Vr_Spline / Rhor_Spline / Frho_Spline range rules (Filedatas_Func_Lspt.F90:340-500):
    natural spline inside the data, the first value with zero slope below it, and above it
    zero (V, rho) or the last value with zero slope (F)."""
    t = np.asarray(t, np.float64)
    f, df = np.zeros_like(t), np.zeros_like(t)
    if xy is None:
        return f, df
    x, y = f64(xy[0]), f64(xy[1])
    m = np.zeros_like(x)
    lib().orc_spline_knots(len(x), _d(x), _d(y), _d(m))
    tc = np.clip(t, x[0], x[-1])
    lib().orc_spline_knots_eval(len(x), _d(x), _d(y), _d(m), len(tc), _d(f64(tc)), _d(f), _d(df))
    inside = (t >= x[0]) & (t <= x[-1])
    df = np.where(inside, df, 0.0)
    if not keep_above:
        f = np.where(t > x[-1], 0.0, f)
    return f, df


def lspt_tables(d, ntab=10000, nembd=10000, rmax=None):
    """All NE^2 pair tables (column (I, J) = I * NE + J: V of the pair, density of element J at
    an element-I host, zero when element I has no F(rho)) on the sqrt(r) grid up to rmax (the
    pair files' largest r) and the NE embedding tables on RHOD = largest F(rho) knot / nembd,
    the reader's RHOMX that Generate_NIST_ForceTalbe keeps (NIST_ForceTable.F90:379-413)."""
    ne = len(d["elements"])
    rmax = d["rmax"] if rmax is None else rmax
    r = (np.arange(1, ntab + 1) * (np.sqrt(rmax) / ntab)) ** 2
    potr, fpotr, potb, fpotb = (np.zeros((ntab, ne * ne)) for _ in range(4))
    for i in range(ne):
        for j in range(ne):
            c = i * ne + j
            v, dv = _spt_eval(d["vr"][(max(i, j), min(i, j))], r, False)
            potr[:, c], fpotr[:, c] = 0.5 * v * r, -dv * r
            if d["frho"][i] is not None:
                rho, drho = _spt_eval(d["rhor"][j], r, False)
                potb[:, c], fpotb[:, c] = rho, -drho
    rhod = d["rhomax"] / nembd if d["rhomax"] > 0.0 else 1.0
    fembd, dfembd = np.zeros((nembd, ne)), np.zeros((nembd, ne))
    for e in range(ne):
        fembd[:, e], dfembd[:, e] = _spt_eval(d["frho"][e], np.arange(nembd) * rhod, True)
    kpair = np.arange(1, ne * ne + 1, dtype=np.int32).reshape(ne, ne)   # KPAIR(I, J) at [I-1, J-1]
    return dict(potr=potr, fpotr=fpotr, potb=potb, fpotb=fpotb, fembd=fembd, dfembd=dfembd,
                rhod=rhod, kpair=kpair, kembd=np.arange(1, ne + 1, dtype=np.int32), ntab=ntab,
                nembd=nembd, rmax=rmax)


def bonny_tables(sub, rmax=5.4604375, ntab=10000, nembd=10000, rhoscal=20.0):
    """Bonny W-H-He EAM tables (sub 1 = EAM1, 2 = EAM2): NKIND = 9 (10) pair/density tables on
    the sqrt(r) grid up to rmax, POTR = (V/2) r, FPOTR = -V' r, POTB = rho, FPOTB = -rho'
    (Create_Pairwise_ForceTable, MD_TypeDef_ForceTable.F90:949-976); embedding tables of W, H,
    He on RHOD = rhoscal * max POTB / nembd (:965, 1040-1048); KPAIR(I, J) = (I-1)*3 + J with
    I the host (groups W, H, He)."""
    nk = 10 if sub == 2 else 9
    r = (np.arange(1, ntab + 1) * (np.sqrt(rmax) / ntab)) ** 2
    out = {k: np.zeros((ntab, nk)) for k in ("potr", "fpotr", "potb", "fpotb")}
    a, b, c, d = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    for t in range(nk):
        for i, ri in enumerate(r):
            if lib().orc_bonny_pair(sub, t + 1, C.c_double(ri), C.byref(a), C.byref(b), C.byref(c), C.byref(d)):
                raise RuntimeError("unknown Bonny table")
            out["potr"][i, t], out["fpotr"][i, t] = a.value * ri, b.value * ri
            out["potb"][i, t], out["fpotb"][i, t] = c.value, d.value
    rhod = rhoscal * out["potb"].max() / nembd
    fe, dfe = np.zeros((nembd, 3)), np.zeros((nembd, 3))
    for g in range(3):
        for i in range(nembd):
            lib().orc_bonny_embed(sub, g + 1, C.c_double(i * rhod), C.byref(a), C.byref(b))
            fe[i, g], dfe[i, g] = a.value, b.value
    out.update(fembd=fe, dfembd=dfe, rhod=rhod, nkind=nk, rmax=rmax,
               kpair=np.arange(1, 10, dtype=np.int32).reshape(3, 3), kembd=np.arange(1, 4, dtype=np.int32))
    return out


def read_moldy(path):
    """Moldy file (get_filedatas_moldy, Filedatas_Func_Moldy.F90:27-77): symbol, then the
    numbers of four lines (pair a_k, pair r_k, density A_k, density R_k) and of a constants
    line whose first entry is the lattice constant; knots scaled by it, a_k by its -3rd and
    A_k by its -6th power."""
    lines = open(path).read().split("\n")

    def nums(s):
        out = []
        for tok in re.split(r"[ \t,()\[\]{}=]+", s.strip()):
            try:
                out.append(float(tok))
            except ValueError:
                pass
        return np.array(out)

    av, rv, ab, rb, c = (nums(lines[k]) for k in range(1, 6))
    a0 = c[0]
    return dict(symbol=lines[0].strip(), av=av / a0 ** 3, rv=rv * a0, ab=ab / a0 ** 6, rb=rb * a0, a0=a0)


def moldy_tables(d, rmax, ntab=10000, nembd=10000, rhoscal=20.0):
    """Moldy tables: V = sum a (r_k - r)^3 [r <= r_k] (POTR = V r / 2, FPOTR = -V' r),
    rho = sum A (R_k - r)^3 [r <= R_k], F = -sqrt(rho) on RHOD = rhoscal max POTB / nembd."""
    r = (np.arange(1, ntab + 1) * (np.sqrt(rmax) / ntab)) ** 2
    x = d["rv"][None, :] - r[:, None]
    h = (x >= 0.0)
    v = (d["av"] * x ** 3 * h).sum(1)
    mdv = 3.0 * (d["av"] * x ** 2 * h).sum(1)
    y = d["rb"][None, :] - r[:, None]
    g = (y >= 0.0)
    rho = (d["ab"] * y ** 3 * g).sum(1)
    mdrho = 3.0 * (d["ab"] * y ** 2 * g).sum(1)
    rhod = rhoscal * rho.max() / nembd
    q = np.arange(nembd) * rhod
    safe = np.where(q > 0.0, q, 1.0)
    return dict(potr=0.5 * v * r, fpotr=mdv * r, potb=rho, fpotb=mdrho, rhod=rhod, ntab=ntab, nembd=nembd,
                rmax=rmax, fembd=np.where(q > 0.0, -np.sqrt(safe), 0.0),
                dfembd=np.where(q > 0.0, -0.5 / np.sqrt(safe), 0.0))


def make_box(lo, length, ifpd=(1, 1, 1), shape=None):
    """shape: BOXSHAPE as a 3x3 array (row K maps SEP to DXYZ(K)); None = cubic."""
    b = OrcBox()
    for k in range(3):
        b.lo[k] = float(lo[k])
        b.len[k] = float(length[k])
        b.ifpd[k] = int(ifpd[k])
    bs = np.eye(3) if shape is None else np.asarray(shape, np.float64).reshape(3, 3)
    for m in range(9):
        b.bs[m] = float(bs.reshape(-1)[m])
    b.shaped = 0 if shape is None or np.array_equal(bs, np.eye(3)) else 1
    return b


def nlist(pos, statu, box, rc_nl, mxkvois=128, brute=False):
    n = pos.shape[0]
    x, y, z = (f64(pos[:, k]) for k in range(3))
    st = i32(statu)
    kvois = np.zeros(n, np.int32)
    indi = np.zeros(n * mxkvois, np.int32)
    if brute:
        rc = lib().orc_nlist_brute(n, _d(x), _d(y), _d(z), _i(st), C.byref(box),
                                   C.c_double(rc_nl), mxkvois, _i(kvois), _i(indi))
    else:
        nc = np.zeros(3, np.int32)
        rc = lib().orc_nlist(n, _d(x), _d(y), _d(z), _i(st), C.byref(box), C.c_double(rc_nl),
                             mxkvois, _i(kvois), _i(indi), _i(nc))
    if rc != 0:
        raise RuntimeError("oracle neighbour list failed: %d" % rc)
    return kvois, indi.reshape(mxkvois, n)


def force(pos, ityp, statu, box, kvois, indi, tables, want_virial=True, want_epot=True,
          nthreads=0):
    n = pos.shape[0]
    x, y, z = (f64(pos[:, k]) for k in range(3))
    ty, st = i32(ityp), i32(statu)
    kv = i32(kvois)
    ind = i32(indi)
    ldi = ind.shape[1] if ind.ndim == 2 else n
    den = np.zeros(n)
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    epot = np.zeros(n) if want_epot else None
    vir = np.zeros(9) if want_virial else None
    nbad = lib().orc_force(n, _d(x), _d(y), _d(z), _i(ty), _i(st), C.byref(box), _i(kv),
                           _i(ind), ldi, C.byref(tables.s), _d(den), _d(fx), _d(fy), _d(fz),
                           _d(epot) if want_epot else None, _d(vir) if want_virial else None,
                           nthreads)
    return dict(den=den, f=np.stack([fx, fy, fz], 1), epot=epot,
                vir=vir.reshape(3, 3) if want_virial else None, nbad=nbad)


def atomic_stress(pos, ityp, statu, box, kvois, indi, tables, den, nthreads=0):
    """Per-atom virial tensors, shape (N, 3, 3); den = F'(rho) from force()."""
    n = pos.shape[0]
    x, y, z = (f64(pos[:, k]) for k in range(3))
    kv, ind = i32(kvois), i32(indi)
    ap = np.zeros(9 * n)
    lib().orc_atomic_stress(n, _d(x), _d(y), _d(z), _i(i32(ityp)), _i(i32(statu)), C.byref(box),
                            _i(kv), _i(ind), ind.shape[1] if ind.ndim == 2 else n, C.byref(tables.s),
                            _d(f64(den)), _d(ap), nthreads)
    return ap.reshape(9, n).T.reshape(n, 3, 3).copy()


def hvp(pos, ityp, statu, box, kvois, indi, tables, v, nthreads=0):
    n = pos.shape[0]
    x, y, z = (f64(pos[:, k]) for k in range(3))
    vx, vy, vz = (f64(v[:, k]) for k in range(3))
    ty, st = i32(ityp), i32(statu)
    kv, ind = i32(kvois), i32(indi)
    hx, hy, hz = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().orc_hvp(n, _d(x), _d(y), _d(z), _i(ty), _i(st), C.byref(box), _i(kv), _i(ind),
                  ind.shape[1] if ind.ndim == 2 else n, C.byref(tables.s), _d(vx), _d(vy),
                  _d(vz), _d(hx), _d(hy), _d(hz), nthreads)
    return np.stack([hx, hy, hz], 1)


def md(pos, vel, ityp, statu, box, tables, cm, h, nsteps, rc_nl, skin_trigger=0.0, nb_uptab=10,
       mxkvois=128, nthreads=0, fext=None):
    """Runs the NVE loop in place on copies; returns (pos, vel, force, statu, rebuilds).
    fext (N, 3): external force added to every active atom after each force evaluation."""
    n = pos.shape[0]
    x, y, z = (f64(pos[:, k]).copy() for k in range(3))
    vx, vy, vz = (f64(vel[:, k]).copy() for k in range(3))
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    st = i32(statu).copy()
    ty = i32(ityp)
    cmv = f64(cm)
    fe = None if fext is None else f64(np.asarray(fext, np.float64).T.reshape(-1))
    rc = lib().orc_md_ext(n, _d(x), _d(y), _d(z), _d(vx), _d(vy), _d(vz), _d(fx), _d(fy), _d(fz),
                          _i(st), _i(ty), C.byref(box), C.byref(tables.s), _d(cmv), C.c_double(h),
                          nsteps, C.c_double(rc_nl), C.c_double(skin_trigger), nb_uptab, mxkvois,
                          nthreads, _d(fe) if fe is not None else None)
    if rc < 0:
        raise RuntimeError("oracle md failed: %d" % rc)
    return (np.stack([x, y, z], 1), np.stack([vx, vy, vz], 1), np.stack([fx, fy, fz], 1), st, rc)


def cr_dtables(prm, rmax, ntab=10000):
    prm = f64(prm)
    d = np.zeros(15 * ntab)
    lib().orc_cr_dtables(_d(prm), C.c_double(rmax), ntab, _d(d))
    return d


def adjoint_cr(pos, ityp, statu, box, kvois, indi, tables, dtab, ft, nthreads=0):
    n = pos.shape[0]
    x, y, z = (f64(pos[:, k]) for k in range(3))
    tx, ty_, tz = (f64(ft[:, k]) for k in range(3))
    kv, ind = i32(kvois), i32(indi)
    loss = C.c_double()
    grad = np.zeros(5)
    d = f64(dtab)
    lib().orc_adjoint_cr(n, _d(x), _d(y), _d(z), _i(i32(ityp)), _i(i32(statu)), C.byref(box),
                         _i(kv), _i(ind), ind.shape[1] if ind.ndim == 2 else n, C.byref(tables.s),
                         _d(d), _d(tx), _d(ty_), _d(tz), C.byref(loss), _d(grad), nthreads)
    return loss.value, grad


# ---- tables the reference exported, read back -------------------------------------------
EVERG, A2CM = 1.60219e-12, 1e-8        # MSM_Const.F90:67, 83


def read_imported(path, ncol):
    """One exported table file (Import_ForceTable, MD_TypeDef_ForceTable.F90:1485-1527):
    header lines until "&#" -- &POTTYPE "name", &NUMTABLE NC followed by the NC table ids,
    &NUMPOINT NT (comment lines start with "!") -- then NT rows of index, x and ncol numbers
    per table, read as a stream of numbers (list-directed READ)."""
    pottype, ids, npt = None, None, None
    with open(path) as fh:
        lines = fh.read().splitlines()
    k = 0
    while k < len(lines):
        s = lines[k].strip()
        k += 1
        if not s.startswith("&"):
            continue
        key = s.split()[0].upper()
        if key == "&NUMTABLE":
            nums = [int(v) for v in re.findall(r"\d+", s[len("&NUMTABLE"):])]
            ids = nums[1:1 + nums[0]]
        elif key == "&NUMPOINT":
            npt = int(s.split()[1])
        elif key == "&POTTYPE":
            m = re.search(r'"([^"]*)"', s)
            pottype = m.group(1) if m else s.split()[1]
        elif key.startswith("&#"):
            break
    vals = np.array(" ".join(lines[k:]).split()[: npt * (2 + ncol * len(ids))], np.float64)
    rows = vals.reshape(npt, 2 + ncol * len(ids))
    return dict(pottype=pottype.strip().upper(), ids=ids, x=rows[:, 1].copy(),
                cols=rows[:, 2:].reshape(npt, len(ids), ncol))


def import_tables(stem, ptype, rmax, ntab=10000, nembd=10000, cgs=False):
    """Register_Imported_ForceTable (MD_TypeDef_ForceTable.F90:1612-1855) for a box of groups
    whose pairs use the file tables PTYPE (NGROUP x NGROUP, host first): the named tables in
    first-appearance order (New_ForceTable :560-574, 600-610), unit conversion of the import
    (:1529-1540, 1583-1585; the files are in A / eV, `cgs` gives the reference's CGS tables),
    pair columns re-gridded by SPLID1/SPLID2 onto T = K/CSI, embedding columns onto
    rho = (K-1) RHOD, RHOD = RHO(N) N/(N-1) / NEMBD.  Returns the dict layout of lspt_tables
    (arrays (NTAB, NKIND), kpair (NGROUP, NGROUP) with KPAIR(I, J) at [I-1, J-1])."""
    pair = read_imported(stem + ".pair", 4)
    embd = read_imported(stem + ".embd", 2)
    eam = pair["pottype"] == "EAM_TYPE"
    rhounit = 1.0 / (EVERG * EVERG) if (cgs and not eam) else 1.0
    fx = A2CM if cgs else 1.0
    fc = np.array([0.5 * (EVERG * A2CM if cgs else 1.0), EVERG if cgs else 1.0, 1.0 / rhounit,
                   (1.0 / A2CM if cgs else 1.0) / rhounit])
    r = pair["x"] * fx
    pcols = pair["cols"] * fc[None, None, :]
    rho = embd["x"] / rhounit
    ecols = embd["cols"].copy()
    ecols[:, :, 0] *= EVERG if cgs else 1.0
    if not cgs:
        ecols[:, :, 1] /= EVERG
    ptype = np.asarray(ptype, np.int32)
    ng = ptype.shape[0]
    order = []
    for i in range(ng):
        for j in range(ng):
            if int(ptype[i, j]) not in order:
                order.append(int(ptype[i, j]))
    kpair = np.array([[order.index(int(ptype[i, j])) + 1 for j in range(ng)] for i in range(ng)], np.int32)
    nk = len(order)
    out = {name: np.zeros((ntab, nk)) for name in ("potr", "fpotr", "potb", "fpotb")}
    for k, tid in enumerate(order):
        q = pair["ids"].index(tid)
        for c, name in enumerate(("potr", "fpotr", "potb", "fpotb")):
            col = np.zeros(ntab)
            lib().orc_import_regrid_pair(len(r), _d(f64(r)), _d(f64(pcols[:, q, c])), C.c_double(rmax), ntab,
                                         _d(col))
            out[name][:, k] = col
    ne = len(rho)
    rhod = (rho[-1] / float(ne - 1)) * float(ne) / float(nembd)
    if rhod <= 1e-64:
        rhod = 1.0
    emb = []
    for i in range(ng):
        if int(ptype[i, i]) not in emb:
            emb.append(int(ptype[i, i]))
    kembd = np.array([emb.index(int(ptype[i, i])) + 1 for i in range(ng)], np.int32)
    fembd, dfembd = np.zeros((nembd, len(emb))), np.zeros((nembd, len(emb)))
    if eam:
        for k, tid in enumerate(emb):
            q = embd["ids"].index(tid)
            for c, dst in ((0, fembd), (1, dfembd)):
                col = np.zeros(nembd)
                lib().orc_import_regrid_embd(ne, _d(f64(rho)), _d(f64(ecols[:, q, c])), C.c_double(rhod), nembd,
                                             _d(col))
                dst[:, k] = col
    return dict(potr=out["potr"], fpotr=out["fpotr"], potb=out["potb"], fpotb=out["fpotb"],
                fembd=fembd if eam else None, dfembd=dfembd if eam else None, rhod=rhod, kpair=kpair,
                kembd=kembd, ntab=ntab, nembd=nembd, rmax=rmax, pottype=EAM if eam else FS, ids=order)
