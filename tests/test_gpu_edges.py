"""GPU edge cases against the oracle: two atom types with asymmetric density tables
(KPAIR(1,2) != KPAIR(2,1)), non-periodic directions with atoms leaving the box, and the
FIXPOS / FIXVEL status bits of the integrator."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt
from msmpscu_gb300 import _lib as L
from tests.helpers import cu_tables, rel_err, sorted_sets, CR_PRM

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _two_species_tables(oracle, ntab=10000):
    """Four CR tables: 1-1, 2-2, and two different cross densities 1<-2 and 2<-1."""
    base = np.array(CR_PRM)
    prms = [base, base * np.array([1.1, 0.95, 1.0, 1.05, 1.0]),
            base * np.array([1.05, 1.02, 0.98, 1.0, 1.0]), base * np.array([1.05, 0.97, 0.98, 1.03, 1.0])]
    cols = {k: [] for k in ("potr", "fpotr", "potb", "fpotb")}
    for p in prms:
        t = oracle.make_tables(oracle.POT_CR, p, lt.CU_RC, ntab, ntab, 20.0, want_embed=False)
        for k in cols:
            cols[k].append(t[k])
    arr = {k: np.stack(v, 1) for k, v in cols.items()}          # (NTAB, NKIND)
    kpair = np.array([[1, 3], [4, 2]])                          # KPAIR(1,2)=3, KPAIR(2,1)=4
    return arr, kpair


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_two_species_asymmetric_density(oracle, precision):
    pos, vel, L_ = lt.cu_config(8, 0.05, 300.0, 31)
    n = len(pos)
    rng = np.random.default_rng(3)
    ityp = (rng.random(n) < 0.3).astype(np.int32) + 1
    arr, kpair = _two_species_tables(oracle)
    ot = oracle.RawTables(oracle.FS, 10000, 4, lt.CU_RC, lt.CU_RC, arr["potr"], arr["fpotr"],
                          arr["potb"], arr["fpotb"], kpair)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(pos, ityp, st, box, kv, ind, ot)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision=precision)
    e.init_forcetable_raw(L.FS_TYPE, 10000, 4, lt.CU_RC, lt.CU_RC, arr["potr"], arr["fpotr"],
                          arr["potb"], arr["fpotb"], 2, kpair)
    e.set_masses([lt.CU_MASS, 1.3 * lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp)
    e.calforce()
    f = e.get_force()
    if precision == "fp64":
        assert rel_err(f, ref["f"]) < TOL
        vir = e.calptensor()[0]
        assert rel_err(vir, ref["vir"]) < TOL
        e.calepot()
        assert rel_err(e.get_epot(), ref["epot"]) < TOL
    else:
        assert np.linalg.norm(f - ref["f"]) / np.linalg.norm(ref["f"]) < 1e-6
    # MD with two masses (unfused mixed path / FP64 graph)
    cm = np.array([lt.CU_MASS, 1.3 * lt.CU_MASS])
    ox, ov, _, _, _ = oracle.md(pos, vel, ityp, st, box, ot, cm, 1.0, 20, lt.CU_RC_NL, skin_trigger=0.15,
                                mxkvois=96)
    e.run_steps(20, 1.0)
    gx, gv, _, _ = e.get_state()
    dx = gx - ox
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < (1e-9 if precision == "fp64" else 1e-6)
    e.close()


def test_non_periodic_z_atoms_leave_box(oracle):
    """z not periodic: a slab whose top atoms fly out; statuses and forces match the oracle."""
    pos, vel, L_ = lt.cu_config(6, 0.02, 300.0, 41)
    n = len(pos)
    Lz = L_[2] + 4.0                      # vacuum above the slab
    top = pos[:, 2] > L_[2] - 2.0
    vel = vel.copy()
    vel[top, 2] = 0.2                     # 0.2 A/fs upward
    box_len = np.array([L_[0], L_[1], Lz])
    t = cu_tables(oracle)
    obox = oracle.make_box([0, 0, 0], box_len, ifpd=(1, 1, 0))
    st = np.ones(n, np.int32)
    ox, ov, of, ost, _ = oracle.md(pos, vel, np.ones(n, np.int32), st, obox, t, np.array([lt.CU_MASS]),
                                   1.0, 40, lt.CU_RC_NL, skin_trigger=0.15, mxkvois=96)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(box_len), (1, 1, 0))], pos, vel)
    e.run_steps(40, 1.0)
    gx, gv, gst, _ = e.get_state()
    assert np.array_equal(gst, ost)
    assert (ost & L.STATU_OUTOFBOX).sum() > 0
    act = (ost & L.STATU_ACTIVE) == L.STATU_ACTIVE
    dx = gx - ox
    dx[:, :2] -= np.round(dx[:, :2] / box_len[:2]) * box_len[:2]
    assert np.abs(dx[act]).max() < 1e-8
    e.close()


@pytest.mark.parametrize("precision", ["fp64", "ff", "mixed"])
def test_fixpos_fixvel_bits(oracle, precision):
    """Fixed positions and velocities stay bit for bit in every precision, the mixed passes'
    form of the update included; the trajectory follows the oracle's."""
    pos, vel, L_ = lt.cu_config(6, 0.05, 600.0, 51)
    n = len(pos)
    st = np.ones(n, np.int32)
    st[::5] |= L.STATU_FIXPOSX | L.STATU_FIXPOSY | L.STATU_FIXPOSZ
    st[1::7] |= L.STATU_FIXVELZ
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L_)
    ox, ov, _, ost, _ = oracle.md(pos, vel, np.ones(n, np.int32), st, box, t, np.array([lt.CU_MASS]),
                                  1.0, 30, lt.CU_RC_NL, skin_trigger=0.15, mxkvois=96)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64, precision=precision)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, statu=st)
    e.run_steps(30, 1.0)
    gx, gv, gst, _ = e.get_state()
    assert np.array_equal(gst, ost)
    assert np.array_equal(gx[::5], pos[::5])                 # fixed atoms did not move
    assert np.array_equal(gv[::5], vel[::5])
    assert np.array_equal(gv[1::7, 2], vel[1::7, 2])         # fixed z-velocities unchanged
    dx = gx - ox
    dx -= np.round(dx / L_) * L_
    assert np.abs(dx).max() < (1e-6 if precision == "mixed" else 1e-8)
    e.close()


@pytest.mark.parametrize("kind", ["cu", "w", "two_species"])
def test_atomic_stress_parity(oracle, kind):
    """pCalAVStress: per-atom virial tensors against the oracle (FP64, 1e-10), both orders."""
    from tests.helpers import w_tables
    if kind == "w":
        pos, L_ = lt.w_sia_config(6, 0.02, 12)
        vel = np.zeros_like(pos)
        t = w_tables(oracle)
        rc_nl, ityp = lt.W_RC_NL, np.ones(len(pos), np.int32)
    else:
        pos, vel, L_ = lt.cu_config(8, 0.05, 300.0, 33)
        rc_nl = lt.CU_RC_NL
        ityp = np.ones(len(pos), np.int32)
        t = cu_tables(oracle)
    n = len(pos)
    st = np.ones(n, np.int32)
    box = oracle.make_box([0, 0, 0], L_)
    e = Engine(n, rc_nl, mxkvois=96)
    if kind == "two_species":
        ityp = (np.random.default_rng(8).random(n) < 0.4).astype(np.int32) + 1
        arr, kpair = _two_species_tables(oracle)
        t = oracle.RawTables(oracle.FS, 10000, 4, lt.CU_RC, lt.CU_RC, arr["potr"], arr["fpotr"],
                             arr["potb"], arr["fpotb"], kpair)
        e.init_forcetable_raw(L.FS_TYPE, 10000, 4, lt.CU_RC, lt.CU_RC, arr["potr"], arr["fpotr"],
                              arr["potb"], arr["fpotb"], 2, kpair)
    elif kind == "w":
        e.init_forcetable(ForceTable.marinica_eam2(rc=lt.W_RC))
    else:
        e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    kv, ind = oracle.nlist(pos, st, box, rc_nl, 128)
    ref = oracle.force(pos, ityp, st, box, kv, ind, t)
    ap_ref = oracle.atomic_stress(pos, ityp, st, box, kv, ind, t, ref["den"])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp)
    ap = e.atomic_stress()
    assert rel_err(ap, ap_ref) < TOL
    aps = e.atomic_stress(order=L.ORDER_SORTED)
    gid = e.get_gid()
    assert np.array_equal(aps, ap[gid])
    e.close()


def test_atomic_stress_sum_is_twice_virial_large():
    """256,000 atoms: the per-atom tensors add up to twice the box virial of calptensor."""
    pos, vel, L_ = lt.cu_config(40, 0.05, 600.0, 7)
    n = len(pos)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    vir = e.calptensor()[0]
    ap = e.atomic_stress()
    assert np.allclose(ap, ap.transpose(0, 2, 1), rtol=0, atol=1e-9 * np.abs(ap).max())
    assert rel_err(ap.sum(0), 2.0 * vir) < 1e-9
    e.close()


@pytest.mark.parametrize("precision", ["fp64", "ff", "mixed"])
def test_embedding_density_beyond_table_reported(precision):
    """EAM: an F(rho) table that ends below the crystal's electron density (RHOMX = 0.5 max
    POTB) is reported as MSMGB_ERR_RHO_RANGE by every precision; with a proper table the same
    context then computes forces."""
    pos, L_ = lt.w_sia_config(6, 0.02, 4)
    n = len(pos)
    e = Engine(n, lt.W_RC_NL, mxkvois=96, precision=precision)
    e.init_forcetable(ForceTable.marinica_eam2(rhoscal=0.5))
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos)
    with pytest.raises(MSMError) as ei:
        e.calforce()
    assert ei.value.code == L.ERR_RHO_RANGE
    e.init_forcetable(ForceTable.marinica_eam2())
    e.calforce()
    assert np.isfinite(e.get_force()).all()
    e.close()


def test_non_finite_positions_rejected(oracle):
    """A NaN or infinite coordinate is an argument error: at copy-in (checked in the pack
    kernel; the context is left without a state until a valid copy-in) and in a position
    update (the atom keeps its old position)."""
    from msmpscu_gb300 import MSMError
    from msmpscu_gb300 import _lib as L
    pos, vel, L_ = lt.cu_config(5, 0.05, 300.0, 3)
    n = len(pos)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    bad = pos.copy()
    bad[7, 1] = np.nan
    with pytest.raises(MSMError) as ex:
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], bad)
    assert ex.value.code == L.ERR_ARG
    with pytest.raises(MSMError):
        e.calforce()                        # no state after the failed copy-in
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos)
    e.calforce()
    f0 = e.get_force()
    upd = pos.copy()
    upd[11, 2] = np.inf
    with pytest.raises(MSMError) as ex:
        e.update_positions(upd)
    assert ex.value.code == L.ERR_ARG
    e.update_positions(pos)                 # the context stays usable
    e.calforce()
    assert np.array_equal(e.get_force(), f0)
    e.close()


def test_list_validation_mode(oracle, monkeypatch):
    """MSMGB_CHECK_LISTS=1 validates every list after its build (indices in range, not the atom
    itself, same box, counts within MXKVOIS) with an extra kernel; a correct run passes it,
    including the rebuilds inside the MD step graphs, and gives the same trajectory."""
    pos, vel, L_ = lt.cu_config(6, 0.05, 900.0, 13)
    n = len(pos)
    out = []
    for flag in ("0", "1"):
        monkeypatch.setenv("MSMGB_CHECK_LISTS", flag)
        e = Engine(n, lt.CU_RC_NL, mxkvois=64, skin_trigger=0.05)
        e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
        e.set_masses([lt.CU_MASS])
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        l0 = e.launches
        e.run_steps(40, 1.0)
        out.append((e.get_state()[0], e.launches - l0))
        e.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert out[1][1] > out[0][1]           # the validation kernel ran


def _sparse_config():
    """Isolated atoms (empty lists, rho = 0), a dimer and a 13-atom fcc cluster in a large
    periodic box."""
    L_ = np.array([40.0, 40.0, 40.0])
    iso = np.array([[3.0, 3.0, 3.0], [35.0, 5.0, 20.0], [20.0, 35.0, 8.0]])
    dimer = np.array([[10.0, 30.0, 30.0], [12.4, 30.3, 30.1]])
    a = lt.CU_A
    cl = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5], [-0.5, 0.5, 0], [0.5, -0.5, 0],
                   [-0.5, -0.5, 0], [-0.5, 0, 0.5], [0.5, 0, -0.5], [-0.5, 0, -0.5], [0, -0.5, 0.5],
                   [0, 0.5, -0.5], [0, -0.5, -0.5]]) * a + np.array([20.0, 20.0, 20.0])
    cl = cl + np.random.default_rng(4).normal(scale=0.05, size=cl.shape)
    return np.vstack([iso, dimer, cl]), L_


@pytest.mark.parametrize("kind", ["fs", "eam"])
def test_isolated_atoms_dimer_cluster(oracle, kind):
    pos, L_ = _sparse_config()
    n = len(pos)
    if kind == "fs":
        ft, t, rc = ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC), cu_tables(oracle), lt.CU_RC_NL
    else:
        from tests.helpers import w_tables
        ft, t, rc = ForceTable.marinica_eam2(), w_tables(oracle), lt.W_RC_NL
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, rc, 64)
    assert (kv == 0).sum() == 3
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)
    for precision in ("fp64", "ff", "mixed"):
        e = Engine(n, rc, mxkvois=64, precision=precision)
        e.init_forcetable(ft)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos)
        e.calforce()
        f = e.get_force()
        assert np.all(f[:3] == 0.0), precision
        tol = 1e-6 if precision == "mixed" else 1e-10
        assert np.abs(f - ref["f"]).max() <= tol * np.abs(ref["f"]).max(), precision
        if precision != "mixed":
            e.calepot()
            assert rel_err(e.get_epot(), ref["epot"]) < 1e-10, precision
        e.close()


def test_atoms_on_box_faces(oracle):
    """Atoms exactly on the lower faces and on the upper faces (x = lo + L) of a periodic
    box: binned inside (the reference's -1e-4 cell rule), same neighbour sets and forces as
    the oracle."""
    pos, vel, L_ = lt.cu_config(6, 0.0, 0.0, 1)              # the exact lattice
    pos = pos.copy()
    a = lt.CU_A

    def site(p):
        return int(np.nonzero(np.all(np.abs(pos - p) < 1e-9, axis=1))[0][0])

    i1, i2, i3 = site([0.0, 0.5 * a, 0.5 * a]), site([0.5 * a, 0.0, 0.5 * a]), site([0.0, 0.0, 0.0])
    i0 = site([0.0, 0.0, a])                                   # stays on the lower x and y faces
    face = pos[[i0, i1, i2, i3]].copy()
    face[1, 0] = L_[0]                                         # x = L face
    face[2, 1] = L_[1]                                         # y = L face
    face[3] = L_                                               # the far corner
    pos = pos + np.random.default_rng(2).normal(scale=0.05, size=pos.shape)
    pos -= np.floor(pos / L_) * L_
    pos[[i0, i1, i2, i3]] = face
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, cu_tables(oracle))
    e = Engine(n, lt.CU_RC_NL, mxkvois=96)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos)
    e.cal_neighborelist()
    gk, gi = e.get_neighborelist()
    assert sorted_sets(gk, gi) == sorted_sets(kv, ind)
    e.calforce()
    assert rel_err(e.get_force(), ref["f"]) < 1e-10
    e.close()


def test_kinetic_energy_per_atom():
    """msmgb_calekin (CALEKIN_DEV): 0.5 m v^2 per atom in caller order, -1e32 for inactive
    atoms and atoms with a fixed position component; after MD steps it follows the state."""
    pos, vel, L_ = lt.cu_config(6, 0.05, 600.0, 21)
    n = len(pos)
    ityp = np.ones(n, np.int32)
    ityp[::7] = 2
    statu = np.ones(n, np.int32)
    statu[5] = 0                                             # inactive
    statu[9] |= 4                                            # FIXPOSY
    masses = np.array([lt.CU_MASS, 2.0 * lt.CU_MASS])
    e = Engine(n, lt.CU_RC_NL, mxkvois=64)
    t = ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC)
    kp = np.array([[1, 1], [1, 1]], np.int32)
    e.init_forcetable_raw(L.FS_TYPE, t.ntab, 1, t.rmax, t.ru, t.potr, t.fpotr, t.potb, t.fpotb, 2, kp)
    e.set_masses(masses)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp, statu=statu)

    def expect(v):
        ek = 0.5 * masses[ityp - 1] * (v * v).sum(axis=1)
        ek[5] = ek[9] = -1.0e32
        return ek

    ek = e.get_ekin()
    np.testing.assert_allclose(ek, expect(vel), rtol=1e-15)
    e.run_steps(5, 1.0)
    _, v, _, _ = e.get_state()
    np.testing.assert_allclose(e.get_ekin(), expect(v), rtol=1e-15)
    e.close()
