"""GPU parity tests: libmsmgb.so (through its C ABI) against the CPU oracle on the same seeded
inputs.  Neighbour lists must be identical per-atom index sets; FP64 forces, F'(rho),
energies and virial must agree within 1e-10 relative (max abs difference over the max
magnitude); trajectories within 1e-8 A."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt
from msmpscu_gb300 import _lib as L
from tests.helpers import cu_tables, w_tables, sorted_sets, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _cu_engine(n, nbox=1, precision="fp64", mxk=64, skin=0.15, nb_uptab=10):
    e = Engine(n, lt.CU_RC_NL, max_boxes=nbox, mxkvois=mxk, skin_trigger=skin,
               nb_uptab=nb_uptab, precision=precision)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


def _box(n, L_):
    return [(n, (0, 0, 0), tuple(L_), (1, 1, 1))]


def _oracle_force(oracle, pos, L_, tables, rc_nl=lt.CU_RC_NL, mxk=96, statu=None):
    n = len(pos)
    st = np.ones(n, np.int32) if statu is None else statu
    box = oracle.make_box([0, 0, 0], L_)
    kv, ind = oracle.nlist(pos, st, box, rc_nl, mxk)
    out = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, tables)
    return out, kv, ind


@pytest.mark.parametrize("ncell,sigma,seed", [(10, 0.02, 1), (6, 0.1, 2)])
def test_neighbour_sets_identical(oracle, ncell, sigma, seed):
    pos, vel, L_ = lt.cu_config(ncell, sigma, 300.0, seed)
    e = _cu_engine(len(pos))
    e.copyin(_box(len(pos), L_), pos, vel)
    e.cal_neighborelist()
    kv, ind = e.get_neighborelist()
    box = oracle.make_box([0, 0, 0], L_)
    okv, oind = oracle.nlist(pos, np.ones(len(pos), np.int32), box, lt.CU_RC_NL, 96)
    assert sorted_sets(kv, ind) == sorted_sets(okv, oind)
    # sorted order is a permutation and the device list maps back consistently
    gid = e.get_gid()
    assert sorted(gid.tolist()) == list(range(len(pos)))
    e.close()


def test_small_box_neighbours_complete(oracle):
    """edge 4 cells: NCELL forced to 3 (cells narrower than the cutoff, the reference's NCELL >= 3 rule)."""
    pos, vel, L_ = lt.cu_config(4, 0.05, 300.0, 9)
    e = _cu_engine(len(pos))
    e.copyin(_box(len(pos), L_), pos, vel)
    e.cal_neighborelist()
    kv, ind = e.get_neighborelist()
    box = oracle.make_box([0, 0, 0], L_)
    okv, oind = oracle.nlist(pos, np.ones(len(pos), np.int32), box, lt.CU_RC_NL, 96, brute=True)
    assert sorted_sets(kv, ind) == sorted_sets(okv, oind)
    e.close()


def test_fs_force_energy_virial_parity(oracle):
    pos, vel, L_ = lt.cu_config(10, 0.02, 300.0, 1)     # 4,000 atoms
    t = cu_tables(oracle)
    ref, _, _ = _oracle_force(oracle, pos, L_, t)
    e = _cu_engine(len(pos))
    e.copyin(_box(len(pos), L_), pos, vel)
    vir = e.calptensor()[0]
    f = e.get_force()
    assert rel_err(f, ref["f"]) < TOL
    assert rel_err(e.get_den(), ref["den"]) < TOL
    assert rel_err(vir, ref["vir"]) < TOL
    e.calepot()
    assert rel_err(e.get_epot(), ref["epot"]) < TOL
    e.calforce()
    assert rel_err(e.get_force(), ref["f"]) < TOL
    e.close()


@pytest.mark.parametrize("subtype", ["EAM2", "EAM3", "EAM4"])
def test_eam_force_parity_w_sia(oracle, subtype):
    pos, L_ = lt.w_sia_config(8, 0.02, 3)                # 1,025 atoms with a <111> dumbbell
    pot = {"EAM2": oracle.POT_MARINICA2, "EAM3": oracle.POT_MARINICA3, "EAM4": oracle.POT_MARINICA4}[subtype]
    t = oracle.Tables(oracle.make_tables(pot, None, lt.W_RC, 10000, 10000, 20.0, want_embed=True),
                      oracle.EAM, lt.W_RC)
    ref, _, _ = _oracle_force(oracle, pos, L_, t, rc_nl=lt.W_RC_NL, mxk=128)
    e = Engine(len(pos), lt.W_RC_NL, mxkvois=96)
    e.init_forcetable(ForceTable.marinica_eam2(subtype=subtype))
    e.copyin(_box(len(pos), L_), pos)
    vir = e.calptensor()[0]
    assert rel_err(e.get_force(), ref["f"]) < TOL
    assert rel_err(e.get_den(), ref["den"]) < TOL
    assert rel_err(vir, ref["vir"]) < TOL
    e.calepot()
    assert rel_err(e.get_epot(), ref["epot"]) < TOL
    e.close()


def test_inactive_atoms(oracle):
    pos, vel, L_ = lt.cu_config(6, 0.05, 300.0, 4)
    n = len(pos)
    st = np.ones(n, np.int32)
    st[::7] = 0                                          # deactivated (STATU bit 0 clear)
    t = cu_tables(oracle)
    ref, _, _ = _oracle_force(oracle, pos, L_, t, statu=st)
    e = _cu_engine(n)
    e.copyin(_box(n, L_), pos, vel, statu=st)
    e.calforce()
    f = e.get_force()
    assert np.all(f[::7] == 0.0)
    assert rel_err(f, ref["f"]) < TOL
    e.close()


def test_predictor_corrector_parity(oracle):
    pos, vel, L_ = lt.cu_config(6, 0.05, 600.0, 5)
    n = len(pos)
    t = cu_tables(oracle)
    ref, kv, ind = _oracle_force(oracle, pos, L_, t)
    e = _cu_engine(n)
    e.copyin(_box(n, L_), pos, vel)
    e.calforce()
    h = 1.0
    e.predictor(h)
    x = pos.copy(); v = vel.copy(); f = ref["f"]
    dis = np.zeros_like(x)
    st = np.ones(n, np.int32)
    box = oracle.make_box([0, 0, 0], L_)
    xs = [np.ascontiguousarray(x[:, k]) for k in range(3)]
    vs = [np.ascontiguousarray(v[:, k]) for k in range(3)]
    fs = [np.ascontiguousarray(f[:, k]) for k in range(3)]
    ds = [np.zeros(n) for _ in range(3)]
    d = oracle._d
    oracle.lib().orc_predictor(n, *[d(a) for a in xs], *[d(a) for a in vs], *[d(a) for a in fs],
                               *[d(a) for a in ds], oracle._i(st), oracle._i(np.ones(n, np.int32)),
                               d(np.array([lt.CU_MASS])), oracle.C.c_double(h), oracle.C.byref(box))
    gx, gv, gst, gdis = e.get_state()
    assert np.max(np.abs(gx - np.stack(xs, 1))) < 1e-12
    assert np.max(np.abs(gv - np.stack(vs, 1))) < 1e-14
    assert np.max(np.abs(gdis - np.stack(ds, 1))) < 1e-12
    e.close()


@pytest.mark.parametrize("precision_steps", [("fp64", 100)])
def test_md_trajectory_parity_cu4000(oracle, precision_steps):
    """Cu 4,000 atoms, 300 K, sigma 0.02 A, 100 NVE steps of 1 fs with the skin trigger."""
    prec, nsteps = precision_steps
    pos, vel, L_ = lt.cu_config(10, 0.02, 300.0, 1)
    n = len(pos)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L_)
    ox, ov, of, ost, oreb = oracle.md(pos, vel, np.ones(n, np.int32), np.ones(n, np.int32), box, t,
                                      np.array([lt.CU_MASS]), 1.0, nsteps, lt.CU_RC_NL,
                                      skin_trigger=0.15, mxkvois=96)
    e = _cu_engine(n, precision=prec)
    e.copyin(_box(n, L_), pos, vel)
    nreb = e.run_steps(nsteps, 1.0)
    gx, gv, gst, _ = e.get_state()
    dx = gx - ox
    dx -= np.round(dx / L_) * L_
    assert np.max(np.abs(dx)) < 1e-8
    assert np.max(np.abs(gv - ov)) < 1e-10
    assert rel_err(e.get_force(), of) < 1e-8
    assert nreb == oreb
    e.close()


def test_fixed_interval_rebuild(oracle):
    pos, vel, L_ = lt.cu_config(6, 0.02, 300.0, 12)
    n = len(pos)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L_)
    ox, ov, of, _, oreb = oracle.md(pos, vel, np.ones(n, np.int32), np.ones(n, np.int32), box, t,
                                    np.array([lt.CU_MASS]), 1.0, 30, lt.CU_RC_NL, skin_trigger=0.0,
                                    nb_uptab=10, mxkvois=96)
    e = _cu_engine(n, skin=0.0, nb_uptab=10)
    e.copyin(_box(n, L_), pos, vel)
    nreb = e.run_steps(30, 1.0)
    gx, gv, _, _ = e.get_state()
    dx = gx - ox
    dx -= np.round(dx / L_) * L_
    assert nreb == oreb == 3
    assert np.max(np.abs(dx)) < 1e-9
    e.close()


def test_batched_uneven_boxes_parity(oracle):
    boxes = lt.uneven_batch(6, seed=21, cmin=4, cmax=7)
    pos = np.vstack([b[0] for b in boxes])
    vel = np.vstack([b[1] for b in boxes])
    desc = [(len(b[0]), (0, 0, 0), tuple(b[2]), (1, 1, 1)) for b in boxes]
    e = _cu_engine(len(pos), nbox=len(boxes))
    e.copyin(desc, pos, vel)
    vir = e.calptensor()
    f = e.get_force()
    t = cu_tables(oracle)
    off = 0
    for k, (p, v, L_) in enumerate(boxes):
        ref, _, _ = _oracle_force(oracle, p, L_, t)
        sl = slice(off, off + len(p))
        assert rel_err(f[sl], ref["f"]) < TOL
        assert rel_err(vir[k], ref["vir"]) < TOL
        off += len(p)
    # batched MD == per-box MD
    e.run_steps(20, 1.0)
    gx, gv, _, _ = e.get_state()
    off = 0
    for k, (p, v, L_) in enumerate(boxes[:3]):
        box = oracle.make_box([0, 0, 0], L_)
        ox, ov, _, _, _ = oracle.md(p, v, np.ones(len(p), np.int32), np.ones(len(p), np.int32), box,
                                    t, np.array([lt.CU_MASS]), 1.0, 20, lt.CU_RC_NL, skin_trigger=0.15,
                                    mxkvois=96)
        dx = gx[off:off + len(p)] - ox
        dx -= np.round(dx / L_) * L_
        assert np.max(np.abs(dx)) < 1e-9
        off += len(p)
    e.close()


def test_hvp_parity_and_finite_difference(oracle):
    pos, L_ = lt.w_sia_config(6, 0.02, 8)
    n = len(pos)
    t = w_tables(oracle)
    box = oracle.make_box([0, 0, 0], L_)
    st, ty = np.ones(n, np.int32), np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.W_RC_NL, 128)
    rng = np.random.default_rng(3)
    v = rng.normal(size=pos.shape)
    v /= np.linalg.norm(v)
    ref = oracle.hvp(pos, ty, st, box, kv, ind, t, v)
    e = Engine(n, lt.W_RC_NL, mxkvois=96)
    e.init_forcetable(ForceTable.marinica_eam2())
    e.copyin(_box(n, L_), pos)
    hv = e.hvp(v)
    assert rel_err(hv, ref) < TOL
    eps = 1e-6
    e.copyin(_box(n, L_), pos + eps * v)
    e.calforce()
    fp = e.get_force()
    e.copyin(_box(n, L_), pos - eps * v)
    e.calforce()
    fm = e.get_force()
    fd = -(fp - fm) / (2 * eps)
    assert np.linalg.norm(fd - hv) / np.linalg.norm(hv) < 1e-3
    e.close()


@pytest.mark.parametrize("outer_skin", [0.0, 1.0])   # list overflow / candidate-list overflow
def test_neighbour_overflow_reported(outer_skin):
    pos, vel, L_ = lt.cu_config(6, 0.02, 300.0, 1)
    e = _cu_engine(len(pos), mxk=16)
    e.set_outer_skin(outer_skin)
    e.copyin(_box(len(pos), L_), pos, vel)
    with pytest.raises(MSMError) as ei:
        e.cal_neighborelist()
    assert ei.value.code == L.ERR_NL_OVERFLOW
    e.close()


def test_atom_out_of_box_reported():
    pos, vel, L_ = lt.cu_config(6, 0.02, 300.0, 1)
    pos = pos.copy()
    pos[5, 0] = -0.6 * L_[0]
    e = _cu_engine(len(pos))
    e.copyin(_box(len(pos), L_), pos, vel)
    with pytest.raises(MSMError) as ei:
        e.cal_neighborelist()
    assert ei.value.code == L.ERR_OUT_OF_BOX
    e.close()


def test_box_too_small_rejected():
    pos, vel, L_ = lt.cu_config(2, 0.0, 0.0, 1)
    e = _cu_engine(len(pos))
    with pytest.raises(MSMError) as ei:
        e.copyin(_box(len(pos), L_), pos, vel)
    assert ei.value.code == L.ERR_BOX_TOO_SMALL
    e.close()


def test_full_size_c2_fp64_properties_and_sample_parity(oracle):
    """2,048,000-atom Cu (80^3 cells, sigma 0.05 A): momentum conservation of the whole
    force field and oracle parity on the full list (OpenMP oracle)."""
    pos, vel, L_ = lt.cu_config(80, 0.05, 600.0, 2024)
    n = len(pos)
    e = _cu_engine(n)
    e.copyin(_box(n, L_), pos, vel)
    e.calforce()
    f = e.get_force()
    assert np.abs(f.sum(0)).max() < 1e-9 * np.sqrt(n) * np.abs(f).max()
    t = cu_tables(oracle)
    ref, okv, oind = _oracle_force(oracle, pos, L_, t, mxk=80)
    assert rel_err(f, ref["f"]) < TOL
    kv, ind = e.get_neighborelist()
    assert np.array_equal(np.sort(kv), np.sort(okv))
    rng = np.random.default_rng(0)
    for i in rng.choice(n, 2000, replace=False):
        assert sorted(ind[:kv[i], i].tolist()) == sorted(oind[:okv[i], i].tolist())
    e.close()


# ---- mixed precision ------------------------------------------------------------------------

def _force_err(f, ref):
    return (np.linalg.norm(f - ref) / np.linalg.norm(ref), np.abs(f - ref).max() / np.abs(ref).max())


def test_full_size_c2_mixed_md_properties_and_parity(oracle):
    """2,048,000-atom Cu in mixed precision with the autotuned kernels (the fixed-point force
    records, the two-level list): after 60 MD steps with list rebuilds inside the step graph,
    the forces at the final positions against the FP64 oracle's (norm and max below 1e-6),
    momentum conservation of the force field, and the neighbour sets of a sample of atoms
    after a full list build at those positions."""
    pos, vel, L_ = lt.cu_config(80, 0.05, 600.0, 7)
    n = len(pos)
    e = _cu_engine(n, precision="mixed")
    e.set_masses([lt.CU_MASS])
    e.copyin(_box(n, L_), pos, vel)
    reb = e.run_steps(60, 1.0)
    assert reb > 0
    x = e.get_state()[0]
    f = e.get_force()
    assert np.abs(f.sum(0)).max() < 1e-6 * np.sqrt(n) * np.abs(f).max()
    t = cu_tables(oracle)
    ref, okv, oind = _oracle_force(oracle, x, L_, t, mxk=80)
    nrm, mx = _force_err(f, ref["f"])
    assert nrm < 1e-6 and mx < 1e-6, (nrm, mx)
    e.cal_neighborelist()            # a full build at the final positions
    kv, ind = e.get_neighborelist()
    rng = np.random.default_rng(1)
    for i in rng.choice(n, 2000, replace=False):
        assert sorted(ind[:kv[i], i].tolist()) == sorted(oind[:okv[i], i].tolist())
    e.close()


@pytest.mark.parametrize("ncell,sigma,seed", [(10, 0.05, 2024), (8, 0.1, 5)])
def test_mixed_force_error_below_1e6(oracle, ncell, sigma, seed):
    """FP32 pair/density/table terms: force error against the FP64 oracle (norm-wise and
    max-abs, both relative) below 1e-6."""
    pos, vel, L_ = lt.cu_config(ncell, sigma, 600.0, seed)
    t = cu_tables(oracle)
    ref, _, _ = _oracle_force(oracle, pos, L_, t)
    e = _cu_engine(len(pos), precision="mixed")
    e.copyin(_box(len(pos), L_), pos, vel)
    e.calforce()
    nrm, mx = _force_err(e.get_force(), ref["f"])
    assert nrm < 1e-6 and mx < 1e-6, (nrm, mx)
    assert rel_err(e.get_den(), ref["den"]) < 1e-6
    # FP64 virial / energy requests still run the FP64 passes
    vir = e.calptensor()[0]
    assert rel_err(vir, ref["vir"]) < TOL
    e.close()


def test_mixed_md_tracks_fp64(oracle):
    pos, vel, L_ = lt.cu_config(8, 0.05, 600.0, 6)
    n = len(pos)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L_)
    ox, ov, of, _, _ = oracle.md(pos, vel, np.ones(n, np.int32), np.ones(n, np.int32), box, t,
                                 np.array([lt.CU_MASS]), 1.0, 50, lt.CU_RC_NL, skin_trigger=0.15,
                                 mxkvois=96)
    e = _cu_engine(n, precision="mixed")
    e.copyin(_box(n, L_), pos, vel)
    e.run_steps(50, 1.0)
    gx, gv, _, _ = e.get_state()
    dx = gx - ox
    dx -= np.round(dx / L_) * L_
    assert np.max(np.abs(dx)) < 1e-6
    nrm, mx = _force_err(e.get_force(), of)
    assert nrm < 2e-6
    e.close()


def test_mixed_eam_force_error(oracle):
    pos, L_ = lt.w_sia_config(8, 0.03, 13)
    t = w_tables(oracle)
    ref, _, _ = _oracle_force(oracle, pos, L_, t, rc_nl=lt.W_RC_NL, mxk=128)
    e = Engine(len(pos), lt.W_RC_NL, mxkvois=96, precision="mixed")
    e.init_forcetable(ForceTable.marinica_eam2())
    e.copyin(_box(len(pos), L_), pos)
    e.calforce()
    nrm, mx = _force_err(e.get_force(), ref["f"])
    assert nrm < 1e-6 and mx < 2e-6, (nrm, mx)
    e.close()


def test_mixed_batched_boxes(oracle):
    boxes = lt.uneven_batch(5, seed=33, cmin=4, cmax=6)
    pos = np.vstack([b[0] for b in boxes])
    vel = np.vstack([b[1] for b in boxes])
    desc = [(len(b[0]), (0, 0, 0), tuple(b[2]), (1, 1, 1)) for b in boxes]
    e = _cu_engine(len(pos), nbox=len(boxes), precision="mixed")
    e.copyin(desc, pos, vel)
    e.calforce()
    f = e.get_force()
    t = cu_tables(oracle)
    off = 0
    for p, v, L_ in boxes:
        ref, _, _ = _oracle_force(oracle, p, L_, t)
        nrm, mx = _force_err(f[off:off + len(p)], ref["f"])
        assert nrm < 1e-6 and mx < 1e-6
        off += len(p)
    e.close()


# ---- parameter adjoint ------------------------------------------------------------------

def test_param_adjoint_parity_and_fd(oracle):
    """Force-matching gradient w.r.t. (A, xi, p, q, r0): device adjoint vs the oracle's
    forward-mode gradient (1e-10) and vs central FD of the device FP64 loss (step 1e-6)."""
    boxes = [lt.cu_config(6, 0.1, 300.0, s) for s in (41, 42, 43)]
    pos = np.vstack([b[0] for b in boxes])
    desc = [(len(b[0]), (0, 0, 0), tuple(b[2]), (1, 1, 1)) for b in boxes]
    prm = np.array([lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")])
    e = Engine(len(pos), lt.CU_RC_NL, max_boxes=len(boxes), mxkvois=64)
    e.init_forcetable(ForceTable(L.POT_CR, prm * 1.02, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
    e.copyin(desc, pos)
    e.calforce()
    ft = e.get_force()
    e.init_forcetable(ForceTable(L.POT_CR, prm, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
    loss, grad = e.param_adjoint(prm, ft)
    # oracle, box by box
    og = np.zeros(5)
    ol = 0.0
    off = 0
    t = oracle.Tables(oracle.make_tables(oracle.POT_CR, prm, lt.CU_RC, 10000, 10000, 20.0,
                                         want_embed=False), oracle.FS, lt.CU_RC)
    d = oracle.cr_dtables(prm, lt.CU_RC)
    for p, _, L_ in boxes:
        n = len(p)
        box = oracle.make_box([0, 0, 0], L_)
        st = np.ones(n, np.int32)
        kv, ind = oracle.nlist(p, st, box, lt.CU_RC_NL, 96)
        l, g = oracle.adjoint_cr(p, st, st, box, kv, ind, t, d, ft[off:off + n])
        ol += l
        og += g
        off += n
    assert loss == pytest.approx(ol, rel=1e-10)
    assert rel_err(grad, og) < 1e-10

    def dev_loss(q):
        e.init_forcetable(ForceTable(L.POT_CR, q, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
        e.calforce()
        return float(((e.get_force() - ft) ** 2).sum())

    for m in range(5):
        h = 1e-6 * prm[m]
        pp, pm = prm.copy(), prm.copy()
        pp[m] += h
        pm[m] -= h
        fd = (dev_loss(pp) - dev_loss(pm)) / (2 * h)
        assert grad[m] == pytest.approx(fd, rel=1e-6), (m, grad[m], fd)
    e.close()
