"""Two-level neighbour list: a full rebuild keeps the candidates within rc_nl + outer skin and
later rebuilds inside MD steps re-select the list from them.  The re-selected lists against the
oracle's lists at the same positions (identical sets, MD_NeighborsList.F90:396-633 semantics),
full rebuilds once the displacement bound passes half the outer skin, atoms leaving an open
face, and two-level MD against single-level MD."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from helpers import sorted_sets

pytestmark = pytest.mark.gpu


def _engine(n, prec, outer_skin, nbox=1, skin=0.0, nb_uptab=5, mxk=96):
    e = Engine(n, lt.CU_RC_NL, max_boxes=nbox, mxkvois=mxk, skin_trigger=skin, nb_uptab=nb_uptab,
               precision=prec, outer_skin=outer_skin)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


@pytest.mark.parametrize("prec", ["fp64", "mixed", "ff"])
def test_reselected_lists_equal_oracle(oracle, prec):
    # a rebuild every 5 steps (fixed interval): after run_steps(5) the list belongs to the
    # current positions; the hot lattice makes some rebuilds full and the others re-selections
    pos, vel, L_ = lt.cu_config(8, 0.05, 1500.0, 4)
    n = len(pos)
    e = _engine(n, prec, 0.6)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    box = oracle.make_box([0, 0, 0], L_)
    for _ in range(8):
        e.run_steps(5, 1.0)
        kv, ind = e.get_neighborelist()
        x = e.get_state()[0]
        okv, oind = oracle.nlist(x, np.ones(n, np.int32), box, lt.CU_RC_NL, 96)
        assert sorted_sets(kv, ind) == sorted_sets(okv, oind)
    reb, full = e.rebuild_counts()
    e.close()
    assert reb == 8 and 0 < full < 8


def test_reselection_small_box_and_open_face(oracle):
    # 4-cell box (cells forced to 3 per edge, minimum image) with an open z face that atoms leave
    rng = np.random.default_rng(3)
    p, L_ = lt.fcc(4, 4, 4, lt.CU_A)
    p = lt.displace(p, 0.05, rng, np.zeros(3), L_)
    p[:, 2] = np.clip(p[:, 2], 0.05, L_[2] - 0.05)
    n = len(p)
    v = lt.velocities(n, lt.CU_MASS, 1500.0, rng)
    v[:8, 2] = np.where(p[:8, 2] > L_[2] / 2, 0.05, -0.05)   # fast atoms toward the open faces
    e = _engine(n, "fp64", 0.8)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 0))], p, v)
    box = oracle.make_box([0, 0, 0], L_, ifpd=(1, 1, 0))
    for _ in range(6):
        e.run_steps(5, 1.0)
        kv, ind = e.get_neighborelist()
        x, _, st, _ = e.get_state()
        okv, oind = oracle.nlist(x, st, box, lt.CU_RC_NL, 96, brute=True)
        assert sorted_sets(kv, ind) == sorted_sets(okv, oind)
    e.close()


def test_two_level_md_matches_single_level():
    # same trajectory (FP64; only the summation order of a few lists differs) with the skin trigger
    pos, vel, L_ = lt.cu_config(10, 0.05, 900.0, 8)
    n = len(pos)
    out = []
    for skin in (0.0, 1.0):
        e = _engine(n, "fp64", skin, skin=0.15, nb_uptab=10)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        nr = e.run_steps(60, 1.0)
        x, v, _, _ = e.get_state()
        out.append((x, v, e.get_force(), nr, e.rebuild_counts()))
        e.close()
    (x0, v0, f0, n0, c0), (x1, v1, f1, n1, c1) = out
    assert n0 == n1 and n0 > 1
    assert c0 == (n0, n0) and c1[0] == n1 and c1[1] < n1
    assert np.abs(x0 - x1).max() < 1e-9 and np.abs(v0 - v1).max() < 1e-12
    assert np.abs(f0 - f1).max() < 1e-8 * np.abs(f0).max()


def test_batched_boxes_reselection(oracle):
    boxes, P, V = [], [], []
    rng = np.random.default_rng(12)
    for nc in (4, 7, 5, 9):
        p, L_ = lt.fcc(nc, nc, nc, lt.CU_A)
        P.append(lt.displace(p, 0.05, rng, np.zeros(3), L_))
        V.append(lt.velocities(len(p), lt.CU_MASS, 1200.0, rng))
        boxes.append((len(p), (0, 0, 0), tuple(L_), (1, 1, 1)))
    pos, vel = np.vstack(P), np.vstack(V)
    n = len(pos)
    e = _engine(n, "mixed", 0.6, nbox=len(boxes))
    e.copyin(boxes, pos, vel)
    for _ in range(5):
        e.run_steps(5, 1.0)
    kv, ind = e.get_neighborelist()
    x = e.get_state()[0]
    off = 0
    got = sorted_sets(kv, ind)
    for (na, _, L_, _) in boxes:
        box = oracle.make_box([0, 0, 0], L_)
        okv, oind = oracle.nlist(x[off:off + na], np.ones(na, np.int32), box, lt.CU_RC_NL, 96)
        want = [tuple(j + off for j in s) for s in sorted_sets(okv, oind)]
        assert got[off:off + na] == want
        off += na
    reb, full = e.rebuild_counts()
    e.close()
    assert reb == 5 and full < 5


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_new_state_of_same_layout_reuses_step_graphs(prec):
    # a second copy-in of the same atom count and boxes keeps the captured step graphs; the
    # trajectory equals that of a fresh context
    p1, v1, L_ = lt.cu_config(12, 0.05, 900.0, 31)
    p2, v2, _ = lt.cu_config(12, 0.08, 1200.0, 32)
    n = len(p1)
    box = [(n, (0, 0, 0), tuple(L_), (1, 1, 1))]
    # mixed: the same kernel variants in both contexts (two autotuner runs may pick variants
    # with other record formats, whose arithmetic differs)
    pin = dict(density=275, force=128 + 50, fused=128 + 32 + 15) if prec == "mixed" else None
    a = _engine(n, prec, 1.0, skin=0.15, nb_uptab=10)
    a.copyin(box, p1, v1)
    if pin:
        a.set_tuning(**pin)
    a.run_steps(30, 1.0)
    a.copyin(box, p2, v2)
    ra = a.run_steps(30, 1.0)
    xa, va, _, _ = a.get_state()
    fa = a.get_force()
    a.close()
    b = _engine(n, prec, 1.0, skin=0.15, nb_uptab=10)
    b.copyin(box, p2, v2)
    if pin:
        b.set_tuning(**pin)
    rb = b.run_steps(30, 1.0)
    xb, vb, _, _ = b.get_state()
    fb = b.get_force()
    b.close()
    assert ra == rb and ra > 0
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa, fb)


def test_candidate_buffer_grows_for_a_dense_cluster(oracle):
    # a bulk-density cluster in a box of 64x its volume: the candidate buffer sized from the
    # box's mean density is too small at the first full build, is grown and the build redone
    rng = np.random.default_rng(41)
    p, Lc = lt.fcc(6, 6, 6, lt.CU_A)
    L_ = 4.0 * Lc
    pos = p + 1.5 * Lc + rng.normal(0.0, 0.03, p.shape)
    n = len(pos)
    vel = lt.velocities(n, lt.CU_MASS, 300.0, rng)
    e = _engine(n, "mixed", 1.0, skin=0.15, nb_uptab=10)
    e.copyin([(n, (0, 0, 0), tuple(L_), (0, 0, 0))], pos, vel)
    e.cal_neighborelist()
    kv, ind = e.get_neighborelist()
    box = oracle.make_box([0, 0, 0], L_, ifpd=(0, 0, 0))
    okv, oind = oracle.nlist(pos, np.ones(n, np.int32), box, lt.CU_RC_NL, 96)
    assert sorted_sets(kv, ind) == sorted_sets(okv, oind)
    e.run_steps(40, 1.0)
    kv, ind = e.get_neighborelist()
    assert kv.max() > 40
    e.close()


def test_reselection_bcc_w_eam(oracle):
    # bcc W with a <111> dumbbell (Marinica EAM2, rc_nl = 5.76 A): re-selected lists equal the
    # oracle's, FP64 forces at 1e-10 after the steps
    from helpers import rel_err, w_tables
    pos, L_ = lt.w_sia_config(8, 0.03, 5)
    n = len(pos)
    vel = lt.velocities(n, lt.W_MASS, 1500.0, np.random.default_rng(6))
    e = Engine(n, lt.W_RC_NL, mxkvois=128, skin_trigger=0.0, nb_uptab=5, outer_skin=0.8)
    e.init_forcetable(ForceTable.marinica_eam2(rc=lt.W_RC))
    e.set_masses([lt.W_MASS])
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    box = oracle.make_box([0, 0, 0], L_)
    t = w_tables(oracle)
    st = np.ones(n, np.int32)
    for _ in range(6):
        e.run_steps(5, 1.0)
        kv, ind = e.get_neighborelist()
        x = e.get_state()[0]
        okv, oind = oracle.nlist(x, st, box, lt.W_RC_NL, 128)
        assert sorted_sets(kv, ind) == sorted_sets(okv, oind)
    reb, full = e.rebuild_counts()
    assert reb == 6 and full < 6
    e.calforce()
    ref = oracle.force(x, np.ones(n, np.int32), st, box, okv, oind, t)
    assert rel_err(e.get_force(), ref["f"]) < 1e-10
    e.close()


@pytest.mark.parametrize("u256,u128", [(0, 32), (3, 35)])
def test_two_species_fused_128_thread_blocks(oracle, u256, u128):
    # several table kinds: the fused step kernel's 128-thread variants against the 256-thread
    # ones (bitwise), with the two-level list
    from test_gpu_edges import _two_species_tables
    from msmpscu_gb300 import _lib as L
    pos, vel, L_ = lt.cu_config(9, 0.05, 900.0, 44)
    n = len(pos)
    ityp = (np.random.default_rng(2).random(n) < 0.35).astype(np.int32) + 1
    arr, kpair = _two_species_tables(oracle)
    out = []
    for code in (u256, u128):
        e = Engine(n, lt.CU_RC_NL, mxkvois=80, precision="mixed")
        e.init_forcetable_raw(L.FS_TYPE, 10000, 4, lt.CU_RC, lt.CU_RC, arr["potr"], arr["fpotr"],
                              arr["potb"], arr["fpotb"], 2, kpair)
        e.set_masses([lt.CU_MASS, 1.3 * lt.CU_MASS])
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel, ityp=ityp)
        e.set_tuning(density=3, force=3, fused=code)
        e.run_steps(25, 1.0)
        x, v, _, _ = e.get_state()
        out.append((x, v, e.get_force()))
        e.close()
    assert all(np.array_equal(a, b) for a, b in zip(out[0], out[1]))


def test_pairs_at_the_cutoff_decided_by_the_fp64_rule(oracle):
    """Pairs placed at rc_nl itself and one or a few FP64 ulps either side: the re-selection's
    float-float distance cannot separate them from rc_nl, so they fall through to the exact
    FP64 rule, and the sets equal the oracle's (d^2 < rc^2 in FP64)."""
    rng = np.random.default_rng(17)
    p, L_ = lt.fcc(8, 8, 8, lt.CU_A)
    p = lt.displace(p, 0.05, rng, np.zeros(3), L_)
    n = len(p)
    rc = lt.CU_RC_NL
    # move atom b of some pairs so that |x_a - x_b| is rc (and rc +- k ulp) along a random direction
    picks = rng.choice(n, 40, replace=False)
    for m in range(0, 40, 2):
        a_, b_ = picks[m], picks[m + 1]
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        r = np.nextafter(rc, np.inf if m % 4 == 0 else -np.inf) if m % 8 else rc
        p[b_] = (p[a_] + r * d) % L_
    for prec in ("fp64", "mixed"):
        e = _engine(n, prec, 1.0)
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], p)
        e.calforce()
        kv, ind = e.get_neighborelist()
        x = e.get_state()[0]
        okv, oind = oracle.nlist(x, np.ones(n, np.int32), oracle.make_box([0, 0, 0], L_), rc, 96)
        assert sorted_sets(kv, ind) == sorted_sets(okv, oind), prec
        e.close()
