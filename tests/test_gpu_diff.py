"""GPU tests of the differentiation kernels at the benchmark sizes:
* bcc W 20^3 cells + one <111> dumbbell (16,001 atoms), Marinica EAM2: HVP against central
  finite differences of the device forces (delta = 1e-4 A, unit probes) at <= 1e-8, against
  the oracle's HVP at 1e-10, and the lowest curvature of 50 Lanczos iterations agreeing
  with a Lanczos run on the oracle's HVP;
* 64 Cu snapshots of 4,000 atoms (sigma 0.1 A): force-matching gradient w.r.t. the five
  Cleri-Rosato parameters (targets from parameters x 1.02) against central FD (relative
  step 1e-6) of the device FP64 loss;
and the torch.autograd harness around both."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from msmpscu_gb300 import _lib as L
from msmpscu_gb300.lanczos import lanczos_lowest, fd_hvp
from tests.helpers import cu_tables, w_tables, rel_err

pytestmark = pytest.mark.gpu


def _w_engine(n):
    e = Engine(n, lt.W_RC_NL, mxkvois=96)
    e.init_forcetable(ForceTable.marinica_eam2())
    return e


def test_c4_hvp_vs_fd_oracle_and_lanczos(oracle):
    pos, L_ = lt.w_sia_config(20, 0.0, 1)
    n = len(pos)
    assert n == 16001
    box = [(n, (0, 0, 0), tuple(L_), (1, 1, 1))]
    e = _w_engine(n)
    e.copyin(box, pos)

    def force(x):
        e.copyin(box, x)
        e.calforce()
        return e.get_force()

    def hvp(v):
        e.copyin(box, pos)
        return e.hvp(v)

    t = w_tables(oracle)
    ob = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, ob, lt.W_RC_NL, 128)
    rng = np.random.default_rng(2024)
    worst_fd = 0.0
    for _ in range(3):
        v = rng.normal(size=pos.shape)
        v /= np.linalg.norm(v)
        hv = hvp(v)
        ref = oracle.hvp(pos, st, st, ob, kv, ind, t, v)
        assert rel_err(hv, ref) < 1e-10
        fd = fd_hvp(force, pos, v, 1e-4)
        worst_fd = max(worst_fd, np.linalg.norm(fd - hv) / np.linalg.norm(hv))
    assert worst_fd < 1e-8, worst_fd

    lam, mode, ev, _ = lanczos_lowest(hvp, n, iters=50, seed=7)
    lam_o, _, _, _ = lanczos_lowest(lambda v: oracle.hvp(pos, st, st, ob, kv, ind, t, v), n,
                                    iters=50, seed=7)
    assert lam == pytest.approx(lam_o, rel=1e-8, abs=1e-10)
    # the Ritz pair is a curvature along the mode: v.Hv equals the Ritz value
    hm = hvp(mode)
    assert float((mode * hm).sum()) == pytest.approx(lam, rel=1e-6, abs=1e-8)
    ms_hvp, ms_force = e.time_hvp(mode, reps=10)
    assert ms_hvp > 0 and ms_force > 0
    e.close()


@pytest.mark.parametrize("system", ["w_250k", "cu_2048k"])
def test_hvp_large_systems_vs_oracle(oracle, system):
    """The HVP at the sizes where its pair buffer (40 B x MXKVOIS per atom slot, allocated on the
    first call) grows large: bcc W 50^3 cells + a <111> dumbbell (250,001 atoms, EAM) and fcc Cu
    80^3 cells (2,048,000 atoms, FS; 5.2 GB of pair buffer at MXKVOIS 64), against the oracle's
    HVP at 1e-10, and linear in the probe."""
    if system == "w_250k":
        pos, L_ = lt.w_sia_config(50, 0.02, 3)
        e = _w_engine(len(pos))
        t, rcnl, mxk = w_tables(oracle), lt.W_RC_NL, 128
    else:
        pos, _, L_ = lt.cu_config(80, 0.05, 600.0, 5)
        e = Engine(len(pos), lt.CU_RC_NL, mxkvois=64)
        e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
        t, rcnl, mxk = cu_tables(oracle), lt.CU_RC_NL, 96
    n = len(pos)
    e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos)
    ob = oracle.make_box([0, 0, 0], L_)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, ob, rcnl, mxk)
    rng = np.random.default_rng(11)
    v1 = rng.normal(size=pos.shape)
    v2 = rng.normal(size=pos.shape)
    h1 = e.hvp(v1)
    assert rel_err(h1, oracle.hvp(pos, st, st, ob, kv, ind, t, v1)) < 1e-10
    h2 = e.hvp(v2)
    h12 = e.hvp(v1 + 2.0 * v2)
    assert rel_err(h12, h1 + 2.0 * h2) < 1e-12
    e.close()


def test_c5_adjoint_64_snapshots_vs_fd():
    snaps = [lt.cu_config(10, 0.1, 300.0, 1000 + s) for s in range(64)]
    pos = np.vstack([s[0] for s in snaps])
    desc = [(len(s[0]), (0, 0, 0), tuple(s[2]), (1, 1, 1)) for s in snaps]
    prm = np.array([lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")])
    e = Engine(len(pos), lt.CU_RC_NL, max_boxes=64, mxkvois=64)
    e.init_forcetable(ForceTable(L.POT_CR, prm * 1.02, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
    e.copyin(desc, pos)
    e.calforce()
    ft = e.get_force()

    def loss(q):
        e.init_forcetable(ForceTable(L.POT_CR, q, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
        e.calforce()
        return float(((e.get_force() - ft) ** 2).sum())

    e.init_forcetable(ForceTable(L.POT_CR, prm, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
    l0, grad = e.param_adjoint(prm, ft)
    assert l0 == pytest.approx(loss(prm), rel=1e-12)
    for m in range(5):
        h = 1e-6 * prm[m]
        pp, pm = prm.copy(), prm.copy()
        pp[m] += h
        pm[m] -= h
        fd = (loss(pp) - loss(pm)) / (2 * h)
        assert grad[m] == pytest.approx(fd, rel=1e-6), (m, grad[m], fd)
    e.close()


def test_autograd_harness():
    torch = pytest.importorskip("torch")
    from msmpscu_gb300.autograd import EAMForce, ForceMatchLoss
    pos, L_ = lt.w_sia_config(4, 0.05, 5)
    n = len(pos)
    box = [(n, (0, 0, 0), tuple(L_), (1, 1, 1))]
    e = _w_engine(n)
    x = torch.tensor(pos, dtype=torch.float64, requires_grad=True)
    f = lambda xx: EAMForce.apply(xx, e, box)
    assert torch.autograd.gradcheck(f, (x,), eps=1e-6, atol=1e-5, rtol=1e-3, fast_mode=True)
    e.close()

    snaps = [lt.cu_config(6, 0.1, 300.0, 500 + s) for s in range(4)]
    p = np.vstack([s[0] for s in snaps])
    desc = [(len(s[0]), (0, 0, 0), tuple(s[2]), (1, 1, 1)) for s in snaps]
    prm = np.array([lt.CU_CR[k] for k in ("A", "xi", "p", "q", "r0")])
    e2 = Engine(len(p), lt.CU_RC_NL, max_boxes=4, mxkvois=64)
    e2.init_forcetable(ForceTable(L.POT_CR, prm * 1.02, lt.CU_RC, lt.CU_RC, L.FS_TYPE))
    e2.copyin(desc, p)
    e2.calforce()
    ft = e2.get_force()
    theta = torch.tensor(prm, dtype=torch.float64, requires_grad=True)
    g = lambda th: ForceMatchLoss.apply(th, e2, ft, lt.CU_RC)
    assert torch.autograd.gradcheck(g, (theta,), eps=1e-7, atol=1e-6, rtol=1e-5)
    e2.close()
