"""Consumers of the device force and HVP calls: an L-BFGS quench and a min-mode-following
saddle search (Lanczos lowest mode of the HVP), on the nearest-neighbour vacancy jump in fcc
Cu (Cleri-Rosato).  The jump is symmetric under a two-fold rotation about the midpoint of the
two sites, so the saddle must put the jumping atom on that midpoint."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt
from msmpscu_gb300.relax import energy, lbfgs_quench, saddle_search
from tests.helpers import cu_tables

pytestmark = pytest.mark.gpu


def _vacancy_box():
    pos, L = lt.fcc(5, 5, 5, lt.CU_A)
    a = 0                                         # vacancy site
    d = pos - pos[a]
    d -= np.round(d / L) * L
    r = np.sqrt((d * d).sum(axis=1))
    r[a] = np.inf
    b = int(np.argmin(r))                         # a nearest neighbour jumps into it
    keep = np.ones(len(pos), bool)
    keep[a] = False
    site_a, site_b = pos[a].copy(), pos[b].copy()
    ib = int(np.nonzero(keep)[0].tolist().index(b))
    return pos[keep], L, site_a, site_b, ib


def test_quench_and_vacancy_migration_saddle(oracle):
    pos, L, site_a, site_b, ib = _vacancy_box()
    n = len(pos)
    e = Engine(n, lt.CU_RC_NL, mxkvois=96, precision="fp64")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    rng = np.random.default_rng(1)
    e.copyin([(n, (0, 0, 0), tuple(L), (1, 1, 1))], pos + rng.normal(scale=0.02, size=pos.shape))
    x_min, f_min, it = lbfgs_quench(e, pos + rng.normal(scale=0.02, size=pos.shape), fmax=1e-4)
    assert np.abs(f_min).max() < 1e-4 and it < 2000
    # the oracle agrees that the quenched state is a minimum
    box = oracle.make_box([0, 0, 0], L)
    st = np.ones(n, np.int32)
    xw = x_min - np.floor(x_min / L) * L
    kv, ind = oracle.nlist(xw, st, box, lt.CU_RC_NL, 128)
    assert np.abs(oracle.force(xw, st, st, box, kv, ind, cu_tables(oracle))["f"]).max() < 1e-4
    e_min = energy(e, x_min)
    # start 45 % along the jump and search the saddle
    jump = site_a - site_b
    jump -= np.round(jump / L) * L
    x0 = x_min.copy()
    x0[ib] = site_b + 0.45 * jump
    xs, fs, lam, mode, its = saddle_search(e, x0, fmax=1e-3)
    assert np.abs(fs).max() < 1e-3, (np.abs(fs).max(), its)
    assert lam < 0.0
    mid = site_b + 0.5 * jump
    dmid = xs[ib] - mid
    dmid -= np.round(dmid / L) * L
    assert np.sqrt((dmid * dmid).sum()) < 0.02, dmid
    barrier = energy(e, xs) - e_min
    assert 0.2 < barrier < 2.0, barrier
    # the unstable mode is dominated by the jumping atom, along the jump
    assert abs(float(mode[ib] @ (jump / np.linalg.norm(jump)))) > 0.5
    e.close()


def test_quench_and_saddle_resident_on_device(oracle):
    """The same vacancy quench and saddle search with every vector on the GPU (positions,
    forces and HVPs passed to the library by device pointer): same saddle, same barrier."""
    import torch
    pos, L, site_a, site_b, ib = _vacancy_box()
    n = len(pos)
    e = Engine(n, lt.CU_RC_NL, mxkvois=96, precision="fp64")
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    rng = np.random.default_rng(1)
    start = pos + rng.normal(scale=0.02, size=pos.shape)
    e.copyin([(n, (0, 0, 0), tuple(L), (1, 1, 1))], start)
    x0 = torch.tensor(start.T.copy(), device="cuda")
    x_min, f_min, it = lbfgs_quench(e, x0, fmax=1e-4)
    assert x_min.is_cuda and f_min.is_cuda and float(f_min.abs().max()) < 1e-4
    xm = x_min.T.cpu().numpy()
    e_min = energy(e, xm)
    jump = site_a - site_b
    jump -= np.round(jump / L) * L
    xs0 = xm.copy()
    xs0[ib] = site_b + 0.45 * jump
    xs, fs, lam, mode, its = saddle_search(e, xs0, fmax=1e-3, device="cuda")
    assert np.abs(fs).max() < 1e-3 and lam < 0.0
    dmid = xs[ib] - (site_b + 0.5 * jump)
    dmid -= np.round(dmid / L) * L
    assert np.sqrt((dmid * dmid).sum()) < 0.02
    barrier = energy(e, xs) - e_min
    assert 0.2 < barrier < 2.0
    # the host-driven search of the same start reaches the same barrier
    xh, fh, lamh, _, _ = saddle_search(e, xs0, fmax=1e-3)
    assert abs((energy(e, xh) - e_min) - barrier) < 1e-3
    e.close()
