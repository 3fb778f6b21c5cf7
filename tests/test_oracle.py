"""CPU tests of the oracle: pinned against the reference's exported force table, then
checked for the physical invariants the reference path must satisfy."""
import os

import numpy as np
import pytest

from msmpscu_gb300 import lattice as lt
from tests.helpers import cu_tables, w_tables, sorted_sets, CR_PRM

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ackland_ww_pair_rows.txt")


def test_table_generator_matches_reference_export(oracle):
    """EM_TB_WANGJUN_W-HE_2010.pair table #1 (Ackland-Thetford W-W), written by the
    reference's Export_ForceTable: r*V, -r dV/dr, RHO, -dRHO/dr on the sqrt(r) grid,
    printed with 10 significant digits."""
    d = np.loadtxt(GOLDEN)
    idx = d[:, 0].astype(int)
    t = oracle.make_tables(oracle.POT_ACKLAND_WW, None, 10.0, 10000, 10000, 20.0, want_embed=False)
    csiv = np.sqrt(10.0) / 10000
    mine = np.stack([(idx * csiv) ** 2, 2.0 * t["potr"][idx - 1], t["fpotr"][idx - 1],
                     t["potb"][idx - 1], t["fpotb"][idx - 1]], 1)
    ref = d[:, 1:]
    nz = ref != 0
    rel = np.abs(mine[nz] - ref[nz]) / np.abs(ref[nz])
    assert rel.max() < 6e-10
    assert np.all(np.abs(mine[~nz]) < 1e-300)


def test_cr_functions_closed_form(oracle):
    A, xi, p, q, r0 = CR_PRM
    for r in (2.2, 2.5563, 3.0, 4.77):
        potr, fpotr, potb, fpotb = oracle.pot_eval(oracle.POT_CR, CR_PRM, r)
        v = A * np.exp(-p * (r / r0 - 1))
        rho = xi * xi * np.exp(-2 * q * (r / r0 - 1))
        assert potr == pytest.approx(v, rel=1e-15)
        assert fpotr == pytest.approx(2 * v * p / r0, rel=1e-15)
        assert potb == pytest.approx(rho, rel=1e-15)
        assert fpotb == pytest.approx(2 * q / r0 * rho, rel=1e-15)


def _cu_small(seed=1, ncell=5, sigma=0.05):
    pos, vel, length = lt.cu_config(ncell, sigma, 300.0, seed)
    return pos, vel, length


def test_cell_list_equals_brute_force(oracle):
    pos, _, L = _cu_small()
    box = oracle.make_box([0, 0, 0], L)
    st = np.ones(len(pos), np.int32)
    k1, i1 = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    k2, i2 = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96, brute=True)
    assert sorted_sets(k1, i1) == sorted_sets(k2, i2)
    assert 40 <= k1.mean() <= 60


def test_small_box_minimum_image_list(oracle):
    """4-cell box: NCELL is forced to 3 with cells narrower than the cutoff (the reference's NCELL >= 3 rule);
    the minimum-image rule still finds every neighbour."""
    pos, _, L = lt.cu_config(4, 0.05, 300.0, 7)
    box = oracle.make_box([0, 0, 0], L)
    st = np.ones(len(pos), np.int32)
    k1, i1 = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    k2, i2 = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96, brute=True)
    assert sorted_sets(k1, i1) == sorted_sets(k2, i2)


def test_perfect_lattice_zero_force_and_cohesive_energy(oracle):
    pos, length = lt.fcc(5, 5, 5, lt.CU_A)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], length)
    st = np.ones(len(pos), np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    out = oracle.force(pos, np.ones(len(pos), np.int32), st, box, kv, ind, t)
    assert np.abs(out["f"]).max() < 1e-10
    e = out["epot"]
    assert np.ptp(e) < 1e-12
    # CR-Cu cohesive energy ~ -3.5 eV (Cleri & Rosato fit)
    assert -3.7 < e.mean() < -3.3


def test_momentum_conservation_and_energy_gradient(oracle):
    pos, _, L = _cu_small(seed=3)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L)
    n = len(pos)
    st, ty = np.ones(n, np.int32), np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    out = oracle.force(pos, ty, st, box, kv, ind, t)
    f = out["f"]
    assert np.abs(f.sum(0)).max() < 1e-10 * np.abs(f).max() * n
    # finite difference of the total energy (tables: agreement to interpolation error)
    rng = np.random.default_rng(0)
    for a in rng.choice(n, 3, replace=False):
        for k in range(3):
            h = 1e-5
            pp, pm = pos.copy(), pos.copy()
            pp[a, k] += h
            pm[a, k] -= h
            ep = oracle.force(pp, ty, st, box, kv, ind, t)["epot"].sum()
            em = oracle.force(pm, ty, st, box, kv, ind, t)["epot"].sum()
            assert -(ep - em) / (2 * h) == pytest.approx(f[a, k], abs=2e-3, rel=2e-3)


def test_virial_trace_matches_sum_r_dot_f(oracle):
    """For pair-decomposed forces the virial trace equals 1/2 sum_ij r_ij . f_ij."""
    pos, _, L = _cu_small(seed=5)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L)
    n = len(pos)
    st, ty = np.ones(n, np.int32), np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    out = oracle.force(pos, ty, st, box, kv, ind, t)
    vir = out["vir"]
    assert np.allclose(vir, vir.T)
    assert abs(np.trace(vir)) > 0


def test_atomic_stress_sums_to_virial_and_strain_derivative(oracle):
    """Per-atom tensors (pCalAVStress) are symmetric, sum to twice the box virial, and the
    virial is minus the derivative of the energy under a homogeneous strain of the box."""
    pos, _, L = _cu_small(seed=6)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L)
    n = len(pos)
    st, ty = np.ones(n, np.int32), np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    out = oracle.force(pos, ty, st, box, kv, ind, t)
    ap = oracle.atomic_stress(pos, ty, st, box, kv, ind, t, out["den"])
    assert np.allclose(ap, ap.transpose(0, 2, 1), rtol=0, atol=1e-12)
    assert np.allclose(ap.sum(0), 2.0 * out["vir"], rtol=1e-12, atol=1e-9)
    for a in (0, 2):
        e = []
        for sgn in (1.0, -1.0):
            scale = np.ones(3)
            scale[a] += sgn * 1e-6
            bx = oracle.make_box([0, 0, 0], L * scale)
            e.append(oracle.force(pos * scale, ty, st, bx, kv, ind, t)["epot"].sum())
        dE = (e[0] - e[1]) / 2e-6
        assert dE == pytest.approx(-out["vir"][a, a], rel=2e-3)


def test_eam_w_force_and_hvp_finite_difference(oracle):
    pos, L = lt.w_sia_config(4, 0.02, 11)
    t = w_tables(oracle)
    box = oracle.make_box([0, 0, 0], L)
    n = len(pos)
    st, ty = np.ones(n, np.int32), np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.W_RC_NL, 128)
    out = oracle.force(pos, ty, st, box, kv, ind, t)
    assert out["nbad"] == 0
    assert np.abs(out["f"].sum(0)).max() < 1e-9
    rng = np.random.default_rng(4)
    v = rng.normal(size=pos.shape)
    v /= np.linalg.norm(v)
    hv = oracle.hvp(pos, ty, st, box, kv, ind, t, v)
    eps = 1e-6
    fp = oracle.force(pos + eps * v, ty, st, box, kv, ind, t)["f"]
    fm = oracle.force(pos - eps * v, ty, st, box, kv, ind, t)["f"]
    fd = -(fp - fm) / (2 * eps)
    # table mode: knot crossings make FD differ from the exact interpolant derivative
    assert np.linalg.norm(fd - hv) / np.linalg.norm(hv) < 1e-3


def test_md_energy_conservation(oracle):
    pos, vel, L = lt.cu_config(5, 0.02, 300.0, 2)
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], L)
    n = len(pos)
    st, ty = np.ones(n, np.int32), np.ones(n, np.int32)
    cm = np.array([lt.CU_MASS])

    def etot(p, v):
        kv, ind = oracle.nlist(p, st, box, lt.CU_RC_NL, 96)
        e = oracle.force(p, ty, st, box, kv, ind, t)["epot"].sum()
        return e + 0.5 * lt.CU_MASS * (v * v).sum()

    e0 = etot(pos, vel)
    p1, v1, f1, st1, nreb = oracle.md(pos, vel, ty, st, box, t, cm, 1.0, 50, lt.CU_RC_NL,
                                      skin_trigger=0.15, mxkvois=96)
    e1 = etot(p1, v1)
    assert abs(e1 - e0) / n < 2e-4


def _loss(oracle, prm, pos, box, kv, ind, ft, rc=lt.CU_RC):
    tabs = oracle.make_tables(oracle.POT_CR, prm, rc, 10000, 10000, 20.0, want_embed=False)
    t = oracle.Tables(tabs, oracle.FS, rc)
    n = len(pos)
    f = oracle.force(pos, np.ones(n, np.int32), np.ones(n, np.int32), box, kv, ind, t,
                     want_virial=False, want_epot=False)["f"]
    return float(((f - ft) ** 2).sum())


def test_force_matching_gradient_vs_central_fd(oracle):
    """Oracle's forward-mode parameter gradient against central finite differences of the
    loss (relative step 1e-6) with targets from parameters scaled by +2%."""
    pos, _, L = lt.cu_config(5, 0.1, 300.0, 17)
    n = len(pos)
    box = oracle.make_box([0, 0, 0], L)
    st = np.ones(n, np.int32)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    prm = np.array(CR_PRM)
    tt = oracle.Tables(oracle.make_tables(oracle.POT_CR, prm * 1.02, lt.CU_RC, 10000, 10000, 20.0,
                                          want_embed=False), oracle.FS, lt.CU_RC)
    ft = oracle.force(pos, st, st, box, kv, ind, tt)["f"]
    t = oracle.Tables(oracle.make_tables(oracle.POT_CR, prm, lt.CU_RC, 10000, 10000, 20.0,
                                         want_embed=False), oracle.FS, lt.CU_RC)
    d = oracle.cr_dtables(prm, lt.CU_RC)
    loss, grad = oracle.adjoint_cr(pos, st, st, box, kv, ind, t, d, ft)
    assert loss == pytest.approx(_loss(oracle, prm, pos, box, kv, ind, ft), rel=1e-14)
    for m in range(5):
        h = 1e-6 * prm[m]
        pp, pm = prm.copy(), prm.copy()
        pp[m] += h
        pm[m] -= h
        fd = (_loss(oracle, pp, pos, box, kv, ind, ft) - _loss(oracle, pm, pos, box, kv, ind, ft)) / (2 * h)
        assert grad[m] == pytest.approx(fd, rel=1e-6), m


WANGJUN = os.path.join(os.path.dirname(__file__), "golden", "wangjun_pair_rows.txt")


@pytest.mark.parametrize("col,pot", [(0, "POT_HEHE_EXP6"), (1, "POT_HEW_ZBL"), (2, "POT_HEW_ZBL"),
                                     (3, "POT_DERLET_WW")])
def test_wangjun_library_tables_match_reference_export(oracle, col, pot):
    """Tables #2-#5 of EM_TB_WANGJUN_W-HE_2010.pair (He-He, He-W, W-He, Derlet W-W), with the
    rows around every piece boundary: the oracle's Angstrom/eV restatement and the library's
    CGS evaluation both reproduce the export's 10 printed digits (this also pins the
    single-precision literals of the reference source and its switch derivative)."""
    from msmpscu_gb300 import ForceTable, _lib as L
    d = np.loadtxt(WANGJUN)
    idx = d[:, 0].astype(int)
    ref = d[:, 2 + 4 * col:6 + 4 * col]
    t = oracle.make_tables(getattr(oracle, pot), None, 10.0, 10000, 10000, 20.0, want_embed=False)
    lib = ForceTable(getattr(L, pot), None, 10.0, 10.0, L.FS_TYPE)
    assert np.allclose((idx * np.sqrt(10.0) / 10000) ** 2, d[:, 1], rtol=1e-9)
    for src in ((t["potr"], t["fpotr"], t["potb"], t["fpotb"]), (lib.potr, lib.fpotr, lib.potb, lib.fpotb)):
        mine = np.stack([2.0 * src[0][idx - 1], src[1][idx - 1], src[2][idx - 1], src[3][idx - 1]], 1)
        nz = ref != 0
        assert (np.abs(mine[nz] - ref[nz]) / np.abs(ref[nz])).max() < 6e-10
        assert not mine[~nz].any()
