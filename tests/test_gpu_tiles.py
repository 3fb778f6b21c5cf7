"""Cell-tile variants of the mixed passes (each block's halo of cells staged in shared memory,
neighbours read through their halo position) against the variants that gather neighbours from
global memory with the same arithmetic in the same order: identical densities, forces and
trajectories, across list rebuilds, several boxes, non-periodic faces, narrow boxes and blocks
that fall back to global gathers."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, MSMError, lattice as lt

pytestmark = pytest.mark.gpu

# (density, fused) variant pairs: global gathers / cell tiles with the same neighbours in flight
GLOBAL_TILE = [((19, 12), (66, 20)), ((21, 13), (68, 21)), ((19, 12), (82, 22)), ((21, 13), (84, 23))]


def _engine(n, nbox=1, prec="mixed"):
    # cells sized by rc_nl (single-level list): the halos of 256 atoms fit the tile capacity
    e = Engine(n, lt.CU_RC_NL, mxkvois=80, max_boxes=nbox, precision=prec, outer_skin=0.0)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    return e


def _run(boxes, pos, vel, dens, fused, steps):
    e = _engine(len(pos), len(boxes))
    e.copyin(boxes, pos, vel)
    e.set_tuning(density=dens, force=20, fused=fused)
    e.calforce()
    f0 = e.get_force()
    stats = e.tile_stats()
    stats["rebuilds"] = e.run_steps(steps, 1.0)
    x, v, _, _ = e.get_state()
    f = e.get_force()
    t = e.tuning()
    assert (t["density_variant"], t["fused_variant"]) == (dens, fused)
    e.close()
    return f0, x, v, f, stats


@pytest.mark.parametrize("ncell", [7, 30])          # 1,372 atoms (a partial last block), 108,000
@pytest.mark.parametrize("glob,tile", GLOBAL_TILE)
def test_tiles_match_global_gathers(ncell, glob, tile):
    pos, vel, L_ = lt.cu_config(ncell, 0.08, 1500.0, 11)
    boxes = [(len(pos), (0, 0, 0), tuple(L_), (1, 1, 1))]
    fa, xa, va, fa2, _ = _run(boxes, pos, vel, *glob, steps=40)
    fb, xb, vb, fb2, st = _run(boxes, pos, vel, *tile, steps=40)
    assert np.array_equal(fa, fb)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa2, fb2)
    assert st["rebuilds"] > 0
    if ncell >= 30:
        assert st["tiled"] == st["blocks"] and 0 < st["mean_halo"] <= 2048


def test_tiles_several_boxes_and_open_faces():
    rng = np.random.default_rng(5)
    boxes, P, V = [], [], []
    for k, (nc, pd) in enumerate([(5, (1, 1, 1)), (9, (1, 1, 0)), (4, (1, 1, 1)), (11, (0, 1, 1)), (6, (1, 1, 1))]):
        p, L_ = lt.fcc(nc, nc, nc, lt.CU_A)
        p = lt.displace(p, 0.05, rng, np.zeros(3), L_)
        if not all(pd):                      # keep atoms off the open faces
            for d in range(3):
                if not pd[d]:
                    p[:, d] = np.clip(p[:, d], 0.01, L_[d] - 0.01)
        P.append(p)
        V.append(lt.velocities(len(p), lt.CU_MASS, 900.0, rng))
        boxes.append((len(p), (0, 0, 0), tuple(L_), pd))
    pos, vel = np.vstack(P), np.vstack(V)
    fa, xa, va, fa2, _ = _run(boxes, pos, vel, 19, 12, steps=30)
    fb, xb, vb, fb2, st = _run(boxes, pos, vel, 66, 20, steps=30)
    assert np.array_equal(fa, fb)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa2, fb2)
    assert st["tiled"] > 0


def test_sparse_blocks_fall_back_to_global_gathers():
    # a lattice with 80 % of its sites empty: 256 sorted atoms span more cells than a tile
    # holds, so those blocks gather from global memory; the results stay those of the
    # global variants
    rng = np.random.default_rng(9)
    p, L_ = lt.fcc(12, 12, 12, lt.CU_A)
    keep = rng.random(len(p)) < 0.2
    pos = lt.displace(p[keep], 0.05, rng, np.zeros(3), L_)
    n = len(pos)
    vel = lt.velocities(n, lt.CU_MASS, 300.0, rng)
    boxes = [(n, (0, 0, 0), tuple(L_), (1, 1, 1))]
    fa, xa, va, fa2, _ = _run(boxes, pos, vel, 19, 12, steps=5)
    fb, xb, vb, fb2, st = _run(boxes, pos, vel, 66, 20, steps=5)
    assert st["tiled"] < st["blocks"]
    assert np.array_equal(fa, fb) and np.array_equal(xa, xb) and np.array_equal(fa2, fb2)


def test_tiles_mixed_force_matches_fp64_oracle_scale():
    # the tile path's forces against the FP64 passes: the mixed-precision error bound
    pos, vel, L_ = lt.cu_config(12, 0.05, 600.0, 21)
    n = len(pos)
    boxes = [(n, (0, 0, 0), tuple(L_), (1, 1, 1))]
    e = _engine(n, prec="fp64")
    e.copyin(boxes, pos, vel)
    e.calforce()
    f64 = e.get_force()
    e.set_precision("mixed")
    e.set_tuning(density=68, force=20, fused=21)
    e.calforce()
    f32 = e.get_force()
    assert e.tile_stats()["tiled"] > 0
    e.close()
    err = np.abs(f32 - f64).max() / np.abs(f64).max()
    assert err < 1e-6


def test_tile_variants_need_mixed_single_kind():
    pos, vel, L_ = lt.cu_config(4, 0.05, 300.0, 1)
    e = _engine(len(pos), prec="fp64")
    e.copyin([(len(pos), (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
    with pytest.raises(MSMError):
        e.set_tuning(density=66)
    e.close()


@pytest.mark.parametrize("d256,d128,u256,u128", [(3, 131, 14, 46), (19, 147, 12, 44), (5, 133, 17, 49)])
def test_128_thread_block_variants_match(d256, d128, u256, u128):
    # the block size changes only the grid, not the arithmetic of an atom
    pos, vel, L_ = lt.cu_config(9, 0.08, 1200.0, 17)      # 2,916 atoms: partial last blocks
    boxes = [(len(pos), (0, 0, 0), tuple(L_), (1, 1, 1))]
    fa, xa, va, fa2, _ = _run(boxes, pos, vel, d256, u256, steps=30)
    fb, xb, vb, fb2, _ = _run(boxes, pos, vel, d128, u128, steps=30)
    assert np.array_equal(fa, fb)
    assert np.array_equal(xa, xb) and np.array_equal(va, vb) and np.array_equal(fa2, fb2)


def test_tiles_eam_w_match_global_gathers():
    # EAM (Marinica W, F'(rho) from the embedding table) on cell tiles against global gathers
    pos, L_ = lt.w_sia_config(10, 0.03, 12)
    n = len(pos)
    vel = lt.velocities(n, lt.W_MASS, 900.0, np.random.default_rng(13))
    out = []
    for dens, fused in ((19, 12), (66, 20)):
        e = Engine(n, lt.W_RC_NL, mxkvois=96, precision="mixed", outer_skin=0.0)
        e.init_forcetable(ForceTable.marinica_eam2(rc=lt.W_RC))
        e.set_masses([lt.W_MASS])
        e.copyin([(n, (0, 0, 0), tuple(L_), (1, 1, 1))], pos, vel)
        e.set_tuning(density=dens, force=20, fused=fused)
        e.calforce()
        f0 = e.get_force()
        st = e.tile_stats()
        e.run_steps(20, 1.0)
        x, v, _, _ = e.get_state()
        out.append((f0, x, v, e.get_force()))
        e.close()
    assert st["tiled"] > 0
    assert all(np.array_equal(a, b) for a, b in zip(out[0], out[1]))
