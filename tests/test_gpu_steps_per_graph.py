"""Several MD steps per CUDA graph launch (msmgb_set_steps_per_graph): the same steps as one
graph per step, bitwise (positions, velocities, forces, rebuild counts), in every precision,
for one box and for a batch of uneven boxes, with far fewer graph launches."""
import numpy as np
import pytest

from msmpscu_gb300 import Engine, ForceTable, lattice as lt

pytestmark = pytest.mark.gpu


def _run(boxes, pos, vel, prec, k, steps):
    e = Engine(len(pos), lt.CU_RC_NL, max_boxes=len(boxes), mxkvois=64, precision=prec, skin_trigger=0.15)
    e.init_forcetable(ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    e.set_masses([lt.CU_MASS])
    e.copyin(boxes, pos, vel)
    if prec == "mixed":
        # the same kernel variants in both runs (the autotuner may pick variants with other
        # record formats, whose arithmetic differs)
        e.set_tuning(density=275, force=128 + 50, fused=128 + 32 + 15)
    e.set_steps_per_graph(k)
    g0 = e.graph_launches
    reb = e.run_steps(steps, 1.0)
    launches = e.graph_launches - g0
    x, v, _, _ = e.get_state()
    f = e.get_force()
    e.close()
    return x, v, f, reb, launches


@pytest.mark.parametrize("prec", ["fp64", "mixed", "ff"])
def test_k_steps_per_graph_bitwise(prec):
    pos, vel, L_ = lt.cu_config(8, 0.08, 1500.0, 21)
    boxes = [(len(pos), (0, 0, 0), tuple(L_), (1, 1, 1))]
    steps = 37
    x1, v1, f1, r1, g1 = _run(boxes, pos, vel, prec, 1, steps)
    x8, v8, f8, r8, g8 = _run(boxes, pos, vel, prec, 8, steps)
    assert np.array_equal(x1, x8) and np.array_equal(v1, v8) and np.array_equal(f1, f8)
    assert r1 == r8 and r1 > 0
    assert g8 <= g1 // 3


def test_k_steps_per_graph_batched_boxes():
    boxes_raw = lt.uneven_batch(24, seed=8, cmin=4, cmax=7)
    pos = np.vstack([b[0] for b in boxes_raw])
    vel = np.vstack([b[1] for b in boxes_raw])
    boxes = [(len(b[0]), (0, 0, 0), tuple(b[2]), (1, 1, 1)) for b in boxes_raw]
    a = _run(boxes, pos, vel, "mixed", 1, 40)
    b = _run(boxes, pos, vel, "mixed", 10, 40)
    for u, w in zip(a[:3], b[:3]):
        assert np.array_equal(u, w)
    assert a[3] == b[3] and a[3] > 0
    # first step, 3 graphs of 10 steps, 9 single steps, last step
    assert a[4] == 41 and b[4] == 14
