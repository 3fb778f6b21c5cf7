"""GPU tests of msmgb_calforce_noalloc, the force call for callers that cannot let the library
allocate device memory (their device arrays are owned by their own runtime or budgeted by
their own allocator).  The inputs and the output here live in buffers that the tests make
with torch, standing in for such a caller's arrays; the entry point itself allocates
nothing and keeps F'(rho) in its fixed in-library array.  Its forces must equal those of
the context path (msmgb_calforce) within the FP64 tolerance of the other parity tests, on
two calls in a row (the second call reuses the array the first one left behind), and the
oracle's for an EAM potential and for a state with inactive atoms.  A density beyond the
F(rho) table and a neighbour id outside the atom range come back as status codes.

This file is collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import cu_tables, w_tables, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _torch():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    return torch


class _Call:
    """The argument block of one msmgb_calforce_noalloc call with every array in device memory
    (torch tensors kept alive here), neighbour list in the caller's (original) atom order."""

    def __init__(self, torch, pos, box_len, statu, kvois, indi, table):
        from msmpscu_gb300 import _lib as L
        self.L = L
        n = len(pos)
        dev = torch.device("cuda:0")
        self.keep = []

        def dt(a, dtype):
            t = torch.tensor(np.ascontiguousarray(a).reshape(-1), dtype=dtype, device=dev)
            self.keep.append(t)
            return t.data_ptr()

        self.fp = torch.zeros(3 * n, dtype=torch.float64, device=dev)
        self.errbuf = C.create_string_buffer(256)
        a = L.ForceNoAlloc()
        a.n, a.ld = n, indi.shape[1]
        a.xp = dt(pos.T, torch.float64)
        a.statu = dt(statu, torch.int32)
        a.kvois = dt(kvois, torch.int32)
        a.indi = dt(indi, torch.int32)
        for d in range(3):
            a.box_len[d] = float(box_len[d])
            a.ifpd[d] = 1
        a.pottype, a.ntab, a.rmax, a.ru = table.pottype, table.ntab, table.rmax, table.ru
        a.potb, a.fpotr, a.fpotb = (dt(getattr(table, k), torch.float64) for k in ("potb", "fpotr", "fpotb"))
        if table.pottype == L.EAM_TYPE:
            a.nembd, a.rhod, a.dfembd = table.nembd, table.rhod, dt(table.dfembd, torch.float64)
        else:
            a.nembd, a.rhod, a.dfembd = 0, 0.0, None
        a.fp = self.fp.data_ptr()
        a.stream = None
        a.errbuf, a.errlen = C.cast(self.errbuf, C.c_char_p), 256
        self.a = a
        self.n = n
        self.torch = torch
        torch.cuda.synchronize()

    def run(self):
        self.fp.fill_(float("nan"))
        self.torch.cuda.synchronize()
        rc = self.L.load().msmgb_calforce_noalloc(C.byref(self.a))
        return rc, self.fp.cpu().numpy().reshape(3, self.n).T


def test_noalloc_force_matches_context_path_twice():
    torch = _torch()
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    from msmpscu_gb300 import _lib as L

    pos, vel, box_len = lt.cu_config(12, 0.05, 600.0, 77)          # 6,912 atoms
    n = len(pos)
    table = ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC)
    e = Engine(n, lt.CU_RC_NL, mxkvois=64)
    e.init_forcetable(table)
    e.copyin([(n, (0, 0, 0), tuple(box_len), (1, 1, 1))], pos, vel)
    e.calforce()
    f_ref = e.get_force()
    kvois, indi = e.get_neighborelist()                              # caller order
    e.close()

    call = _Call(torch, pos, box_len, np.ones(n, np.int32), kvois, indi, table)
    for k in range(2):
        rc, f = call.run()
        assert rc == L.OK, call.errbuf.value
        assert rel_err(f, f_ref) < TOL, (k, rel_err(f, f_ref))

    # sizes beyond the fixed array are refused with a clear error, before any GPU work
    call.a.n = call.a.ld = L.NOALLOC_MAX_ATOMS + 1
    assert L.load().msmgb_calforce_noalloc(C.byref(call.a)) == L.ERR_CAPACITY
    assert b"MSMGB_NOALLOC_MAX_ATOMS" in call.errbuf.value


def test_noalloc_eam_matches_oracle_and_context_path(oracle):
    """Marinica EAM2 tungsten with a <111> dumbbell: the EAM branch (DFEMBD interpolation at
    SK = rho/RHOD + 1 with the reference's +1e-6 index rule)."""
    torch = _torch()
    from msmpscu_gb300 import Engine, ForceTable, lattice as lt
    from msmpscu_gb300 import _lib as L

    pos, box_len = lt.w_sia_config(8, 0.02, 3)                       # 1,025 atoms
    n = len(pos)
    st = np.ones(n, np.int32)
    t = w_tables(oracle)
    box = oracle.make_box([0, 0, 0], box_len)
    kv, ind = oracle.nlist(pos, st, box, lt.W_RC_NL, 128)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)["f"]
    table = ForceTable.marinica_eam2()
    e = Engine(n, lt.W_RC_NL, mxkvois=96)
    e.init_forcetable(table)
    e.copyin([(n, (0, 0, 0), tuple(box_len), (1, 1, 1))], pos)
    e.calforce()
    f_ctx = e.get_force()
    e.close()

    call = _Call(torch, pos, box_len, st, kv, ind, table)
    for k in range(2):
        rc, f = call.run()
        assert rc == L.OK, call.errbuf.value
        assert rel_err(f, ref) < TOL, (k, rel_err(f, ref))
        assert rel_err(f, f_ctx) < TOL, (k, rel_err(f, f_ctx))


def test_noalloc_inactive_atoms_match_oracle(oracle):
    """Atoms with STATU bit 0 clear take no part: zero force on them, no contribution to others."""
    torch = _torch()
    from msmpscu_gb300 import ForceTable, lattice as lt
    from msmpscu_gb300 import _lib as L

    pos, vel, box_len = lt.cu_config(6, 0.05, 300.0, 4)             # 864 atoms
    n = len(pos)
    st = np.ones(n, np.int32)
    st[::7] = 0
    t = cu_tables(oracle)
    box = oracle.make_box([0, 0, 0], box_len)
    kv, ind = oracle.nlist(pos, st, box, lt.CU_RC_NL, 96)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, t)["f"]
    call = _Call(torch, pos, box_len, st, kv, ind, ForceTable.cleri_rosato(**lt.CU_CR, rc=lt.CU_RC))
    for k in range(2):
        rc, f = call.run()
        assert rc == L.OK, call.errbuf.value
        assert np.all(f[::7] == 0.0)
        assert rel_err(f, ref) < TOL, (k, rel_err(f, ref))


def test_noalloc_status_codes(oracle):
    """A density beyond the F(rho) table returns MSMGB_ERR_RHO_RANGE (the table is read
    clamped, nothing outside it); neighbour ids outside 0..n-1 (a 1-based Fortran INDI passed
    unchanged) are not read and return MSMGB_ERR_ARG.  A correct call afterwards is exact
    again: the error word starts from zero in every call."""
    torch = _torch()
    from msmpscu_gb300 import ForceTable, lattice as lt
    from msmpscu_gb300 import _lib as L

    pos, box_len = lt.w_sia_config(6, 0.02, 5)                       # 433 atoms
    n = len(pos)
    st = np.ones(n, np.int32)
    box = oracle.make_box([0, 0, 0], box_len)
    kv, ind = oracle.nlist(pos, st, box, lt.W_RC_NL, 128)
    table = ForceTable.marinica_eam2()

    call = _Call(torch, pos, box_len, st, kv, ind, table)
    call.a.rhod = table.rhod / 50.0          # rho / RHOD + 1 then lies far beyond NEMBD
    rc, _ = call.run()
    assert rc == L.ERR_RHO_RANGE, call.errbuf.value
    assert b"F(rho)" in call.errbuf.value

    one_based = np.where(np.arange(ind.shape[0])[:, None] < kv[None, :], ind + 1, 0)
    bad = _Call(torch, pos, box_len, st, kv, one_based.astype(np.int32), table)
    rc, f = bad.run()
    assert rc == L.ERR_ARG, bad.errbuf.value
    assert b"0-based" in bad.errbuf.value

    good = _Call(torch, pos, box_len, st, kv, ind, table)
    ref = oracle.force(pos, np.ones(n, np.int32), st, box, kv, ind, w_tables(oracle))["f"]
    rc, f = good.run()
    assert rc == L.OK, good.errbuf.value
    assert rel_err(f, ref) < TOL
