"""GPU test of msmgb_calforce_noalloc, the force call for callers that cannot let the library
allocate device memory (their device arrays are owned by their own runtime or budgeted by
their own allocator).  The inputs and the output here live in buffers that the test makes
with torch, standing in for such a caller's arrays; the entry point itself allocates
nothing and keeps F'(rho) in its fixed in-library array.  Its forces must equal those of
the context path (msmgb_calforce) within the FP64 tolerance of the other parity tests, on
two calls in a row (the second call reuses the array the first one left behind).

This file is collected last so that a run stopping at the first failure has already run
every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


def test_noalloc_force_matches_context_path_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
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

    dev = torch.device("cuda:0")
    xp = torch.tensor(np.ascontiguousarray(pos.T).reshape(-1), dtype=torch.float64, device=dev)
    statu = torch.ones(n, dtype=torch.int32, device=dev)
    kv = torch.tensor(kvois, dtype=torch.int32, device=dev)
    ind = torch.tensor(np.ascontiguousarray(indi).reshape(-1), dtype=torch.int32, device=dev)
    potb = torch.tensor(table.potb, dtype=torch.float64, device=dev)
    fpotr = torch.tensor(table.fpotr, dtype=torch.float64, device=dev)
    fpotb = torch.tensor(table.fpotb, dtype=torch.float64, device=dev)
    fp = torch.zeros(3 * n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    errbuf = C.create_string_buffer(256)
    a = L.ForceNoAlloc()
    a.n, a.ld = n, n
    a.xp, a.statu, a.kvois, a.indi = xp.data_ptr(), statu.data_ptr(), kv.data_ptr(), ind.data_ptr()
    for d in range(3):
        a.box_len[d] = float(box_len[d])
        a.ifpd[d] = 1
    a.pottype, a.ntab, a.rmax, a.ru = L.FS_TYPE, table.ntab, table.rmax, table.ru
    a.potb, a.fpotr, a.fpotb = potb.data_ptr(), fpotr.data_ptr(), fpotb.data_ptr()
    a.nembd, a.rhod, a.dfembd = 0, 0.0, None
    a.fp = fp.data_ptr()
    a.stream = None
    a.errbuf, a.errlen = C.cast(errbuf, C.c_char_p), 256
    lib = L.load()
    for call in range(2):
        fp.fill_(float("nan"))
        torch.cuda.synchronize()
        rc = lib.msmgb_calforce_noalloc(C.byref(a))
        assert rc == L.OK, errbuf.value
        f = fp.cpu().numpy().reshape(3, n).T
        err = np.abs(f - f_ref).max() / np.abs(f_ref).max()
        assert err < TOL, (call, err)

    # sizes beyond the fixed array are refused with a clear error, before any GPU work
    a.n = a.ld = L.NOALLOC_MAX_ATOMS + 1
    assert lib.msmgb_calforce_noalloc(C.byref(a)) == L.ERR_CAPACITY
    assert b"MSMGB_NOALLOC_MAX_ATOMS" in errbuf.value
