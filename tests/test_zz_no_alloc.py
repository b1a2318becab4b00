"""h4_forces_noalloc: the force sum for callers that cannot allocate.

Applications that give all of the GPU's memory to their own pool at start-up,
or loops that cannot take an allocation's synchronisation, call this entry
point with their own device buffers; its partial sums live in a fixed
file-scope device array.  This test calls it through the C ABI twice in a
row, on different active sets (the shared scratch keeps the first call's
contents), and compares each result with h4_forces_for, the allocating entry
point, within the force tolerance of the parity tests.  It is collected last
(file name) so that a run stopping at the first failure has run every other
test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
FORCE_RTOL = 1e-12


def _rel(a, b):
    return (np.linalg.norm(a - b, axis=1) / np.maximum(np.linalg.norm(b, axis=1), 1e-300)).max()


def test_forces_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    from gravidy_gb300 import Hermite4GPU, NbodySystem, _lib, ics

    n = 5000
    m, p, v = ics.plummer(n, seed=21, imf="salpeter")
    ns = NbodySystem(m, p, v, softening=0.01)
    pr = np.zeros((n, 4)); pr[:, :3] = p; pr[:, 3] = ns.mass
    pv = np.zeros((n, 4)); pv[:, :3] = v
    rng = np.random.default_rng(5)
    moves = [np.sort(rng.choice(n, size=k, replace=False)).astype(np.uint32) for k in (1234, 77)]

    L = _lib.load()
    dev = torch.device("cuda", 0)
    d_pr = torch.from_numpy(pr).to(dev)
    d_pv = torch.from_numpy(pv).to(dev)
    assert d_pr.data_ptr() % 32 == 0 and d_pv.data_ptr() % 32 == 0
    stream = torch.cuda.current_stream(dev)
    with Hermite4GPU(ns) as g:
        for move in moves:
            want = g.forces_for(pr, pv, move)
            d_move = torch.from_numpy(move.astype(np.int32)).to(dev)
            d_out = torch.zeros((len(move), 6), dtype=torch.float64, device=dev)
            st = L.h4_forces_noalloc(n, ns.e2, C.c_void_p(d_pr.data_ptr()), C.c_void_p(d_pv.data_ptr()),
                                     len(move), C.c_void_p(d_move.data_ptr()), C.c_void_p(d_out.data_ptr()),
                                     C.c_void_p(stream.cuda_stream))
            assert st == 0, L.h4_forces_noalloc_error().decode()
            torch.cuda.synchronize()
            got = d_out.cpu().numpy()
            assert _rel(got[:, :3], want[:, :3]) < FORCE_RTOL
            assert _rel(got[:, 3:], want[:, 3:]) < FORCE_RTOL


def test_forces_noalloc_rejects_oversize_active_set():
    from gravidy_gb300 import _lib
    L = _lib.load()
    too_many = (2 * 1024 * 1024) // 6 + 1
    st = L.h4_forces_noalloc(too_many + 1, 1e-4, C.c_void_p(32), C.c_void_p(64), too_many,
                             C.c_void_p(4), C.c_void_p(8), None)
    assert st == 1  # H4_ERR_ARG, before any device work
    assert "H4_NOALLOC_MAX_NACT" in L.h4_forces_noalloc_error().decode()
    # more particles than h4_create accepts (a count that does not fit an int
    # in the kernels): refused before any device work as well
    st = L.h4_forces_noalloc((1 << 28) + 1, 1e-4, C.c_void_p(32), C.c_void_p(64), 5,
                             C.c_void_p(4), C.c_void_p(8), None)
    assert st == 1
    assert "2^28" in L.h4_forces_noalloc_error().decode()
