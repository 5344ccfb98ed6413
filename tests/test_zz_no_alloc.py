"""The single-patch solve that allocates nothing, checked against the allocating entry point.

ef_fv_solve_noalloc serves callers that cannot allocate device memory (stream capture, host
frameworks that own all device memory, real-time loops).  Its scratch lives in a fixed device array
shared by all calls; this test calls it twice in a row through the C ABI, on different patch sizes
and data, and compares each result with ef_fv_solve at the parity tolerance of the other GPU tests.
It sits in its own file that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-12


def test_noalloc_solve_matches_allocating_solve_twice(lib):
    torch = pytest.importorskip("torch")
    from ellipticforest_gb300 import _lib
    cases = [(16, (-1.0, 1.0, -1.0, 1.0), 0.0, 1), (32, (0.0, 2.0, 0.5, 2.5), -2.0, 2)]
    for n, box, lam, seed in cases:
        rng = np.random.default_rng(seed)
        g = rng.standard_normal(4 * n)
        f = rng.standard_normal(n * n)
        u_ref = np.empty(n * n)
        _lib.check(lib.ef_fv_solve(_lib.EF_SOLVER_FISHPACK90, n, *box, lam, _lib.dptr(g), _lib.dptr(f),
                                   _lib.dptr(u_ref)))
        gd = torch.from_numpy(g).cuda()
        fd = torch.from_numpy(f).cuda()
        ud = torch.full((n * n,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        _lib.check(lib.ef_fv_solve_noalloc(_lib.EF_SOLVER_FISHPACK90, n, *box, lam, C.c_void_p(gd.data_ptr()),
                                           C.c_void_p(fd.data_ptr()), C.c_void_p(ud.data_ptr()), None))
        torch.cuda.synchronize()
        u = ud.cpu().numpy()
        assert np.all(np.isfinite(u))
        assert np.abs(u - u_ref).max() <= REL * np.abs(u_ref).max()


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    from ellipticforest_gb300 import _lib
    code = lib.ef_fv_solve_noalloc(_lib.EF_SOLVER_FISHPACK90, 65, 0.0, 1.0, 0.0, 1.0, 0.0,
                                   C.c_void_p(8), None, C.c_void_p(8), None)
    assert code == _lib.EF_ERR_INVALID
    assert b"64" in lib.ef_last_error()
