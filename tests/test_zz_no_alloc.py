"""The single-patch solve that allocates nothing, checked against the allocating entry point.

ef_fv_solve_noalloc serves callers that cannot allocate device memory: plugins inside a host
framework that owns all device memory through its own pool, and real-time loops that must not
allocate after start-up.  Its scratch lives in a fixed device array shared by all calls.  These
tests call it through the C ABI two times in a row, on different patch sizes and data, and compare
each result with ef_fv_solve at the parity tolerance of the other GPU tests: once in this process
(after whatever other tests ran before it) and once in a fresh process whose very first library
call is the no-alloc solve, so nothing else has set up device state it might read.  The file is
named so that pytest collects it last.
"""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-12
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = [(16, (-1.0, 1.0, -1.0, 1.0), 0.0, 1), (64, (0.0, 2.0, 0.5, 2.5), -2.0, 2),
         (32, (-3.0, 1.0, -2.0, 2.0), 1.5, 3)]


def _noalloc(lib, torch, n, box, lam, g, f):
    from ellipticforest_gb300 import _lib
    gd = torch.from_numpy(g).cuda()
    fd = torch.from_numpy(f).cuda()
    ud = torch.full((n * n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    _lib.check(lib.ef_fv_solve_noalloc(_lib.EF_SOLVER_FISHPACK90, n, *box, lam, C.c_void_p(gd.data_ptr()),
                                       C.c_void_p(fd.data_ptr()), C.c_void_p(ud.data_ptr()), None))
    torch.cuda.synchronize()
    return ud.cpu().numpy()


def _allocating(lib, n, box, lam, g, f):
    from ellipticforest_gb300 import _lib
    u_ref = np.empty(n * n)
    _lib.check(lib.ef_fv_solve(_lib.EF_SOLVER_FISHPACK90, n, *box, lam, _lib.dptr(g), _lib.dptr(f),
                               _lib.dptr(u_ref)))
    return u_ref


def _data(n, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(4 * n), rng.standard_normal(n * n)


def test_noalloc_solve_matches_allocating_solve_twice(lib):
    torch = pytest.importorskip("torch")
    for n, box, lam, seed in CASES:
        g, f = _data(n, seed)
        u = _noalloc(lib, torch, n, box, lam, g, f)
        u_ref = _allocating(lib, n, box, lam, g, f)
        assert np.all(np.isfinite(u))
        assert np.abs(u - u_ref).max() <= REL * np.abs(u_ref).max(), n


_FRESH = textwrap.dedent("""
    import sys
    sys.path.insert(0, {root!r})
    import numpy as np
    import torch
    from ellipticforest_gb300 import _lib
    sys.path.insert(0, {tests!r})
    import test_zz_no_alloc as T
    lib = _lib.load()
    cases = T.CASES[:2]
    # the no-alloc solves come first, before any other call into the library
    got = [T._noalloc(lib, torch, n, box, lam, *T._data(n, seed)) for n, box, lam, seed in cases]
    for (n, box, lam, seed), u in zip(cases, got):
        u_ref = T._allocating(lib, n, box, lam, *T._data(n, seed))
        err = np.abs(u - u_ref).max() / np.abs(u_ref).max()
        print(n, err)
        assert np.all(np.isfinite(u)) and err <= T.REL, (n, err)
    print("fresh ok")
""")


def test_noalloc_solve_first_call_in_fresh_process(lib):
    pytest.importorskip("torch")
    code = _FRESH.format(root=ROOT, tests=os.path.join(ROOT, "tests"))
    res = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0 and "fresh ok" in res.stdout, res.stdout + res.stderr


def test_noalloc_rejects_sizes_beyond_its_scratch(lib):
    from ellipticforest_gb300 import _lib
    code = lib.ef_fv_solve_noalloc(_lib.EF_SOLVER_FISHPACK90, 65, 0.0, 1.0, 0.0, 1.0, 0.0,
                                   C.c_void_p(8), None, C.c_void_p(8), None)
    assert code == _lib.EF_ERR_INVALID
    assert b"64" in lib.ef_last_error()
