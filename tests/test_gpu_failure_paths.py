"""Failure paths that return status codes instead of wrong numbers (no GPU fault involved).

- FivePointStencil leaves are factored without pivoting, which is safe exactly when the operator
  alpha div(beta grad) + lambda is (alpha-scaled) negative definite.  A small positive lambda keeps
  it definite and must still match the oracle (the reference factors with a pivoted LU); a lambda
  above the smallest eigenvalue of the diffusion part, or alpha*beta changing sign, must be refused
  with EF_ERR_UNSUPPORTED.
- A leaf operator with a zero pivot (alpha = 0, lambda = 0) is reported as EF_ERR_SINGULAR.
- A server request for a tree that does not exist is refused with EF_ERR_INVALID.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ef(lib):
    import ellipticforest_gb300
    return ellipticforest_gb300


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _fv5(lib, n, box, alpha, beta, lam):
    from ellipticforest_gb300 import _lib
    from ellipticforest_gb300.hps import FiniteVolumeGrid, FiniteVolumeSolver, sample_coefficients
    s = FiniteVolumeSolver(alpha_function=alpha, beta_function=beta, lambda_function=lam)
    a, b, l = (np.ascontiguousarray(v) for v in sample_coefficients(s, FiniteVolumeGrid(n, box[0], box[1], n, box[2], box[3])))
    T = np.empty((4 * n, 4 * n))
    code = lib.ef_fv5_build_d2n(n, *box, _lib.dptr(a), _lib.dptr(b), _lib.dptr(l), _lib.dptr(T))
    return code, T


def test_small_positive_lambda_matches_oracle(ef, lib):
    # lambda = +20 on a 0.5 x 0.5 patch: below the smallest eigenvalue (~2 pi^2 / 0.25 = 79) of the
    # Laplacian there, so the operator is still negative definite
    n, box = 16, (0.0, 0.5, 0.0, 0.5)
    alpha = lambda x, y: 1.0 + 0.0 * x
    beta = lambda x, y: 1.0 + 0.25 * np.sin(3 * x) * np.cos(2 * y)
    lam = lambda x, y: 20.0 + 0.0 * x
    code, T = _fv5(lib, n, box, alpha, beta, lam)
    assert code == 0
    To = O.FiniteVolumeSolver(alpha_function=alpha, beta_function=beta, lambda_function=lam,
                              solver_type=O.FIVE_POINT_STENCIL).buildD2N(O.FiniteVolumeGrid(n, *box[:2], n, *box[2:]))
    assert rel(T, To) <= 1e-12


@pytest.mark.parametrize("what", ["lambda", "sign"])
def test_indefinite_five_point_operator_is_refused(ef, lib, what):
    from ellipticforest_gb300 import _lib
    n, box = 16, (0.0, 0.5, 0.0, 0.5)
    if what == "lambda":   # far above the smallest eigenvalue: indefinite Helmholtz
        alpha, beta, lam = (lambda x, y: 1.0 + 0.0 * x), (lambda x, y: 1.0 + 0.0 * x), (lambda x, y: 5000.0 + 0.0 * x)
    else:                  # alpha * beta changes sign across the patch
        alpha, beta, lam = (lambda x, y: 1.0 + 0.0 * x), (lambda x, y: x - 0.25), (lambda x, y: 0.0 * x)
    code, _ = _fv5(lib, n, box, alpha, beta, lam)
    assert code == _lib.EF_ERR_UNSUPPORTED
    assert b"negative definite" in lib.ef_last_error()
    # the same on a tree: the build stage refuses it
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, *box[:2], 8, *box[2:]))
    mesh = ef.Mesh().uniform(1, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(alpha_function=alpha, beta_function=beta, lambda_function=lam,
                                                      solver_type=ef.FivePointStencil))
    with pytest.raises(_lib.EFError) as ei:
        hps.buildStage()
    assert ei.value.code == _lib.EF_ERR_UNSUPPORTED


def test_zero_pivot_is_reported_singular(ef, lib):
    from ellipticforest_gb300 import _lib
    zero = lambda x, y: 0.0 * x
    code, _ = _fv5(lib, 8, (0.0, 1.0, 0.0, 1.0), zero, lambda x, y: 1.0 + 0.0 * x, zero)
    assert code == _lib.EF_ERR_SINGULAR


def test_server_rejects_an_unknown_tree(ef, lib):
    from ellipticforest_gb300 import _lib
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -1.0, 1.0, 16, -1.0, 1.0))
    mesh = ef.Mesh().uniform(2, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    srv = ef.Server([hps], bmax=4, lanes=1)
    cells = hps.num_leaves * 256
    f = np.zeros(cells)
    a = np.ones(4 * hps.M)
    r = np.zeros(4 * hps.M)
    u = np.empty(cells)
    rid = C.c_longlong(-1)
    for bad in (1, -1, 7):
        code = lib.ef_server_submit(srv._h, bad, _lib.dptr(f), _lib.dptr(a), _lib.dptr(r), _lib.dptr(u), C.byref(rid))
        assert code == _lib.EF_ERR_INVALID
    # the server still answers a valid request
    rid_ok = srv.submit(0, np.ones(cells), a, np.ones(4 * hps.M))
    uu, _ = srv.wait(rid_ok)
    assert np.all(np.isfinite(uu))
    del srv


@pytest.mark.parametrize("tensor_cores", [0, 2])
def test_bounded_tma_wait_runs_out_and_returns_an_error(ef, lib, tensor_cores):
    """The node GEMMs wait for their TMA copies with a limit.  With the failure-path test switch on,
    every CTA's first wait is on an mbarrier that nothing arrives on (limit 1 ms); the kernels drain
    their copies in flight and set the error word, the mixed solve returns EF_ERR_CUDA, and with the
    switch off again the same handle solves correctly (the context stays usable)."""
    from ellipticforest_gb300 import _lib
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -1.0, 1.0, 16, -1.0, 1.0))
    mesh = ef.Mesh().uniform(3, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    _lib.check(lib.ef_hps_set_option(hps.handle, b"tensor-cores", tensor_cores))
    hps.mixed_init(2)
    X, Y = mesh.cell_centres()
    F = np.stack([np.sin(X + k) * np.cos(Y) for k in range(2)])
    R = np.stack([np.concatenate([np.cos(x - y + k) for x, y in hps.boundary_points()]) for k in range(2)])
    A = np.ones_like(R)
    good = hps.mixed_solve(F, A, R, sweeps=1)
    _lib.check(lib.ef_hps_set_option(hps.handle, b"inject-wait-timeout", 1))
    try:
        u = np.empty_like(F)
        code = lib.ef_hps_mixed_solve(hps.handle, 2, 1, _lib.dptr(F), _lib.dptr(A), _lib.dptr(R), _lib.dptr(u))
        assert code == _lib.EF_ERR_CUDA
        assert b"did not complete" in lib.ef_last_error()
    finally:
        _lib.check(lib.ef_hps_set_option(hps.handle, b"inject-wait-timeout", 0))
    again = hps.mixed_solve(F, A, R, sweeps=1)
    assert np.array_equal(again, good)
    _lib.check(lib.ef_hps_set_option(hps.handle, b"tensor-cores", 1))
