"""Global 5-point finite-volume solve on a uniform mesh (TEST INFRASTRUCTURE ONLY).

A second, independent oracle.  On a uniform quadtree the HPS solution with the leaf DtN of
``FiniteVolumeSolver.cpp:296-353`` reproduces the global cell-centred 5-point system exactly (up to
roundoff): the leaf flux is ``h = (2/d)(u - g)``, so flux continuity across an interface forces
``g = (u_L + u_R)/2``, which is the global stencil.  This module assembles that global system with
the Dirichlet ghost ``u_ghost = 2 g - u`` of ``FiniteVolumeSolver.cpp:100-184`` and solves it with
``scipy.sparse``.  Only ``tests/`` and the CPU-baseline legs of ``bench.py`` import it.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def assemble(nx: int, ny: int, xl: float, xu: float, yl: float, yu: float,
             alpha=None, beta=None, lam=None):
    """Global operator for alpha div(beta grad u) + lambda u (vectorised FiniteVolumeSolver.cpp:66-100).

    alpha, beta, lam are vectorised callables f(X, Y) (defaults 1, 1, 0).  Global cell index is
    ``j + i*ny`` as in the leaf solver.  Returns (A, cW, cE, cS, cN, x, y).
    """
    dx = (xu - xl) / nx
    dy = (yu - yl) / ny
    x = (xl + dx / 2) + np.arange(nx) * dx
    y = (yl + dy / 2) + np.arange(ny) * dy
    X, Y = np.meshgrid(x, y, indexing="ij")
    one = lambda X, Y: np.ones_like(X)
    zero = lambda X, Y: np.zeros_like(X)
    alpha = alpha or one
    beta = beta or one
    lam = lam or zero
    a = alpha(X, Y)
    bW = beta(X - dx / 2, Y); bE = beta(X + dx / 2, Y)
    bS = beta(X, Y - dy / 2); bN = beta(X, Y + dy / 2)
    cW = a * bW / dx ** 2; cE = a * bE / dx ** 2
    cS = a * bS / dy ** 2; cN = a * bN / dy ** 2
    cC = -a * ((bE + bW) / dx ** 2 + (bN + bS) / dy ** 2) + lam(X, Y)
    diag = cC.copy()
    diag[0, :] -= cW[0, :]
    diag[-1, :] -= cE[-1, :]
    diag[:, 0] -= cS[:, 0]
    diag[:, -1] -= cN[:, -1]
    idx = (np.arange(nx)[:, None] * ny + np.arange(ny)[None, :])
    rows = [idx.ravel()]; cols = [idx.ravel()]; vals = [diag.ravel()]
    rows.append(idx[1:, :].ravel()); cols.append(idx[:-1, :].ravel()); vals.append(cW[1:, :].ravel())
    rows.append(idx[:-1, :].ravel()); cols.append(idx[1:, :].ravel()); vals.append(cE[:-1, :].ravel())
    rows.append(idx[:, 1:].ravel()); cols.append(idx[:, :-1].ravel()); vals.append(cS[:, 1:].ravel())
    rows.append(idx[:, :-1].ravel()); cols.append(idx[:, 1:].ravel()); vals.append(cN[:, :-1].ravel())
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(nx * ny, nx * ny))
    return A, cW, cE, cS, cN, x, y


def solve_dirichlet(nx, ny, xl, xu, yl, yu, f_fn, g_fn, alpha=None, beta=None, lam=None):
    """Solve with load f_fn(X, Y) at cell centres and Dirichlet data g_fn(x, y) at face centres.

    Returns U[i, j] (x-index outer) and the cell-centre coordinates.
    """
    A, cW, cE, cS, cN, x, y = assemble(nx, ny, xl, xu, yl, yu, alpha, beta, lam)
    X, Y = np.meshgrid(x, y, indexing="ij")
    F = np.array(f_fn(X, Y), dtype=np.float64)
    gW = g_fn(np.full(ny, xl), y); gE = g_fn(np.full(ny, xu), y)
    gS = g_fn(x, np.full(nx, yl)); gN = g_fn(x, np.full(nx, yu))
    F[0, :] += -2.0 * cW[0, :] * gW
    F[-1, :] += -2.0 * cE[-1, :] * gE
    F[:, 0] += -2.0 * cS[:, 0] * gS
    F[:, -1] += -2.0 * cN[:, -1] * gN
    u = spla.spsolve(A.tocsc(), F.ravel())
    return u.reshape(nx, ny), x, y


def to_leaf_order(U: np.ndarray, level: int, n: int) -> np.ndarray:
    """Reorder a global (2^L n) x (2^L n) cell array into the HPS leaf order: leaves in z-order
    (pre-order of the quadtree, child ids 0=SW,1=SE,2=NW,3=NE), each leaf's cells as j + i*n."""
    out = []

    def rec(lvl, ix, iy):
        if lvl == level:
            out.append(U[ix * n:(ix + 1) * n, iy * n:(iy + 1) * n].ravel())
            return
        for c in range(4):
            rec(lvl + 1, 2 * ix + (c & 1), 2 * iy + (c >> 1))
    rec(0, 0, 0)
    return np.concatenate(out)


def solve_poisson_dst(F: np.ndarray, gW, gE, gS, gN, xl: float, xu: float, yl: float, yu: float,
                      lam: float = 0.0) -> np.ndarray:
    """Direct solve of the same global system for constant coefficients (alpha = beta = 1, constant
    lambda) by the sine transform that diagonalises it: with the Dirichlet ghost ``2 g - u`` the 1-D
    second difference has the eigenvectors sin(pi (k+1)(i+1/2)/N) (the orthonormal DST-II basis) and
    eigenvalues -(4/d^2) sin^2(pi (k+1)/(2N)).  O(N^2 log N) instead of a sparse LU, so the level-7
    grid (2048^2 cells) solves in seconds; pinned against ``solve_dirichlet`` (sparse LU) in the
    tests.  F is the load at cell centres [nx, ny] (x index outer); g* the face data per side.
    """
    import scipy.fft as fft
    nx, ny = F.shape
    dx, dy = (xu - xl) / nx, (yu - yl) / ny
    R = np.array(F, dtype=np.float64, copy=True)
    R[0, :] += -2.0 * gW / dx ** 2
    R[-1, :] += -2.0 * gE / dx ** 2
    R[:, 0] += -2.0 * gS / dy ** 2
    R[:, -1] += -2.0 * gN / dy ** 2
    mx = -(4.0 / dx ** 2) * np.sin(np.pi * (np.arange(nx) + 1) / (2 * nx)) ** 2
    my = -(4.0 / dy ** 2) * np.sin(np.pi * (np.arange(ny) + 1) / (2 * ny)) ** 2
    Rh = fft.dstn(R, type=2, norm="ortho", workers=-1)
    Uh = Rh / (mx[:, None] + my[None, :] + lam)
    return fft.idstn(Uh, type=2, norm="ortho", workers=-1)
