"""CPU oracle for the quadtree-adaptive HPS path of EllipticForest (TEST INFRASTRUCTURE ONLY).

This module is the checker, not the product.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import it.  The product path (``ellipticforest_gb300``) never
calls into it and fails loudly when its CUDA library is missing.

It restates, in numpy (FP64), the reference's algorithm step for step:

* ``FiniteVolumeGrid``  -- ``src/Patches/FiniteVolume/FiniteVolumeGrid.cpp:9-36`` (cell centres
  ``x_lower + dx/2 + i*dx``).
* ``FiniteVolumeSolver`` -- ``src/Patches/FiniteVolume/FiniteVolumeSolver.cpp``:
  ``solve`` FivePointStencil branch ``:27-223`` (5-point operator, ghost value ``2g - u``, the
  boundary rows ``cC -= c_side`` and ``f += -2 c_side g``), the FISHPACK90 branch ``:224-290``
  (same discrete system with alpha = beta = 1 and ``lambda = lambda_function(0,0)``; the FISHPACK90
  ``hstcrt_`` dependency is not vendored in the reference, so its cyclic-reduction solver is
  replaced by the LAPACK dgesv inverse of the identical 5-point system), ``mapD2N`` ``:296-353``,
  ``buildD2N``
  ``:355-455`` (the ``#else`` branch: 4n unit Dirichlet solves) and ``particularNeumannData``
  ``:457-462``.
* Interpolation operators -- ``src/SpecialMatrices.hpp:93-173``.
* ``Matrix`` ops -- ``src/Matrix.hpp:430-480`` (``blockPermute``), ``:789-952`` (dgemv, dgemm, dgesv
  wrappers; numpy's ``@`` and ``numpy.linalg.solve`` make the same BLAS/LAPACK calls), ``:962-981``
  (``blockDiagonalMatrix``).
* ``Quadtree`` / ``Mesh::refineByFunction`` -- ``src/Mesh.hpp:111-180`` with the p4est calls restated:
  uniform ``p4est_new_ext`` at ``min_level``, recursive ``p4est_refine`` with the cell-centre test,
  ``p4est_balance(P4EST_CONNECT_CORNER)`` (coarsest 2:1 corner-balanced refinement), node creation by
  ``FiniteVolumeNodeFactory::createChildNode`` (``FiniteVolumeNodeFactory.cpp:15-66``), and the merge
  (post-order) / split (pre-order) traversals of ``src/Quadtree.hpp:322-360,438-511``.
* ``HPSAlgorithm`` -- ``src/HPSAlgorithm.hpp``: ``buildStage`` ``:120-161``, ``upwardsStage``
  ``:178-272``, ``solveStage`` ``:291-445``, ``merge4to1`` ``:497-518``, ``upwards4to1``
  ``:529-551``, ``split1to4`` ``:562-577``, ``leafSolve`` ``:584-596`` and every private step
  ``:676-1230``.

The two hot-path option keys ``cache-operators`` and ``homogeneous-rhs`` keep the reference's
meaning.  ``cache-operators`` keys its cache by the leaf grid's (nx, ny, dx, dy) instead of the
reference's single ``"T_leaf"`` key, which is only correct on uniform meshes.
"""
from __future__ import annotations

import math
from typing import Callable, Dict, List, Optional, Tuple

import numpy as np
import scipy.linalg as sla

FIVE_POINT_STENCIL = "FivePointStencil"
FISHPACK90 = "FISHPACK90"

XDIM, YDIM = 0, 1


# ------------------------------------------------------------------------------------------------
# Grid  (FiniteVolumeGrid.cpp:9-36)
# ------------------------------------------------------------------------------------------------
class FiniteVolumeGrid:
    def __init__(self, nx: int, x_lower: float, x_upper: float, ny: int, y_lower: float, y_upper: float):
        self._nx = int(nx)
        self._ny = int(ny)
        self._xl = float(x_lower)
        self._xu = float(x_upper)
        self._yl = float(y_lower)
        self._yu = float(y_upper)
        self._dx = (self._xu - self._xl) / self._nx if self._nx else 0.0
        self._dy = (self._yu - self._yl) / self._ny if self._ny else 0.0

    def nx(self): return self._nx
    def ny(self): return self._ny
    def xLower(self): return self._xl
    def xUpper(self): return self._xu
    def yLower(self): return self._yl
    def yUpper(self): return self._yu
    def dx(self): return self._dx
    def dy(self): return self._dy

    def point(self, dim: int, index: int) -> float:
        # FiniteVolumeGrid.cpp:24-36: (lower + d/2) + index*d
        if dim == XDIM:
            return (self._xl + self._dx / 2) + index * self._dx
        if dim == YDIM:
            return (self._yl + self._dy / 2) + index * self._dy
        raise ValueError("Invalid `dim` argument.")

    __call__ = point

    def points(self, dim: int) -> np.ndarray:
        if dim == XDIM:
            return (self._xl + self._dx / 2) + np.arange(self._nx) * self._dx
        return (self._yl + self._dy / 2) + np.arange(self._ny) * self._dy


# ------------------------------------------------------------------------------------------------
# Interpolation operators  (SpecialMatrices.hpp:93-173)
# ------------------------------------------------------------------------------------------------
def interpolation_fine2coarse(ncoarse: int) -> np.ndarray:
    """SpecialMatrices.hpp:93-116: row i averages fine entries 2i and 2i+1 with weights 0.5/0.5."""
    L = np.zeros((ncoarse, 2 * ncoarse))
    for i in range(ncoarse):
        L[i, 2 * i] = 0.5
        L[i, 2 * i + 1] = 0.5
    return L


def interpolation_coarse2fine(nfine: int) -> np.ndarray:
    """SpecialMatrices.hpp:136-173: 0.75/0.25 interior pairs, 3-tap one-sided rows at both ends."""
    nrows, ncols = nfine, nfine // 2
    L = np.zeros((nrows, ncols))
    edge = (1.40625, -0.5625, 0.15625)
    k = 3
    for i in range(nrows):
        for j in range(ncols):
            if i == 0 and j == 0:
                L[i, j], L[i, j + 1], L[i, j + 2] = edge[0], edge[1], edge[2]
            elif i == nrows - 1 and j == ncols - k:
                L[i, j], L[i, j + 1], L[i, j + 2] = edge[2], edge[1], edge[0]
            elif i == 2 * j + 1 and i % 2 == 1 and i != nrows - 1:
                L[i, j] = 0.75
                L[i, j + 1] = 0.25
                L[i + 1, j] = 0.25
                L[i + 1, j + 1] = 0.75
    return L


def block_diagonal(blocks: List[np.ndarray]) -> np.ndarray:
    """Matrix.hpp:962-981 (blockDiagonalMatrix)."""
    return sla.block_diag(*blocks)


def block_permute(A: np.ndarray, I, J, R, C) -> np.ndarray:
    """Matrix.hpp:430-480: new row block i is old row block I[i] (sizes R), same for columns."""
    if sum(R) != A.shape[0] or sum(C) != A.shape[1]:
        raise ValueError("[blockPermute] block sizes do not add up")
    rstart = np.concatenate([[0], np.cumsum(R)])
    cstart = np.concatenate([[0], np.cumsum(C)])
    rows = np.concatenate([np.arange(rstart[b], rstart[b] + R[b]) for b in I])
    cols = np.concatenate([np.arange(cstart[b], cstart[b] + C[b]) for b in J])
    return A[np.ix_(rows, cols)]


def vector_block_permute(v: np.ndarray, I, R) -> np.ndarray:
    """Vector.hpp:432 (Vector::blockPermute)."""
    start = np.concatenate([[0], np.cumsum(R)])
    idx = np.concatenate([np.arange(start[b], start[b] + R[b]) for b in I])
    return v[idx]


def dgesv(A: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Matrix.hpp:866-952: LAPACK dgesv (LU with partial pivoting) -- numpy.linalg.solve calls dgesv."""
    return np.linalg.solve(A, B)


# ------------------------------------------------------------------------------------------------
# Patch solver  (FiniteVolumeSolver.cpp)
# ------------------------------------------------------------------------------------------------
def five_point_matrix(grid: FiniteVolumeGrid, alpha_fn, beta_fn, lambda_fn):
    """Dense 5-point operator and boundary-coupling coefficients (FiniteVolumeSolver.cpp:66-200).

    Returns (A, cW, cE, cS, cN) with A[IC, J] as PETSc MatSetValues would hold it; the c* arrays are
    per cell (index j + i*ny) and are used for the boundary right-hand side
    ``f_boundary = -2 c_side g_side`` (cpp:96-184).
    """
    nx, ny = grid.nx(), grid.ny()
    N = nx * ny
    dx, dy = grid.dx(), grid.dy()
    A = np.zeros((N, N))
    cWa = np.zeros(N); cEa = np.zeros(N); cSa = np.zeros(N); cNa = np.zeros(N)
    for j in range(ny):
        for i in range(nx):
            xi = grid(0, i)
            yj = grid(1, j)
            xip = xi + dx / 2.0
            xim = xi - dx / 2.0
            yjp = yj + dy / 2.0
            yjm = yj - dy / 2.0
            alpha_ij = alpha_fn(xi, yj)
            beta_ipj = beta_fn(xip, yj)
            beta_imj = beta_fn(xim, yj)
            beta_ijp = beta_fn(xi, yjp)
            beta_ijm = beta_fn(xi, yjm)
            lambda_ij = lambda_fn(xi, yj)
            cW = alpha_ij * beta_imj / dx ** 2
            cE = alpha_ij * beta_ipj / dx ** 2
            cS = alpha_ij * beta_ijm / dy ** 2
            cN = alpha_ij * beta_ijp / dy ** 2
            cC = -alpha_ij * ((beta_ipj + beta_imj) / dx ** 2 + (beta_ijp + beta_ijm) / dy ** 2) + lambda_ij
            IC = j + i * ny
            cWa[IC], cEa[IC], cSa[IC], cNa[IC] = cW, cE, cS, cN
            diag = cC
            if i > 0:
                A[IC, IC - ny] = cW
            else:
                diag -= cW
            if i < nx - 1:
                A[IC, IC + ny] = cE
            else:
                diag -= cE
            if j > 0:
                A[IC, IC - 1] = cS
            else:
                diag -= cS
            if j < ny - 1:
                A[IC, IC + 1] = cN
            else:
                diag -= cN
            A[IC, IC] = diag
    return A, cWa, cEa, cSa, cNa


def boundary_rhs(grid: FiniteVolumeGrid, g: np.ndarray, cW, cE, cS, cN) -> np.ndarray:
    """The ``f_boundary`` additions of FiniteVolumeSolver.cpp:96-184 for WESN Dirichlet data ``g``.

    ``g`` may be a vector (4n) or a matrix (4n x k) of several Dirichlet data sets.
    """
    nx, ny = grid.nx(), grid.ny()
    n = nx
    g = np.asarray(g, dtype=np.float64)
    gW, gE, gS, gN = g[0:n], g[n:2 * n], g[2 * n:3 * n], g[3 * n:4 * n]
    shape = (nx * ny,) + g.shape[1:]
    fb = np.zeros(shape)
    for i in range(nx):
        for j in range(ny):
            if 0 < i < nx - 1 and 0 < j < ny - 1:
                continue
            ic = j + i * ny
            # cpp:100-184: f_boundary = -2.0*(c_x*g_x + c_y*g_y) at corners, -2.0*(c*g) on edges
            acc = None
            if i == 0:
                acc = cW[ic] * gW[j]
            elif i == nx - 1:
                acc = cE[ic] * gE[j]
            if j == 0:
                t = cS[ic] * gS[i]
                acc = t if acc is None else acc + t
            elif j == ny - 1:
                t = cN[ic] * gN[i]
                acc = t if acc is None else acc + t
            fb[ic] = -2.0 * acc
    return fb


class FiniteVolumeSolver:
    """Restatement of FiniteVolumeSolver (FiniteVolumeSolver.hpp:53-162).

    The dense 5-point matrix for a grid is inverted once with LAPACK dgesv (numpy) and kept (keyed
    by the grid and the solver type); each call applies the inverse.  The reference refactors for
    every call (PETSc ``MatLUFactor`` per solve, or one ``hstcrt_`` per solve); the solution of the
    same linear system is the same up to roundoff.  Every LAPACK/BLAS call of the oracle goes
    through numpy's library, so the CPU timings see one BLAS thread pool as the reference does.
    """

    def __init__(self, alpha_function=None, beta_function=None, lambda_function=None, rhs_function=None,
                 solver_type: str = FIVE_POINT_STENCIL):
        self.solver_type = solver_type
        self.alpha_function = alpha_function or (lambda x, y: 1.0)
        self.beta_function = beta_function or (lambda x, y: 1.0)
        self.lambda_function = lambda_function or (lambda x, y: 0.0)
        self.rhs_function = rhs_function
        self._factor_cache: Dict[tuple, tuple] = {}

    def name(self):
        return "FiniteVolumeSolver"

    # -- operator ---------------------------------------------------------------------------
    def _operator(self, grid: FiniteVolumeGrid):
        key = (self.solver_type, grid.nx(), grid.ny(), grid.dx(), grid.dy(),
               grid.xLower(), grid.yLower())
        if self.solver_type == FISHPACK90:
            # hstcrt_ solves u_xx + u_yy + lambda u = f; alpha and beta are not used
            # (FiniteVolumeSolver.cpp:224-290, ELMBDA = lambda_function(0,0) at :253).
            lam = float(self.lambda_function(0, 0))
            key = (self.solver_type, grid.nx(), grid.ny(), grid.dx(), grid.dy(), lam)
        hit = self._factor_cache.get(key)
        if hit is not None:
            return hit
        if self.solver_type == FISHPACK90:
            one = lambda x, y: 1.0
            lamc = lambda x, y: lam
            A, cW, cE, cS, cN = five_point_matrix(grid, one, one, lamc)
        else:
            A, cW, cE, cS, cN = five_point_matrix(grid, self.alpha_function, self.beta_function,
                                                  self.lambda_function)
        Ainv = np.linalg.solve(A, np.eye(A.shape[0]))
        entry = (Ainv, cW, cE, cS, cN)
        self._factor_cache[key] = entry
        return entry

    def solve(self, grid: FiniteVolumeGrid, dirichlet_data, rhs_data) -> np.ndarray:
        """FiniteVolumeSolver.cpp:27-290: u = A^{-1} (f + f_boundary(g)); several columns allowed."""
        Ainv, cW, cE, cS, cN = self._operator(grid)
        f = np.asarray(rhs_data, dtype=np.float64)
        g = np.asarray(dirichlet_data, dtype=np.float64)
        rhs = f + boundary_rhs(grid, g, cW, cE, cS, cN)
        return Ainv @ rhs

    def mapD2N(self, grid: FiniteVolumeGrid, dirichlet_data, rhs_data) -> np.ndarray:
        """FiniteVolumeSolver.cpp:296-353: h_W = (2/dx)(u_W - g_W), h_E = -(2/dx)(u_E - g_E), ..."""
        n = grid.nx()
        g = np.asarray(dirichlet_data, dtype=np.float64)
        u = self.solve(grid, g, rhs_data)
        idxW = np.arange(n)
        idxE = (n - 1) * n + np.arange(n)
        idxS = np.arange(n) * n
        idxN = (np.arange(n) + 1) * n - 1
        dtn_x = 2.0 / grid.dx()
        dtn_y = 2.0 / grid.dy()
        h = np.empty_like(g)
        h[0:n] = dtn_x * (u[idxW] - g[0:n])
        h[n:2 * n] = (-dtn_x) * (u[idxE] - g[n:2 * n])
        h[2 * n:3 * n] = dtn_y * (u[idxS] - g[2 * n:3 * n])
        h[3 * n:4 * n] = (-dtn_y) * (u[idxN] - g[3 * n:4 * n])
        return h

    def buildD2N(self, grid: FiniteVolumeGrid) -> np.ndarray:
        """FiniteVolumeSolver.cpp:355-455 (#else branch): column j = mapD2N(e_j, f = 0)."""
        n = grid.nx()
        M = 4 * n
        E = np.eye(M)
        fz = np.zeros((n * grid.ny(), M))
        return self.mapD2N(grid, E, fz)

    def particularNeumannData(self, grid: FiniteVolumeGrid, rhs_data) -> np.ndarray:
        """FiniteVolumeSolver.cpp:457-462: mapD2N(g = 0, f)."""
        g0 = np.zeros(2 * grid.nx() + 2 * grid.ny())
        return self.mapD2N(grid, g0, rhs_data)


# ------------------------------------------------------------------------------------------------
# Patch / node / node factory  (FiniteVolumePatch.hpp, QuadNode.hpp, FiniteVolumeNodeFactory.cpp)
# ------------------------------------------------------------------------------------------------
class FiniteVolumePatch:
    def __init__(self, grid: Optional[FiniteVolumeGrid] = None):
        self._grid = grid if grid is not None else FiniteVolumeGrid(0, 0, 0, 0, 0, 0)
        self.n_coarsens = 0
        self.X = np.zeros((0, 0)); self.H = np.zeros((0, 0))
        self.S = np.zeros((0, 0)); self.T = np.zeros((0, 0))
        self.u = np.zeros(0); self.g = np.zeros(0); self.v = np.zeros(0)
        self.f = np.zeros(0); self.h = np.zeros(0); self.w = np.zeros(0)

    def name(self): return "FiniteVolumePatch"
    def grid(self) -> FiniteVolumeGrid: return self._grid
    def set_grid(self, grid: FiniteVolumeGrid): self._grid = grid

    def size(self) -> int:
        # Patch.hpp:99-101
        return int(self._grid.nx() / 2 ** self.n_coarsens)


class Node:
    def __init__(self, data: FiniteVolumePatch, path: str, level: int):
        self.data = data
        self.path = path
        self.level = level
        self.leaf = False


class FiniteVolumeNodeFactory:
    """FiniteVolumeNodeFactory.cpp:11-66."""

    def createNode(self, data: FiniteVolumePatch, path: str, level: int) -> Node:
        return Node(data, path, level)

    def createChildNode(self, parent: Node, sibling_id: int) -> Node:
        pg = parent.data.grid()
        nx, ny = pg.nx(), pg.ny()
        xl, xu = pg.xLower(), pg.xUpper()
        yl, yu = pg.yLower(), pg.yUpper()
        xm = (xl + xu) / 2.0
        ym = (yl + yu) / 2.0
        if sibling_id == 0:
            g = FiniteVolumeGrid(nx, xl, xm, ny, yl, ym)
        elif sibling_id == 1:
            g = FiniteVolumeGrid(nx, xm, xu, ny, yl, ym)
        elif sibling_id == 2:
            g = FiniteVolumeGrid(nx, xl, xm, ny, ym, yu)
        else:
            g = FiniteVolumeGrid(nx, xm, xu, ny, ym, yu)
        return Node(FiniteVolumePatch(g), parent.path + str(sibling_id), parent.level + 1)


# ------------------------------------------------------------------------------------------------
# Quadtree refinement restating the p4est calls of Mesh::refineByFunction (Mesh.hpp:111-180)
# ------------------------------------------------------------------------------------------------
P4EST_MAXLEVEL = 30
P4EST_ROOT_LEN = 1 << P4EST_MAXLEVEL


def qcoord_to_vertex(xl, xu, yl, yu, qx: int, qy: int) -> Tuple[float, float]:
    """Bilinear vertex interpolation of one square tree (p4est_qcoord_to_vertex on the
    connectivity of P4est.cpp:7-33)."""
    wx1 = qx / P4EST_ROOT_LEN
    wx0 = 1.0 - wx1
    wy1 = qy / P4EST_ROOT_LEN
    wy0 = 1.0 - wy1
    verts = ((xl, yl), (xu, yl), (xl, yu), (xu, yu))
    vx = 0.0
    vy = 0.0
    k = 0
    for wy in (wy0, wy1):
        for wx in (wx0, wx1):
            fac = wy * wx
            vx += fac * verts[k][0]
            vy += fac * verts[k][1]
            k += 1
    return vx, vy


def quadrant_refine_test(fn, xl, xu, yl, yu, nx, ny, level, ix, iy, max_level) -> bool:
    """The p4est_refine callback of Mesh.hpp:135-162."""
    if level >= max_level:
        return False
    qlen = 1 << (P4EST_MAXLEVEL - level)
    qx, qy = ix * qlen, iy * qlen
    x0, y0 = qcoord_to_vertex(xl, xu, yl, yu, qx, qy)
    x1, y1 = qcoord_to_vertex(xl, xu, yl, yu, qx + qlen, qy + qlen)
    dx = (x1 - x0) / nx
    dy = (y1 - y0) / ny
    for i in range(nx):
        for j in range(ny):
            x = x0 + (i + 0.5) * dx
            y = y0 + (j + 0.5) * dy
            if fn(x, y):
                return True
    return False


def refine_leaves(fn, xl, xu, yl, yu, nx, ny, min_level, max_level):
    """Leaves (level, ix, iy) after p4est_new_ext(min_level) + recursive p4est_refine + corner balance."""
    leaves = set()
    stack = [(min_level, ix, iy) for ix in range(1 << min_level) for iy in range(1 << min_level)]
    while stack:
        lvl, ix, iy = stack.pop()
        if quadrant_refine_test(fn, xl, xu, yl, yu, nx, ny, lvl, ix, iy, max_level):
            for c in range(4):
                stack.append((lvl + 1, 2 * ix + (c & 1), 2 * iy + (c >> 1)))
        else:
            leaves.add((lvl, ix, iy))
    return corner_balance(leaves)


def corner_balance(leaves):
    """Coarsest refinement in which leaves sharing a face or a corner differ by at most one level
    (p4est_balance with P4EST_CONNECT_CORNER)."""
    leaves = set(leaves)

    def find_leaf(level, ix, iy):
        # the leaf containing quadrant (level, ix, iy) if it is at that level or coarser
        for l in range(level, -1, -1):
            s = level - l
            key = (l, ix >> s, iy >> s)
            if key in leaves:
                return key
        return None

    changed = True
    while changed:
        changed = False
        # the finest leaves drive refinement of coarse neighbours
        for leaf in sorted(leaves, key=lambda t: -t[0]):
            if leaf not in leaves:
                continue
            lvl, ix, iy = leaf
            if lvl < 2:
                continue
            n = 1 << lvl
            for dxo in (-1, 0, 1):
                for dyo in (-1, 0, 1):
                    if dxo == 0 and dyo == 0:
                        continue
                    jx, jy = ix + dxo, iy + dyo
                    if jx < 0 or jy < 0 or jx >= n or jy >= n:
                        continue
                    nb = find_leaf(lvl, jx, jy)
                    if nb is None or nb[0] >= lvl - 1:
                        continue
                    # neighbour too coarse: split it (and repeat until balanced)
                    leaves.discard(nb)
                    nl, nxi, nyi = nb
                    for c in range(4):
                        leaves.add((nl + 1, 2 * nxi + (c & 1), 2 * nyi + (c >> 1)))
                    changed = True
    return leaves


def leaf_path(level, ix, iy) -> str:
    """p4est_quadrant_path (P4est.cpp:35-43): '0' then the child id at each level (z-order)."""
    p = ""
    for l in range(level, 0, -1):
        s = level - l
        cid = ((ix >> s) & 1) | (((iy >> s) & 1) << 1)
        p = str(cid) + p
    return "0" + p


class Quadtree:
    """Path-indexed quadtree (Quadtree.hpp:48-360) without p4est/MPI."""

    def __init__(self, leaves=None, root_patch: Optional[FiniteVolumePatch] = None,
                 node_factory: Optional[FiniteVolumeNodeFactory] = None):
        self.map: Dict[str, Node] = {}
        self.leaf_set = set()
        if leaves is not None:
            self._build(leaves, root_patch, node_factory or FiniteVolumeNodeFactory())

    def _build(self, leaves, root_patch, factory):
        leaf_paths = {leaf_path(*l) for l in leaves}
        # every ancestor of a leaf is a node (p4est_search_all visits them all)
        paths = set()
        for p in leaf_paths:
            for k in range(1, len(p) + 1):
                paths.add(p[:k])
        root = factory.createNode(FiniteVolumePatch(root_patch.grid()), "0", 0)
        self.map["0"] = root
        for p in sorted(paths, key=lambda s: (len(s), s)):
            if p == "0":
                continue
            parent = self.map[p[:-1]]
            self.map[p] = factory.createChildNode(parent, int(p[-1]))
        for p in leaf_paths:
            self.map[p].leaf = True
        self.leaf_set = leaf_paths

    def root(self) -> FiniteVolumePatch:
        return self.map["0"].data

    def _children(self, node: Node) -> List[Node]:
        return [self.map[node.path + str(i)] for i in range(4)]

    def traversePreOrder(self, visit: Callable[[Node], int]):
        def rec(node):
            visit(node)
            if not node.leaf:
                for c in self._children(node):
                    rec(c)
        rec(self.map["0"])

    def traversePostOrder(self, visit: Callable[[Node], int]):
        def rec(node):
            if not node.leaf:
                for c in self._children(node):
                    rec(c)
            visit(node)
        rec(self.map["0"])

    def merge(self, visit_leaf, visit_family):
        """Quadtree.hpp:322-331 (post-order family callbacks)."""
        def rec(node):
            if node.leaf:
                visit_leaf(node)
                return
            ch = self._children(node)
            for c in ch:
                rec(c)
            visit_family(node, ch)
        rec(self.map["0"])

    def split(self, visit_leaf, visit_family):
        """Quadtree.hpp:345-354 (pre-order family callbacks)."""
        def rec(node):
            if node.leaf:
                visit_leaf(node)
                return
            ch = self._children(node)
            visit_family(node, ch)
            for c in ch:
                rec(c)
        rec(self.map["0"])

    def leaves(self) -> List[Node]:
        out = []
        self.traversePreOrder(lambda n: out.append(n) if n.leaf else None)
        return out


class Mesh:
    """Mesh<FiniteVolumePatch> (Mesh.hpp:13-180) without VTK output."""

    def __init__(self, quadtree: Optional[Quadtree] = None):
        self.quadtree = quadtree or Quadtree()

    def refineByFunction(self, fn, threshold, min_level, max_level, root_patch: FiniteVolumePatch,
                         node_factory: Optional[FiniteVolumeNodeFactory] = None):
        g = root_patch.grid()
        leaves = refine_leaves(fn, g.xLower(), g.xUpper(), g.yLower(), g.yUpper(), g.nx(), g.ny(),
                               min_level, max_level)
        self.quadtree = Quadtree(leaves, root_patch, node_factory)
        return self

    def uniform(self, level: int, root_patch: FiniteVolumePatch,
                node_factory: Optional[FiniteVolumeNodeFactory] = None):
        leaves = {(level, ix, iy) for ix in range(1 << level) for iy in range(1 << level)}
        self.quadtree = Quadtree(leaves, root_patch, node_factory)
        return self

    def iteratePatches(self, fn):
        for node in self.quadtree.leaves():
            fn(node.data)

    def iterateCells(self, fn):
        for node in self.quadtree.leaves():
            g = node.data.grid()
            for i in range(g.nx()):
                for j in range(g.ny()):
                    fn(g(0, i), g(1, j))


# ------------------------------------------------------------------------------------------------
# HPS algorithm  (HPSAlgorithm.hpp)
# ------------------------------------------------------------------------------------------------
PI_WESN = [0, 4, 2, 6, 1, 3, 5, 7]


class HPSAlgorithm:
    """HPSAlgorithm<FiniteVolumeGrid, FiniteVolumeSolver, FiniteVolumePatch, double>."""

    def __init__(self, mesh: Mesh, patch_solver: FiniteVolumeSolver, options: Optional[dict] = None):
        self.mesh = mesh
        self.patch_solver = patch_solver
        self.options = {"cache-operators": False, "homogeneous-rhs": False}
        if options:
            self.options.update(options)
        self.matrixCache: Dict[tuple, np.ndarray] = {}

    # -- stages ------------------------------------------------------------------------------
    def setupStage(self):
        pass

    def buildStage(self):
        """HPSAlgorithm.hpp:120-161."""
        def leaf(node):
            patch = node.data
            if self.options["cache-operators"]:
                g = patch.grid()
                key = (g.nx(), g.ny(), g.dx(), g.dy())
                if key not in self.matrixCache:
                    self.matrixCache[key] = self.patch_solver.buildD2N(g)
                patch.T = self.matrixCache[key].copy()
            else:
                patch.T = self.patch_solver.buildD2N(patch.grid())
            return 1

        def family(parent, children):
            self.merge4to1(parent.data, *[c.data for c in children])
            return 1

        self.mesh.quadtree.merge(leaf, family)

    def upwardsStage(self, rhs):
        """HPSAlgorithm.hpp:178-272.  ``rhs`` is either f(x, y) or a patch callback (patch) -> None;
        a callable with attribute ``patch_callback = True`` is treated as the latter."""
        patch_cb = getattr(rhs, "patch_callback", False)

        def leaf(node):
            patch = node.data
            grid = patch.grid()
            if patch_cb:
                rhs(patch)
            else:
                f = np.empty(grid.nx() * grid.ny())
                for i in range(grid.nx()):
                    x = grid(0, i)
                    for j in range(grid.ny()):
                        y = grid(1, j)
                        f[j + i * grid.ny()] = rhs(x, y)
                patch.f = f
            patch.h = self.patch_solver.particularNeumannData(grid, patch.f)
            return 1

        def family(parent, children):
            self.upwards4to1(parent.data, *[c.data for c in children])
            return 1

        self.mesh.quadtree.merge(leaf, family)

    def solveStage(self, bc):
        """HPSAlgorithm.hpp:291-445.  ``bc`` is either the analytical boundary function
        (side, x, y) -> (r, a, b) or a root-patch callback (attribute ``patch_callback = True``)."""
        root = self.mesh.quadtree.root()
        if getattr(bc, "patch_callback", False):
            bc(root)
        else:
            g = root.grid()
            M = g.nx()
            r = np.zeros(4 * M); a = np.zeros(4 * M); b = np.zeros(4 * M)
            for n in range(4):
                for i in range(M):
                    if n == 0:
                        x, y = g.xLower(), g(1, i)
                    elif n == 1:
                        x, y = g.xUpper(), g(1, i)
                    elif n == 2:
                        x, y = g(0, i), g.yLower()
                    else:
                        x, y = g(0, i), g.yUpper()
                    rv, av, bv = bc(n, x, y)
                    r[n * M + i], a[n * M + i], b[n * M + i] = rv, av, bv
            root.g = self.root_dirichlet(root, a, b, r)

        def leaf(node):
            self.leafSolve(node.data)
            return 1

        def family(parent, children):
            self.split1to4(parent.data, *[c.data for c in children])
            return 1

        self.mesh.quadtree.split(leaf, family)

    def upwards_with_data(self, f_all: np.ndarray):
        """upwardsStage with the load already sampled: f_all holds every leaf's f in pre-order leaf
        order (the values the rhs callback of HPSAlgorithm.hpp:241-249 would produce)."""
        leaves = self.mesh.quadtree.leaves()
        nn = f_all.size // len(leaves)
        data = {id(nd.data): f_all[k * nn:(k + 1) * nn] for k, nd in enumerate(leaves)}

        @patch_callback
        def setf(patch):
            patch.f = data[id(patch)]
        self.upwardsStage(setf)

    def solve_with_data(self, a, b, r):
        """solveStage with the boundary condition already sampled at the root face centres
        (HPSAlgorithm.hpp:375-400): a, b, r are 4M WESN vectors."""
        @patch_callback
        def setg(rp):
            rp.g = self.root_dirichlet(rp, np.asarray(a, float), np.asarray(b, float), np.asarray(r, float))
        self.solveStage(setg)

    def root_dirichlet(self, root: FiniteVolumePatch, a, b, r):
        """HPSAlgorithm.hpp:402-420: g = (diag(a) + diag(b) T)^{-1} (r - diag(b) h)."""
        h = root.h if root.h.size == r.size else np.zeros_like(r)
        A = np.diag(a)
        B = np.diag(b)
        bh = B @ h
        rhs = r - bh
        A = A + B @ root.T
        return dgesv(A, rhs)

    # -- virtual hooks -----------------------------------------------------------------------
    def merge4to1(self, tau, alpha, beta, gamma, omega):
        """HPSAlgorithm.hpp:497-518."""
        self._coarsen(tau, alpha, beta, gamma, omega)
        IS = self._index_sets(alpha, beta, gamma, omega)
        B = self._matrix_blocks(IS, alpha, beta, gamma, omega)
        self._mergeX(tau, B)
        self._mergeS(tau, B)
        self._mergeT(tau, B)
        self._reorder(tau, alpha)
        self._merge_patch(tau, alpha, beta, gamma)

    def upwards4to1(self, tau, alpha, beta, gamma, omega):
        """HPSAlgorithm.hpp:529-551."""
        if not self.options["homogeneous-rhs"]:
            self._coarsen_upwards(alpha, beta, gamma, omega)
            IS = self._index_sets(alpha, beta, gamma, omega)
            B = self._matrix_blocks(IS, alpha, beta, gamma, omega)
            self._mergeX(tau, B)
            self._mergeW(tau, IS, alpha, beta, gamma, omega)
            self._mergeH(tau, IS, alpha, beta, gamma, omega)
            self._reorder_upwards(tau, alpha, beta, gamma, omega)

    def split1to4(self, tau, alpha, beta, gamma, omega):
        """HPSAlgorithm.hpp:562-577."""
        self._uncoarsen(tau)
        self._applyS(tau, alpha, beta, gamma, omega)

    def leafSolve(self, patch):
        """HPSAlgorithm.hpp:584-596."""
        if self.options["homogeneous-rhs"]:
            patch.f = np.zeros(patch.grid().nx() * patch.grid().ny())
        patch.u = self.patch_solver.solve(patch.grid(), patch.g, patch.f)

    # -- merge steps (HPSAlgorithm.hpp:676-1009) ---------------------------------------------
    @staticmethod
    def _tags(patches):
        sides = [p.size() for p in patches]
        mn = min(sides)
        return [int(math.log2(s)) - int(math.log2(mn)) for s in sides]

    def _coarsen(self, tau, *children):
        """HPSAlgorithm.hpp:707-741."""
        tags = self._tags(children)
        for patch, tag in zip(children, tags):
            for n in range(tag):
                ngrid = patch.grid().nx()
                coarsen_factor = tag - (tag - n)
                nfine = int(ngrid / 2 ** coarsen_factor)
                ncoarse = nfine // 2
                L21 = block_diagonal([interpolation_fine2coarse(ncoarse)] * 4)
                L12 = block_diagonal([interpolation_coarse2fine(nfine)] * 4)
                patch.T = L21 @ patch.T
                patch.T = patch.T @ L12
                patch.n_coarsens += 1

    @staticmethod
    def _index_sets(alpha, beta, gamma, omega):
        """HPSAlgorithm.hpp:752-788."""
        n = [alpha.size(), beta.size(), gamma.size(), omega.size()]
        if any(v != n[0] for v in n):
            raise ValueError("[createIndexSets_] Size of children patches are not the same")
        ns = alpha.T.shape[0] // 4
        W = np.arange(0, ns); E = np.arange(ns, 2 * ns)
        S = np.arange(2 * ns, 3 * ns); N = np.arange(3 * ns, 4 * ns)
        return {
            "ab": E, "ag": N, "at": np.concatenate([W, S]),
            "ba": W, "bo": N, "bt": np.concatenate([E, S]),
            "ga": S, "go": E, "gt": np.concatenate([W, N]),
            "ob": S, "og": W, "ot": np.concatenate([E, N]),
        }

    @staticmethod
    def _matrix_blocks(IS, alpha, beta, gamma, omega):
        """HPSAlgorithm.hpp:799-859 (blocks and their negations)."""
        Ta, Tb, Tg, To = alpha.T, beta.T, gamma.T, omega.T
        sub = lambda T, r, c: T[np.ix_(IS[r], IS[c])]
        B = {}
        B["ag_ag"] = sub(Ta, "ag", "ag"); B["ga_ga"] = sub(Tg, "ga", "ga")
        B["ag_ab"] = sub(Ta, "ag", "ab"); B["ga_go"] = sub(Tg, "ga", "go")
        B["bo_bo"] = sub(Tb, "bo", "bo"); B["ob_ob"] = sub(To, "ob", "ob")
        B["bo_ba"] = sub(Tb, "bo", "ba"); B["ob_og"] = sub(To, "ob", "og")
        B["ab_ag"] = sub(Ta, "ab", "ag"); B["ba_bo"] = sub(Tb, "ba", "bo")
        B["ab_ab"] = sub(Ta, "ab", "ab"); B["ba_ba"] = sub(Tb, "ba", "ba")
        B["go_ga"] = sub(Tg, "go", "ga"); B["og_ob"] = sub(To, "og", "ob")
        B["go_go"] = sub(Tg, "go", "go"); B["og_og"] = sub(To, "og", "og")
        B["ag_at"] = sub(Ta, "ag", "at"); B["ga_gt"] = sub(Tg, "ga", "gt")
        B["bo_bt"] = sub(Tb, "bo", "bt"); B["ob_ot"] = sub(To, "ob", "ot")
        B["ab_at"] = sub(Ta, "ab", "at"); B["ba_bt"] = sub(Tb, "ba", "bt")
        B["go_gt"] = sub(Tg, "go", "gt"); B["og_ot"] = sub(To, "og", "ot")
        B["at_at"] = sub(Ta, "at", "at"); B["bt_bt"] = sub(Tb, "bt", "bt")
        B["gt_gt"] = sub(Tg, "gt", "gt"); B["ot_ot"] = sub(To, "ot", "ot")
        B["at_ag"] = sub(Ta, "at", "ag"); B["at_ab"] = sub(Ta, "at", "ab")
        B["bt_bo"] = sub(Tb, "bt", "bo"); B["bt_ba"] = sub(Tb, "bt", "ba")
        B["gt_ga"] = sub(Tg, "gt", "ga"); B["gt_go"] = sub(Tg, "gt", "go")
        B["ot_ob"] = sub(To, "ot", "ob"); B["ot_og"] = sub(To, "ot", "og")
        for k in ("ga_go", "ob_og", "ba_bo", "og_ob", "ag_at", "bo_bt", "ab_at", "go_gt"):
            B[k] = -B[k]
        return B

    @staticmethod
    def _mergeX(tau, B):
        """HPSAlgorithm.hpp:870-895."""
        d = [B["ag_ag"] - B["ga_ga"], B["bo_bo"] - B["ob_ob"], B["ab_ab"] - B["ba_ba"], B["go_go"] - B["og_og"]]
        X = block_diagonal(d)
        rs = np.concatenate([[0], np.cumsum([m.shape[0] for m in d])])
        cs = np.concatenate([[0], np.cumsum([m.shape[1] for m in d])])

        def put(r, c, M):
            X[rs[r]:rs[r] + M.shape[0], cs[c]:cs[c] + M.shape[1]] = M
        put(0, 2, B["ag_ab"]); put(0, 3, B["ga_go"])
        put(1, 2, B["bo_ba"]); put(1, 3, B["ob_og"])
        put(2, 0, B["ab_ag"]); put(2, 1, B["ba_bo"])
        put(3, 0, B["go_ga"]); put(3, 1, B["og_ob"])
        tau.X = X

    @staticmethod
    def _mergeS(tau, B):
        """HPSAlgorithm.hpp:906-929."""
        rows = [B["ag_at"].shape[0], B["bo_bt"].shape[0], B["ab_at"].shape[0], B["go_gt"].shape[0]]
        cols = [B["ag_at"].shape[1], B["bo_bt"].shape[1], B["ga_gt"].shape[1], B["ob_ot"].shape[1]]
        R = np.zeros((sum(rows), sum(cols)))
        rs = np.concatenate([[0], np.cumsum(rows)])
        cs = np.concatenate([[0], np.cumsum(cols)])

        def put(r, c, M):
            R[rs[r]:rs[r] + M.shape[0], cs[c]:cs[c] + M.shape[1]] = M
        put(0, 0, B["ag_at"]); put(0, 2, B["ga_gt"])
        put(1, 1, B["bo_bt"]); put(1, 3, B["ob_ot"])
        put(2, 0, B["ab_at"]); put(2, 1, B["ba_bt"])
        put(3, 2, B["go_gt"]); put(3, 3, B["og_ot"])
        tau.S = dgesv(tau.X, R)

    @staticmethod
    def _mergeT(tau, B):
        """HPSAlgorithm.hpp:940-968."""
        T_LHS = block_diagonal([B["at_at"], B["bt_bt"], B["gt_gt"], B["ot_ot"]])
        rows = [B["at_ag"].shape[0], B["bt_bo"].shape[0], B["gt_ga"].shape[0], B["ot_ob"].shape[0]]
        cols = [B["at_ag"].shape[1], B["bt_bo"].shape[1], B["at_ab"].shape[1], B["gt_go"].shape[1]]
        H = np.zeros((sum(rows), sum(cols)))
        rs = np.concatenate([[0], np.cumsum(rows)])
        cs = np.concatenate([[0], np.cumsum(cols)])

        def put(r, c, M):
            H[rs[r]:rs[r] + M.shape[0], cs[c]:cs[c] + M.shape[1]] = M
        put(0, 0, B["at_ag"]); put(0, 2, B["at_ab"])
        put(1, 1, B["bt_bo"]); put(1, 2, B["bt_ba"])
        put(2, 0, B["gt_ga"]); put(2, 3, B["gt_go"])
        put(3, 1, B["ot_ob"]); put(3, 3, B["ot_og"])
        tau.H = H
        tau.T = T_LHS + H @ tau.S

    @staticmethod
    def _reorder(tau, alpha):
        """HPSAlgorithm.hpp:979-993."""
        ns = alpha.T.shape[0] // 4
        tau.S = block_permute(tau.S, [0, 1, 2, 3], PI_WESN, [ns] * 4, [ns] * 8)
        tau.T = block_permute(tau.T, PI_WESN, PI_WESN, [ns] * 8, [ns] * 8)

    @staticmethod
    def _merge_patch(tau, alpha, beta, gamma):
        """HPSAlgorithm.hpp:1004-1009."""
        ag, bg, gg = alpha.grid(), beta.grid(), gamma.grid()
        tau.set_grid(FiniteVolumeGrid(alpha.size() + beta.size(), ag.xLower(), bg.xUpper(),
                                      alpha.size() + gamma.size(), ag.yLower(), gg.yUpper()))

    # -- upward steps (HPSAlgorithm.hpp:1024-1150) -------------------------------------------
    @staticmethod
    def _coarsen_upwards(*children):
        for patch in children:
            for n in range(patch.n_coarsens):
                ngrid = patch.grid().nx()
                nfine = int(ngrid / 2 ** n)
                ncoarse = nfine // 2
                L21 = block_diagonal([interpolation_fine2coarse(ncoarse)] * 4)
                patch.h = L21 @ patch.h

    @staticmethod
    def _mergeW(tau, IS, alpha, beta, gamma, omega):
        hd = np.concatenate([
            gamma.h[IS["ga"]] - alpha.h[IS["ag"]],
            omega.h[IS["ob"]] - beta.h[IS["bo"]],
            beta.h[IS["ba"]] - alpha.h[IS["ab"]],
            omega.h[IS["og"]] - gamma.h[IS["go"]],
        ])
        tau.w = dgesv(tau.X, hd)

    @staticmethod
    def _mergeH(tau, IS, alpha, beta, gamma, omega):
        h = tau.H @ tau.w
        h = h + np.concatenate([alpha.h[IS["at"]], beta.h[IS["bt"]], gamma.h[IS["gt"]], omega.h[IS["ot"]]])
        tau.h = h

    @staticmethod
    def _reorder_upwards(tau, alpha, beta, gamma, omega):
        n = [alpha.size(), beta.size(), gamma.size(), omega.size()]
        if any(v != n[0] for v in n):
            raise ValueError("[reorderOperatorsUpwards_] Size of children patches are not the same")
        ns = alpha.T.shape[0] // 4
        tau.h = vector_block_permute(tau.h, PI_WESN, [ns] * 8)

    # -- split steps (HPSAlgorithm.hpp:1165-1230) --------------------------------------------
    @staticmethod
    def _uncoarsen(tau):
        for n in range(tau.n_coarsens):
            ngrid = tau.grid().nx()
            coarsen_factor = tau.n_coarsens - (n + 1)
            nfine = int(ngrid / 2 ** coarsen_factor)
            L12 = block_diagonal([interpolation_coarse2fine(nfine)] * 4)
            tau.g = L12 @ tau.g

    def _applyS(self, tau, alpha, beta, gamma, omega):
        u = tau.S @ tau.g
        if not self.options["homogeneous-rhs"]:
            u = u + tau.w
        ns = alpha.size()
        seg = lambda v, k: v[k * ns:(k + 1) * ns]
        g_ag, g_bo, g_ab, g_go = seg(u, 0), seg(u, 1), seg(u, 2), seg(u, 3)
        G = tau.g
        aW, gW, bE, oE = seg(G, 0), seg(G, 1), seg(G, 2), seg(G, 3)
        aS, bS, gN, oN = seg(G, 4), seg(G, 5), seg(G, 6), seg(G, 7)
        alpha.g = np.concatenate([aW, g_ab, aS, g_ag])
        beta.g = np.concatenate([g_ab, bE, bS, g_bo])
        gamma.g = np.concatenate([gW, g_go, g_ag, gN])
        omega.g = np.concatenate([g_go, oE, g_bo, oN])


# ------------------------------------------------------------------------------------------------
# Convenience helpers used by tests and by the CPU baseline
# ------------------------------------------------------------------------------------------------
def patch_callback(fn):
    """Mark ``fn`` as a patch callback for upwardsStage/solveStage."""
    fn.patch_callback = True
    return fn


def leaf_solution(hps: HPSAlgorithm) -> np.ndarray:
    """Leaf u concatenated in pre-order (z-order) leaf order."""
    return np.concatenate([n.data.u for n in hps.mesh.quadtree.leaves()])


def leaf_cell_centres(mesh: Mesh) -> Tuple[np.ndarray, np.ndarray]:
    xs, ys = [], []
    for node in mesh.quadtree.leaves():
        g = node.data.grid()
        X, Y = np.meshgrid(g.points(0), g.points(1), indexing="ij")
        xs.append(X.ravel()); ys.append(Y.ravel())
    return np.concatenate(xs), np.concatenate(ys)
