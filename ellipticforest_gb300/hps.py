"""Python mirror of EllipticForest's HPS path, running on the GB300 CUDA library.

Same class and method names as the reference's C++ API (``src/HPSAlgorithm.hpp``,
``src/Mesh.hpp``, ``src/Patches/FiniteVolume/*``) so that drivers and tests read like the
reference's own.  Every numerical step goes through the C ABI of ``libellipticforest_gb300.so``;
this module only samples the user's callbacks at the reference's sampling points and moves arrays.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Callable, Optional

import numpy as np

from . import _lib
from ._lib import check, dptr

FivePointStencil = "FivePointStencil"
FISHPACK90 = "FISHPACK90"
XDIM, YDIM = 0, 1


def _solver_code(solver_type: str) -> int:
    if solver_type == FISHPACK90:
        return _lib.EF_SOLVER_FISHPACK90
    if solver_type == FivePointStencil:
        return _lib.EF_SOLVER_FIVE_POINT
    raise ValueError(f"unknown solver type {solver_type!r}")


class FiniteVolumeGrid:
    """FiniteVolumeGrid (FiniteVolumeGrid.cpp:9-36)."""

    def __init__(self, nx: int, x_lower: float, x_upper: float, ny: int, y_lower: float, y_upper: float):
        self._nx, self._ny = int(nx), int(ny)
        self._xl, self._xu = float(x_lower), float(x_upper)
        self._yl, self._yu = float(y_lower), float(y_upper)
        self._dx = (self._xu - self._xl) / self._nx
        self._dy = (self._yu - self._yl) / self._ny

    def nx(self): return self._nx
    def ny(self): return self._ny
    def xLower(self): return self._xl
    def xUpper(self): return self._xu
    def yLower(self): return self._yl
    def yUpper(self): return self._yu
    def dx(self): return self._dx
    def dy(self): return self._dy

    def point(self, dim: int, index):
        if dim == XDIM:
            return (self._xl + self._dx / 2) + np.asarray(index) * self._dx
        if dim == YDIM:
            return (self._yl + self._dy / 2) + np.asarray(index) * self._dy
        raise ValueError("Invalid `dim` argument.")

    def __call__(self, dim, index):
        return self.point(dim, index)


def _sample(fn, X, Y):
    v = np.asarray(fn(X, Y), dtype=np.float64)
    return np.ascontiguousarray(np.broadcast_to(v, X.shape), dtype=np.float64)


def sample_coefficients(solver, grid):
    """alpha, beta (W, E, S, N faces of every cell) and lambda of one patch, sampled at the points
    of FiniteVolumeSolver.cpp:66-79 with the same arithmetic (x_i -/+ dx/2.0, y_j -/+ dy/2.0).
    The coefficient functions are called with numpy arrays."""
    n = grid.nx()
    dx, dy = grid.dx(), grid.dy()
    X, Y = np.meshgrid(grid.point(0, np.arange(n)), grid.point(1, np.arange(n)), indexing="ij")
    alpha = _sample(solver.alpha_function, X, Y).ravel()
    beta = np.concatenate([_sample(solver.beta_function, X - dx / 2.0, Y).ravel(),
                           _sample(solver.beta_function, X + dx / 2.0, Y).ravel(),
                           _sample(solver.beta_function, X, Y - dy / 2.0).ravel(),
                           _sample(solver.beta_function, X, Y + dy / 2.0).ravel()])
    lam = _sample(solver.lambda_function, X, Y).ravel()
    return alpha, beta, lam


class FiniteVolumeSolver:
    """FiniteVolumeSolver (FiniteVolumeSolver.hpp:53-162) on the GPU.

    ``solver_type = FISHPACK90`` solves u_xx + u_yy + lambda u = f with
    ``lambda = lambda_function(0, 0)`` (FiniteVolumeSolver.cpp:253); alpha and beta are not used,
    exactly as in the reference's FISHPACK90 branch.  ``solver_type = FivePointStencil`` solves
    alpha div(beta grad u) + lambda u = f with the coefficient functions sampled per cell
    (FiniteVolumeSolver.cpp:27-223); they are called with numpy arrays.
    """

    def __init__(self, alpha_function=None, beta_function=None, lambda_function=None, rhs_function=None,
                 solver_type: str = FivePointStencil):
        self.solver_type = solver_type  # the reference's default is FivePointStencil
        self.alpha_function = alpha_function or (lambda x, y: 1.0)
        self.beta_function = beta_function or (lambda x, y: 1.0)
        self.lambda_function = lambda_function or (lambda x, y: 0.0)
        self.rhs_function = rhs_function

    def name(self):
        return "FiniteVolumeSolver"

    def _lam(self) -> float:
        return float(self.lambda_function(0, 0))

    def _args(self, grid: FiniteVolumeGrid):
        if grid.nx() != grid.ny():
            raise ValueError("square patches only (nx == ny)")
        return (_solver_code(self.solver_type), grid.nx(), grid.xLower(), grid.xUpper(),
                grid.yLower(), grid.yUpper(), self._lam())

    def _fp_args(self, grid: FiniteVolumeGrid):
        if grid.nx() != grid.ny():
            raise ValueError("square patches only (nx == ny)")
        a, b, l = sample_coefficients(self, grid)
        self._keep = (a, b, l)
        return (grid.nx(), grid.xLower(), grid.xUpper(), grid.yLower(), grid.yUpper(), dptr(a), dptr(b), dptr(l))

    def buildD2N(self, grid: FiniteVolumeGrid) -> np.ndarray:
        n = grid.nx()
        T = np.empty((4 * n, 4 * n))
        if self.solver_type == FivePointStencil:
            check(_lib.load().ef_fv5_build_d2n(*self._fp_args(grid), dptr(T)))
        else:
            check(_lib.load().ef_fv_build_d2n(*self._args(grid), dptr(T)))
        return T

    def solve(self, grid: FiniteVolumeGrid, dirichlet_data, rhs_data) -> np.ndarray:
        n = grid.nx()
        g = np.ascontiguousarray(dirichlet_data, dtype=np.float64)
        f = np.ascontiguousarray(rhs_data, dtype=np.float64)
        if g.size != 4 * n or f.size != n * n:
            raise ValueError("size mismatch")
        u = np.empty(n * n)
        if self.solver_type == FivePointStencil:
            check(_lib.load().ef_fv5_solve(*self._fp_args(grid), dptr(g), dptr(f), dptr(u)))
        else:
            check(_lib.load().ef_fv_solve(*self._args(grid), dptr(g), dptr(f), dptr(u)))
        return u

    def mapD2N(self, grid: FiniteVolumeGrid, dirichlet_data, rhs_data) -> np.ndarray:
        n = grid.nx()
        g = np.ascontiguousarray(dirichlet_data, dtype=np.float64)
        f = np.ascontiguousarray(rhs_data, dtype=np.float64)
        if g.size != 4 * n or f.size != n * n:
            raise ValueError("size mismatch")
        h = np.empty(4 * n)
        if self.solver_type == FivePointStencil:
            check(_lib.load().ef_fv5_map_d2n(*self._fp_args(grid), dptr(g), dptr(f), dptr(h)))
        else:
            check(_lib.load().ef_fv_map_d2n(*self._args(grid), dptr(g), dptr(f), dptr(h)))
        return h

    def particularNeumannData(self, grid: FiniteVolumeGrid, rhs_data) -> np.ndarray:
        return self.mapD2N(grid, np.zeros(2 * grid.nx() + 2 * grid.ny()), rhs_data)


class FiniteVolumePatch:
    """FiniteVolumePatch (FiniteVolumePatch.hpp:19-73); leaf data are views of the solver's arrays."""

    def __init__(self, grid: Optional[FiniteVolumeGrid] = None):
        self._grid = grid
        self.n_coarsens = 0
        self.u = np.zeros(0)
        self.f = np.zeros(0)
        self.g = np.zeros(0)
        self.h = np.zeros(0)

    def name(self): return "FiniteVolumePatch"
    def grid(self) -> FiniteVolumeGrid: return self._grid
    def vectorU(self): return self.u
    def vectorF(self): return self.f
    def vectorG(self): return self.g
    def vectorH(self): return self.h

    def size(self) -> int:
        return int(self._grid.nx() / 2 ** self.n_coarsens)


class FiniteVolumeNodeFactory:
    """FiniteVolumeNodeFactory: the child geometry is computed inside the library
    (midpoint halving, FiniteVolumeNodeFactory.cpp:15-66)."""


def _vtk_array(fh, vtype, name, comps, values):
    v = np.asarray(values)
    lo, hi = (float(v.min()), float(v.max())) if v.size else (0.0, 0.0)
    fh.write(f'        <DataArray type="{vtype}" Name="{name}" NumberOfComponents="{comps}" format="ascii" '
             f'RangeMin="{lo!r}" RangeMax="{hi!r}">\n')
    fh.write(" ".join(repr(float(x)) if vtype.startswith("Float") else str(int(x)) for x in v.ravel()))
    fh.write("\n        </DataArray>\n")


def _write_quad_vtu(filename, corners, funcs):
    """VTK XML unstructured grid of quads; corners [ncells, 8] = (x, y) of 4 corners per cell."""
    nc = corners.shape[0]
    pts = np.zeros((4 * nc, 3))
    pts[:, :2] = corners.reshape(4 * nc, 2)
    with open(filename, "w") as fh:
        fh.write('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n'
                 f'  <UnstructuredGrid>\n    <Piece NumberOfPoints="{4 * nc}" NumberOfCells="{nc}">\n      <Points>\n')
        _vtk_array(fh, "Float64", "Points", 3, pts)
        fh.write("      </Points>\n      <Cells>\n")
        _vtk_array(fh, "Int64", "connectivity", 1, np.arange(4 * nc))
        _vtk_array(fh, "Int64", "offsets", 1, 4 * np.arange(1, nc + 1))
        _vtk_array(fh, "UInt8", "types", 1, np.full(nc, 9))
        fh.write("      </Cells>\n      <CellData>\n")
        for name, v in funcs:
            if v.size != nc:
                raise ValueError(f"toVTK: cell data {name!r} has {v.size} values for {nc} cells")
            _vtk_array(fh, "Float64", name, 1, v)
        fh.write("      </CellData>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n")


def _write_pvtu(filename, piece, funcs):
    with open(filename, "w") as fh:
        fh.write('<?xml version="1.0"?>\n<VTKFile type="PUnstructuredGrid" version="0.1" byte_order="LittleEndian">\n'
                 '  <PUnstructuredGrid GhostLevel="0">\n    <PPoints>\n'
                 '      <PDataArray type="Float64" Name="Points" NumberOfComponents="3"/>\n    </PPoints>\n'
                 '    <PCellData>\n')
        for name, _ in funcs:
            fh.write(f'      <PDataArray type="Float64" Name="{name}" NumberOfComponents="1"/>\n')
        fh.write(f'    </PCellData>\n    <Piece Source="{piece}"/>\n  </PUnstructuredGrid>\n</VTKFile>\n')


class Mesh:
    """Mesh<FiniteVolumePatch> (Mesh.hpp) backed by the library's flat quadtree."""

    def __init__(self):
        self._h = None
        self.root_patch: Optional[FiniteVolumePatch] = None
        self.patches: list = []

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib._LIB is not None:
            _lib._LIB.ef_mesh_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def refineByFunction(self, fn: Callable[[float, float], bool], threshold: float, min_level: int,
                         max_level: int, root_patch: FiniteVolumePatch,
                         node_factory: Optional[FiniteVolumeNodeFactory] = None) -> "Mesh":
        lib = _lib.load()
        g = root_patch.grid()

        def tramp(x, y, _ctx):
            return 1 if fn(x, y) else 0
        cb = _lib.REFINE_FN(tramp)
        h = C.c_void_p()
        check(lib.ef_mesh_create_refined(g.xLower(), g.xUpper(), g.yLower(), g.yUpper(), g.nx(), g.ny(),
                                         int(min_level), int(max_level), cb, None, C.byref(h)))
        self._adopt(h, root_patch)
        return self

    def uniform(self, level: int, root_patch: FiniteVolumePatch) -> "Mesh":
        lib = _lib.load()
        g = root_patch.grid()
        h = C.c_void_p()
        check(lib.ef_mesh_create_uniform(g.xLower(), g.xUpper(), g.yLower(), g.yUpper(), g.nx(), g.ny(),
                                         int(level), C.byref(h)))
        self._adopt(h, root_patch)
        return self

    def _adopt(self, h, root_patch):
        if self._h is not None:
            _lib.load().ef_mesh_destroy(self._h)
        self._h = h
        self.root_patch = root_patch
        n = root_patch.grid().nx()
        self.patches = []
        for k in range(self.num_leaves()):
            lvl, _, _, box = self.leaf(k)
            self.patches.append(FiniteVolumePatch(FiniteVolumeGrid(n, box[0], box[1], n, box[2], box[3])))

    def num_leaves(self) -> int:
        v = C.c_int()
        check(_lib.load().ef_mesh_num_leaves(self._h, C.byref(v)))
        return v.value

    # -- subtree split (no reference counterpart in this form; see subtree.py) -------------------
    def level_count(self, level: int) -> int:
        """Number of tree nodes at `level`."""
        v = C.c_int()
        check(_lib.load().ef_mesh_level_count(self._h, int(level), C.byref(v)))
        return v.value

    def subtree(self, level: int, index: int) -> "Mesh":
        """The mesh of the subtree under the index-th node of `level` (z-order): its root patch is that
        node's patch and every leaf patch box is this mesh's, bit for bit."""
        h = C.c_void_p()
        check(_lib.load().ef_mesh_subtree(self._h, int(level), int(index), C.byref(h)))
        sub = Mesh()
        sub._h = h
        n = self.root_patch.grid().nx()
        boxes = np.array([sub.leaf(k)[3] for k in range(sub.num_leaves())])
        sub.root_patch = FiniteVolumePatch(FiniteVolumeGrid(n, boxes[:, 0].min(), boxes[:, 1].max(), n,
                                                            boxes[:, 2].min(), boxes[:, 3].max()))
        sub.patches = [FiniteVolumePatch(FiniteVolumeGrid(n, b[0], b[1], n, b[2], b[3])) for b in boxes]
        return sub

    # -- VTK output (Mesh.hpp:357-424) -------------------------------------------------------------
    def addMeshFunction(self, values, name: Optional[str] = None):
        """Cell data for toVTK: an array in leaf order (cell j + i*n, e.g. HPSAlgorithm.leaf_solution())
        or a vectorised f(x, y) sampled at the leaf cell centres."""
        if not hasattr(self, "_mesh_functions"):
            self._mesh_functions = []
        if callable(values):
            X, Y = self.cell_centres()
            values = values(X, Y)
        v = np.ascontiguousarray(values, dtype=np.float64).ravel()
        self._mesh_functions.append((name or f"mesh_function_{len(self._mesh_functions)}", v))

    def clearMeshFunctions(self):
        self._mesh_functions = []

    def toVTK(self, baseFilename: str, number: int = -1):
        """<base>-mesh[-NNNN].pvtu + -0.vtu (one quad per leaf cell, mesh functions as cell data) and
        <base>-quadtree[-NNNN].vtu (one quad per leaf patch with its level), VTK XML, ASCII."""
        tag = "" if number == -1 else f"-{number:04d}"
        n = self.root_patch.grid().nx()
        corners, boxes, levels = [], [], []
        for k, p in enumerate(self.patches):
            g = p.grid()
            x0 = g.xLower() + np.arange(n) * g.dx()
            y0 = g.yLower() + np.arange(n) * g.dy()
            X0, Y0 = np.meshgrid(x0, y0, indexing="ij")
            X0, Y0 = X0.ravel(), Y0.ravel()
            corners.append(np.stack([X0, Y0, X0 + g.dx(), Y0, X0 + g.dx(), Y0 + g.dy(), X0, Y0 + g.dy()], axis=1))
            boxes.append([g.xLower(), g.yLower(), g.xUpper(), g.yLower(), g.xUpper(), g.yUpper(), g.xLower(), g.yUpper()])
            levels.append(self.leaf(k)[0])
        funcs = getattr(self, "_mesh_functions", [])
        mesh = f"{baseFilename}-mesh{tag}"
        _write_quad_vtu(mesh + "-0.vtu", np.concatenate(corners), funcs)
        _write_pvtu(mesh + ".pvtu", os.path.basename(mesh) + "-0.vtu", funcs)
        nl = len(self.patches)
        _write_quad_vtu(f"{baseFilename}-quadtree{tag}.vtu", np.array(boxes, dtype=np.float64).reshape(nl, 8),
                        [("level", np.array(levels, dtype=np.float64)), ("leaf", np.arange(nl, dtype=np.float64))])

    def num_nodes(self) -> int:
        v = C.c_int()
        check(_lib.load().ef_mesh_num_nodes(self._h, C.byref(v)))
        return v.value

    def leaf(self, k: int):
        lvl = C.c_int()
        ix = C.c_longlong()
        iy = C.c_longlong()
        box = np.zeros(4)
        check(_lib.load().ef_mesh_leaf(self._h, k, C.byref(lvl), C.byref(ix), C.byref(iy), dptr(box)))
        return lvl.value, ix.value, iy.value, box

    def leaf_quads(self):
        return [self.leaf(k)[:3] for k in range(self.num_leaves())]

    def iteratePatches(self, fn):
        for p in self.patches:
            fn(p)

    def cell_centres(self):
        """Leaf cell centres (x, y) in leaf order, cell j + i*n (HPSAlgorithm.hpp:241-249)."""
        n = self.root_patch.grid().nx()
        xs, ys = [], []
        for p in self.patches:
            g = p.grid()
            X, Y = np.meshgrid(g.point(0, np.arange(n)), g.point(1, np.arange(n)), indexing="ij")
            xs.append(X.ravel())
            ys.append(Y.ravel())
        return np.concatenate(xs), np.concatenate(ys)


def kernel_launches() -> int:
    v = C.c_longlong()
    check(_lib.load().ef_kernel_launches(C.byref(v)))
    return v.value


class HPSAlgorithm:
    """HPSAlgorithm<FiniteVolumeGrid, FiniteVolumeSolver, FiniteVolumePatch, double> on one GPU."""

    def __init__(self, mesh: Mesh, patch_solver: FiniteVolumeSolver, options: Optional[dict] = None):
        self.mesh = mesh
        self.patch_solver = patch_solver
        self.options = {"cache-operators": False, "homogeneous-rhs": False}
        if options:
            self.options.update(options)
        lib = _lib.load()
        h = C.c_void_p()
        check(lib.ef_hps_create(mesh.handle, _solver_code(patch_solver.solver_type),
                                float(patch_solver.lambda_function(0, 0)), C.byref(h)))
        self._h = h
        nl, n, M, nb = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        check(lib.ef_hps_info(h, C.byref(nl), C.byref(n), C.byref(M), C.byref(nb)))
        self.num_leaves, self.n, self.M, self.device_bytes = nl.value, n.value, M.value, nb.value
        self._apply_options()
        if patch_solver.solver_type == FivePointStencil:
            self._set_coefficients()

    def save(self, path: str):
        """Solve-time operators of the built tree and its mesh to `path` (no reference counterpart)."""
        check(_lib.load().ef_hps_save(self._h, str(path).encode()))

    @classmethod
    def load(cls, path: str) -> "HPSAlgorithm":
        """A built tree saved by save(): its mesh and a handle that solves without re-merging."""
        lib = _lib.load()
        mh, hh = C.c_void_p(), C.c_void_p()
        check(lib.ef_hps_load(str(path).encode(), C.byref(mh), C.byref(hh)))
        self = cls.__new__(cls)
        self._h = hh
        nl, n, M, nb = C.c_int(), C.c_int(), C.c_int(), C.c_longlong()
        check(lib.ef_hps_info(hh, C.byref(nl), C.byref(n), C.byref(M), C.byref(nb)))
        self.num_leaves, self.n, self.M, self.device_bytes = nl.value, n.value, M.value, nb.value
        mesh = Mesh()
        mesh._h = mh
        boxes = []
        for k in range(nl.value):
            boxes.append(mesh.leaf(k)[3])
        bx = np.array(boxes)
        mesh.root_patch = FiniteVolumePatch(FiniteVolumeGrid(n.value, bx[:, 0].min(), bx[:, 1].max(), n.value,
                                                             bx[:, 2].min(), bx[:, 3].max()))
        mesh.patches = [FiniteVolumePatch(FiniteVolumeGrid(n.value, b[0], b[1], n.value, b[2], b[3])) for b in boxes]
        self.mesh = mesh
        self.patch_solver = FiniteVolumeSolver(solver_type=FISHPACK90)
        self.options = {"cache-operators": False, "homogeneous-rhs": False}
        self._apply_options()
        return self

    def _set_coefficients(self):
        """Samples alpha, beta, lambda on every leaf (FiniteVolumeSolver.cpp:66-79) into the library."""
        parts = [sample_coefficients(self.patch_solver, p.grid()) for p in self.mesh.patches]
        a = np.ascontiguousarray(np.concatenate([p[0] for p in parts]))
        b = np.ascontiguousarray(np.concatenate([p[1] for p in parts]))
        l = np.ascontiguousarray(np.concatenate([p[2] for p in parts]))
        check(_lib.load().ef_hps_set_coefficients(self._h, dptr(a), dptr(b), dptr(l)))

    def __del__(self):
        if getattr(self, "_h", None) is not None and _lib._LIB is not None:
            _lib._LIB.ef_hps_destroy(self._h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def _apply_options(self):
        lib = _lib.load()
        for k in ("cache-operators", "homogeneous-rhs"):
            v = self.options[k]
            if not isinstance(v, bool):
                raise TypeError(f"option {k!r} must be a bool")  # std::get<bool> in the reference
            check(lib.ef_hps_set_option(self._h, k.encode(), int(v)))

    def set_stream(self, cuda_stream_ptr: int):
        check(_lib.load().ef_hps_set_stream(self._h, C.c_void_p(cuda_stream_ptr)))

    @property
    def root_factorizations(self) -> int:
        """LU factorisations of the general root matrix so far (reused while a and b are unchanged)."""
        v = C.c_longlong()
        check(_lib.load().ef_hps_root_factorizations(self._h, C.byref(v)))
        return v.value

    def set_graphs(self, on: bool):
        """CUDA-graph replay of the device-resident solve sequences (default on)."""
        check(_lib.load().ef_hps_set_option(self._h, b"cuda-graphs", int(bool(on))))

    # -- stages --------------------------------------------------------------------------------
    def setupStage(self):
        check(_lib.load().ef_hps_setup(self._h))

    def buildStage(self):
        self._apply_options()
        check(_lib.load().ef_hps_build(self._h))

    def build_info(self):
        """(kernels launched by the merges of the last build, builds replayed from a CUDA graph)"""
        a, b = C.c_longlong(), C.c_longlong()
        check(_lib.load().ef_hps_build_info(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def buildStageFrom(self, old: "HPSAlgorithm") -> int:
        """Build reusing the merges of `old` (a built tree on another mesh of the same domain) whose
        subtrees are unchanged; returns the number of reused merges (no reference counterpart)."""
        self._apply_options()
        n = C.c_int()
        check(_lib.load().ef_hps_build_from(self._h, old._h, C.byref(n)))
        return n.value

    # -- top of a subtree split (no reference counterpart in this form; see subtree.py) ----------
    def split_sizes(self, level: int):
        """4m per node of `level` (z-order): the length of its h and g; its T is 4m x 4m."""
        cnt = self.mesh.level_count(level)
        v = (C.c_int * cnt)()
        check(_lib.load().ef_hps_split_sizes(self._h, int(level), v))
        return list(v)

    def buildStageTop(self, level: int, T_blocks):
        """Merges of levels level-1 .. 0 from the root T of every level-`level` subtree."""
        self._apply_options()
        blocks = [np.ascontiguousarray(T, dtype=np.float64) for T in T_blocks]
        arr = (C.c_void_p * len(blocks))(*[b.ctypes.data for b in blocks])
        check(_lib.load().ef_hps_build_top(self._h, int(level), arr))

    def upwardsStageTop(self, level: int, h_blocks):
        """Upward pass of levels level-1 .. 0 from the root h of every level-`level` subtree."""
        blocks = [np.ascontiguousarray(h, dtype=np.float64) for h in h_blocks]
        arr = (C.c_void_p * len(blocks))(*[b.ctypes.data for b in blocks])
        check(_lib.load().ef_hps_upwards_top(self._h, int(level), arr))

    def solveStageTop(self, level: int, a, b, r):
        """Root data a u + b du/dn = r, downward pass to `level`: the Dirichlet data of every
        level-`level` subtree (list of arrays)."""
        a, b, r = (np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, r))
        gs = [np.empty(m) for m in self.split_sizes(level)]
        arr = (C.c_void_p * len(gs))(*[g.ctypes.data for g in gs])
        check(_lib.load().ef_hps_solve_top(self._h, int(level), dptr(a), dptr(b), dptr(r), arr))
        return gs

    def root_data(self, bc):
        """(a, b, r) of bc(side, x, y) -> (r, a, b) at the root face centres (HPSAlgorithm.hpp:375-400)."""
        rs, as_, bs = [], [], []
        for side, (x, y) in enumerate(self.boundary_points()):
            r, a, b = bc(side, x, y)
            rs.append(np.broadcast_to(np.asarray(r, dtype=np.float64), x.shape))
            as_.append(np.broadcast_to(np.asarray(a, dtype=np.float64), x.shape))
            bs.append(np.broadcast_to(np.asarray(b, dtype=np.float64), x.shape))
        return np.concatenate(as_), np.concatenate(bs), np.concatenate(rs)

    def buildStageMixed(self, fp64_levels: int = 3):
        """Mixed-precision build (no counterpart in the reference): FP32 merges with the interface
        LU of the top `fp64_levels` levels in FP64; prepares the tree for mixed_* and Server only."""
        self._apply_options()
        check(_lib.load().ef_hps_build_mixed(self._h, int(fp64_levels)))

    def upwardsStage(self, rhs, vectorized: bool = True, patch_callback: bool = False):
        """``rhs`` is f(x, y) (sampled at leaf cell centres, HPSAlgorithm.hpp:241-249) or, with
        ``patch_callback=True``, a function that sets ``patch.f`` on each leaf patch."""
        self._apply_options()
        n = self.n
        if patch_callback:
            for p in self.mesh.patches:
                rhs(p)
            f = np.concatenate([np.asarray(p.f, dtype=np.float64).ravel() for p in self.mesh.patches])
        else:
            X, Y = self.mesh.cell_centres()
            if vectorized:
                f = np.asarray(rhs(X, Y), dtype=np.float64)
            else:
                f = np.array([rhs(x, y) for x, y in zip(X, Y)], dtype=np.float64)
            for k, p in enumerate(self.mesh.patches):
                p.f = f[k * n * n:(k + 1) * n * n]
        self.upwards_array(f)

    def upwards_array(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64)
        if f.size != self.num_leaves * self.n * self.n:
            raise ValueError("f has the wrong size")
        check(_lib.load().ef_hps_upwards(self._h, dptr(f)))

    def boundary_points(self):
        """Root face centres per side (HPSAlgorithm.hpp:375-400): lists of (x, y) arrays, WESN."""
        g = self.mesh.root_patch.grid()
        M = self.M
        dx = (g.xUpper() - g.xLower()) / M
        dy = (g.yUpper() - g.yLower()) / M
        xc = (g.xLower() + dx / 2) + np.arange(M) * dx
        yc = (g.yLower() + dy / 2) + np.arange(M) * dy
        return [(np.full(M, g.xLower()), yc), (np.full(M, g.xUpper()), yc),
                (xc, np.full(M, g.yLower())), (xc, np.full(M, g.yUpper()))]

    def solveStage(self, bc, vectorized: bool = True, patch_callback: bool = False):
        """``bc(side, x, y) -> (r, a, b)`` for a u + b du/dn = r on the root faces, or with
        ``patch_callback=True`` a function given the root patch that sets ``root.g``."""
        self._apply_options()
        lib = _lib.load()
        if patch_callback:
            root = FiniteVolumePatch(FiniteVolumeGrid(self.M, *self._root_box()))
            bc(root)
            g = np.ascontiguousarray(root.g, dtype=np.float64)
            if g.size != 4 * self.M:
                raise ValueError("root g has the wrong size")
            check(lib.ef_hps_solve_root_dirichlet(self._h, dptr(g)))
        else:
            r, a, b = [], [], []
            for side, (x, y) in enumerate(self.boundary_points()):
                if vectorized:
                    rv, av, bv = bc(side, x, y)
                    rv = np.broadcast_to(np.asarray(rv, dtype=np.float64), x.shape)
                    av = np.broadcast_to(np.asarray(av, dtype=np.float64), x.shape)
                    bv = np.broadcast_to(np.asarray(bv, dtype=np.float64), x.shape)
                else:
                    vals = [bc(side, xi, yi) for xi, yi in zip(x, y)]
                    rv, av, bv = (np.array([v[k] for v in vals]) for k in range(3))
                r.append(rv); a.append(av); b.append(bv)
            self.solve_arrays(np.concatenate(a), np.concatenate(b), np.concatenate(r))
        u = self.leaf_solution()
        n2 = self.n * self.n
        for k, p in enumerate(self.mesh.patches):
            p.u = u[k * n2:(k + 1) * n2]

    def solve_arrays(self, a, b, r):
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        if not (a.size == b.size == r.size == 4 * self.M):
            raise ValueError("boundary data must have 4*M entries")
        check(_lib.load().ef_hps_solve(self._h, dptr(a), dptr(b), dptr(r)))

    def _root_box(self):
        g = self.mesh.root_patch.grid()
        return g.xLower(), g.xUpper(), self.M, g.yLower(), g.yUpper()

    # -- results ---------------------------------------------------------------------------------
    def leaf_solution(self) -> np.ndarray:
        u = np.empty(self.num_leaves * self.n * self.n)
        check(_lib.load().ef_hps_get_leaf_u(self._h, dptr(u)))
        return u

    def root_T(self) -> np.ndarray:
        m = 4 * self.M
        T = np.empty((m, m))
        check(_lib.load().ef_hps_get_root_T(self._h, dptr(T)))
        return T

    def root_h(self) -> np.ndarray:
        h = np.empty(4 * self.M)
        check(_lib.load().ef_hps_get_root_h(self._h, dptr(h)))
        return h

    def device_buffers(self):
        ptrs = [C.c_void_p() for _ in range(5)]
        check(_lib.load().ef_hps_device_buffers(self._h, *[C.byref(p) for p in ptrs]))
        return [p.value for p in ptrs]  # f, u, a, b, r

    # -- mixed precision, many right-hand sides (no counterpart in the reference) ----------------
    def mixed_init(self, bmax: int):
        """FP32 operator copies for batches of up to bmax requests (after buildStage)."""
        check(_lib.load().ef_hps_mixed_init(self._h, int(bmax)))
        self.mixed_bmax = int(bmax)

    def mixed_gemm_plan(self):
        """[(level, s, code W, code H, code DOWN)] of the tuned node GEMMs: code > 0 CUDA-core kernel
        with that K split, code < 0 tensor-core kernel with K split -code."""
        n = C.c_int()
        check(_lib.load().ef_hps_mixed_gemm_plan(self._h, 0, None, C.byref(n)))
        t = (C.c_int * (5 * n.value))()
        check(_lib.load().ef_hps_mixed_gemm_plan(self._h, n.value, t, C.byref(n)))
        return [tuple(t[5 * i:5 * i + 5]) for i in range(n.value)]

    def mixed_set_gemm_plan(self, plan):
        """Use `plan` (rows (level, s, W, H, DOWN) as mixed_gemm_plan returns them, or rows of the
        three codes) for the block solvers created afterwards instead of timing the candidates."""
        rows = [tuple(r)[-3:] for r in plan]
        codes = (C.c_int * (3 * len(rows)))(*[int(c) for r in rows for c in r])
        check(_lib.load().ef_hps_mixed_set_gemm_plan(self._h, codes, len(rows)))

    def mixed_set_root(self, a, b):
        """Fixed root operator a u + b du/dn = r of the block solver (r per request); b = 0 returns
        to per-request Dirichlet data (no reference counterpart: the reference solves one request)."""
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        if a.shape != (4 * self.M,) or b.shape != (4 * self.M,):
            raise ValueError("mixed_set_root: a and b must have 4M entries")
        check(_lib.load().ef_hps_mixed_set_root(self._h, dptr(a), dptr(b)))

    def mixed_solve(self, f, a, r, sweeps: int = 1) -> np.ndarray:
        """Solve a block of requests: f [B, leaves*n*n], a and r [B, 4M] (a u = r on the root
        faces).  Returns u [B, leaves*n*n] refined to the FP64 HPS solution."""
        f = np.ascontiguousarray(np.atleast_2d(f), dtype=np.float64)
        a = np.ascontiguousarray(np.atleast_2d(a), dtype=np.float64)
        r = np.ascontiguousarray(np.atleast_2d(r), dtype=np.float64)
        B = f.shape[0]
        if f.shape[1] != self.num_leaves * self.n * self.n or a.shape != (B, 4 * self.M) or r.shape != (B, 4 * self.M):
            raise ValueError("mixed_solve: bad shapes")
        u = np.empty_like(f)
        check(_lib.load().ef_hps_mixed_solve(self._h, B, int(sweeps), dptr(f), dptr(a), dptr(r), dptr(u)))
        return u

    def mixed_solve_blocks(self, blocks, sweeps: int = 1, out=None):
        """Pipelined form of mixed_solve for many blocks: blocks is a sequence of (f, a, r) arrays
        shaped as for mixed_solve (each block at most mixed_bmax requests); the blocks rotate over
        three lanes so that host copies overlap the solves.  Returns (or fills) one u array per
        block.  Page-locked arrays keep the copies asynchronous."""
        blocks = [tuple(np.ascontiguousarray(np.atleast_2d(x), dtype=np.float64) for x in blk) for blk in blocks]
        nb = len(blocks)
        for f, a, r in blocks:
            B = f.shape[0]
            if f.shape[1] != self.num_leaves * self.n * self.n or a.shape != (B, 4 * self.M) or r.shape != (B, 4 * self.M):
                raise ValueError("mixed_solve_blocks: bad shapes")
        us = out if out is not None else [np.empty_like(f) for f, _, _ in blocks]
        batch = (C.c_int * nb)(*[f.shape[0] for f, _, _ in blocks])
        ptr = lambda xs: (C.c_void_p * nb)(*[x.ctypes.data for x in xs])
        check(_lib.load().ef_hps_mixed_solve_blocks(self._h, nb, batch, int(sweeps), ptr([b[0] for b in blocks]),
                                                    ptr([b[1] for b in blocks]), ptr([b[2] for b in blocks]),
                                                    ptr(us)))
        return us

    def mixed_residuals(self, passes: int) -> np.ndarray:
        out = np.empty((passes, self.mixed_bmax))
        check(_lib.load().ef_hps_mixed_residuals(self._h, int(passes), dptr(out)))
        return out

    def mixed_buffers(self):
        ptrs = [C.c_void_p() for _ in range(4)]
        check(_lib.load().ef_hps_mixed_buffers(self._h, *[C.byref(p) for p in ptrs]))
        return [p.value for p in ptrs]  # f, a, r, u

    def mixed_solve_async(self, batch: int, sweeps: int = 1, lane: int = 0):
        if lane == 0:
            check(_lib.load().ef_hps_mixed_solve_async(self._h, int(batch), int(sweeps)))
        else:
            check(_lib.load().ef_hps_mixed_lane_solve_async(self._h, int(lane), int(batch), int(sweeps)))

    def mixed_lane(self, lane: int):
        """Device pointers (f, a, r, u) and the CUDA stream (int) of lane 0..3; lanes >= 1 share the
        FP32 operators and are created by the first call for them."""
        ptrs = [C.c_void_p() for _ in range(5)]
        check(_lib.load().ef_hps_mixed_lane(self._h, int(lane), *[C.byref(p) for p in ptrs]))
        return [p.value or 0 for p in ptrs]

    def profile_enable(self, on: bool = True):
        check(_lib.load().ef_hps_profile_enable(self._h, int(on)))

    def profile_reset(self):
        check(_lib.load().ef_hps_profile_reset(self._h))

    def profile(self) -> dict:
        """{section: {ms, launches, calls, bytes, flops}} accumulated since the last reset."""
        lib = _lib.load()
        n = C.c_int()
        check(lib.ef_hps_profile_count(self._h, C.byref(n)))
        out = {}
        for i in range(n.value):
            name = C.create_string_buffer(64)
            ms, by, fl = C.c_double(), C.c_double(), C.c_double()
            la, ca = C.c_longlong(), C.c_longlong()
            check(lib.ef_hps_profile_entry(self._h, i, name, 64, C.byref(ms), C.byref(la), C.byref(ca),
                                           C.byref(by), C.byref(fl)))
            out[name.value.decode()] = {"ms": ms.value, "launches": la.value, "calls": ca.value,
                                        "bytes": by.value, "flops": fl.value}
        return out

    def load_device_async(self, f_ptr=None, a_ptr=None, b_ptr=None, r_ptr=None):
        """Device-to-device copy of new inputs (raw device pointers) into the resident buffers."""
        v = lambda p: C.c_void_p(p) if p else None
        check(_lib.load().ef_hps_load_device_async(self._h, v(f_ptr), v(a_ptr), v(b_ptr), v(r_ptr)))

    def solve_device_async(self, b_is_zero: bool = True):
        check(_lib.load().ef_hps_solve_device_async(self._h, int(bool(b_is_zero))))

    def synchronize(self):
        check(_lib.load().ef_hps_synchronize(self._h))


class Server:
    """Serving loop over several built trees (no counterpart in the reference).

    Requests (tree index, load f, root data a u = r) are answered by the batched mixed-precision
    solver; the scheduler thread of the library forms a block from every request of a tree that has
    arrived whenever one of the tree's lanes is free, and overlaps blocks of different lanes and trees
    on the GPU.  Lanes beyond the first per tree are created only while the device memory of all
    lanes fits hbm_budget_bytes (0: no limit).  sweeps: refinement sweeps per block, one value
    for every tree or one per tree."""

    def __init__(self, trees, bmax, lanes: int = 2, hbm_budget_bytes: int = 0, sweeps=1):
        trees = list(trees)
        bmax = [int(b) for b in (bmax if hasattr(bmax, "__len__") else [bmax] * len(trees))]
        if len(bmax) != len(trees):
            raise ValueError("Server: one bmax per tree")
        self._trees = trees
        lib = _lib.load()
        arr = (C.c_void_p * len(trees))(*[t.handle for t in trees])
        bm = (C.c_int * len(trees))(*bmax)
        h = C.c_void_p()
        sw = [int(x) for x in (sweeps if hasattr(sweeps, "__len__") else [sweeps] * len(trees))]
        if len(sw) != len(trees):
            raise ValueError("Server: one sweeps value per tree")
        check(lib.ef_server_create(arr, bm, len(trees), int(lanes), int(hbm_budget_bytes), sw[0], C.byref(h)))
        self._h = h
        for t, x in enumerate(sw):
            self.set_sweeps(t, x)
        self._live = {}  # id -> arrays kept alive until completion

    def set_root(self, tree: int, a, b) -> None:
        """Root operator a u + b du/dn = r of the tree's later requests (see HPSAlgorithm.mixed_set_root);
        the tree must have no request in flight."""
        t = self._trees[tree]
        a = np.ascontiguousarray(a, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        if a.shape != (4 * t.M,) or b.shape != (4 * t.M,):
            raise ValueError("Server.set_root: a and b must have 4M entries")
        check(_lib.load().ef_server_set_root(self._h, int(tree), dptr(a), dptr(b)))

    def set_sweeps(self, tree: int, sweeps: int) -> None:
        """Refinement sweeps of the tree's blocks from the next block on."""
        check(_lib.load().ef_server_set_sweeps(self._h, int(tree), int(sweeps)))

    def lanes(self, tree: int) -> int:
        n = C.c_int()
        check(_lib.load().ef_server_info(self._h, int(tree), C.byref(n), None))
        return n.value

    def device_bytes(self) -> int:
        b = C.c_longlong()
        check(_lib.load().ef_server_info(self._h, 0, None, C.byref(b)))
        return b.value

    def submit(self, tree: int, f, a, r, out=None) -> int:
        """Queue one request; returns its id.  `out` (optional, float64 [leaves*n*n]) receives u;
        page-locked arrays keep the copies asynchronous."""
        t = self._trees[tree]
        cells = t.num_leaves * t.n * t.n
        f = np.ascontiguousarray(f, dtype=np.float64)
        a = np.ascontiguousarray(a, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        if out is None:
            out = np.empty(cells)
        if f.size != cells or a.size != 4 * t.M or r.size != 4 * t.M or out.size != cells or out.dtype != np.float64:
            raise ValueError("Server.submit: bad shapes")
        rid = C.c_longlong()
        check(_lib.load().ef_server_submit(self._h, int(tree), dptr(f), dptr(a), dptr(r), dptr(out), C.byref(rid)))
        self._live[rid.value] = (f, a, r, out)
        return rid.value

    def poll(self, rid: int):
        """(done, latency_s)"""
        d, lat = C.c_int(), C.c_double()
        check(_lib.load().ef_server_poll(self._h, int(rid), C.byref(d), C.byref(lat)))
        return bool(d.value), lat.value

    def wait(self, rid: int, timeout: float = 120.0):
        """(u, latency_s) of request rid; raises TimeoutError after `timeout` seconds."""
        d, lat = C.c_int(), C.c_double()
        check(_lib.load().ef_server_wait(self._h, int(rid), float(timeout), C.byref(d), C.byref(lat)))
        if not d.value:
            raise TimeoutError(f"request {rid} not done after {timeout} s")
        arrays = self._live.pop(rid)
        return arrays[3], lat.value

    def stats(self) -> dict:
        v = [C.c_longlong() for _ in range(4)]
        check(_lib.load().ef_server_stats(self._h, *[C.byref(x) for x in v]))
        return dict(zip(("submitted", "completed", "blocks", "max_block"), [x.value for x in v]))

    def close(self):
        if getattr(self, "_h", None):
            check(_lib.load().ef_server_destroy(self._h))
            self._h = None
            self._live.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
