"""Pins the CPU oracle (oracle/) to the reference's own known answers before anything is compared
against it: the patch-solver README error table, the Matrix/Grid unit-test values, the global
5-point system on uniform meshes, second-order convergence and the config-2 adaptive mesh."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import global_fv as G
from oracle import hps_oracle as O

GOLD = json.loads((Path(__file__).parent / "golden" / "reference_known_answers.json").read_text())


def u_exact(x, y):
    return np.sin(x) + np.sin(y)


def test_grid_points_known_answer():
    # test/test_finite_volume_grid.cpp:30-49
    gp = GOLD["grid_points"]
    g = O.FiniteVolumeGrid(gp["nx"], gp["x"][0], gp["x"][1], gp["ny"], gp["y"][0], gp["y"][1])
    for i, v in enumerate(gp["xpoints"]):
        assert abs(g.point(O.XDIM, i) - v) <= gp["tol"]
    for j, v in enumerate(gp["ypoints"]):
        assert abs(g.point(O.YDIM, j) - v) <= gp["tol"]


def test_matrix_linear_solve_known_answer():
    # test/test_matrix.cpp:155-192 (dgesv)
    d = GOLD["matrix_linear_solve"]
    A = np.array(d["A"]).reshape(3, 3)
    x = O.dgesv(A, np.array(d["b"]))
    np.testing.assert_allclose(x, d["x"], rtol=0, atol=d["tol_vec"])
    X = O.dgesv(A, np.array(d["B"]).reshape(3, 4))
    np.testing.assert_allclose(X, np.array(d["X"]).reshape(3, 4), rtol=0, atol=d["tol_mat"])


def test_block_permute_known_answer():
    # test/test_matrix.cpp:270-300
    d = GOLD["matrix_block_permute"]
    m1 = np.array(d["m1"]).reshape(d["shape"])
    m2 = O.block_permute(m1, d["pi_rows"], d["pi_cols"], d["R"], d["C"])
    np.testing.assert_array_equal(m2, np.array(d["expected"]).reshape(d["shape"]))


def _patch_error(n, stype):
    g = O.FiniteVolumeGrid(n, -1, 1, n, -1, 1)
    s = O.FiniteVolumeSolver(solver_type=stype)
    x, y = g.points(0), g.points(1)
    gv = np.concatenate([u_exact(-1, y), u_exact(1, y), u_exact(x, -1), u_exact(x, 1)])
    X, Y = np.meshgrid(x, y, indexing="ij")
    ue = u_exact(X, Y).ravel()
    u = s.solve(g, gv, -ue)
    return np.abs(u - ue).max()


@pytest.mark.parametrize("n", [8, 16, 32])
def test_patch_solver_readme_errors_dense(n):
    # examples/patch-solver/README.md:17-25, FivePointStencil dense LU
    ref = GOLD["patch_solver_readme"]["inf_errors"][str(n)]
    err = _patch_error(n, O.FIVE_POINT_STENCIL)
    assert abs(err - ref) <= 1e-8 * ref


@pytest.mark.parametrize("n", [64, 128, 256])
def test_patch_solver_readme_errors_global(n):
    # same table through the independent sparse global solve
    ref = GOLD["patch_solver_readme"]["inf_errors"][str(n)]
    U, x, y = G.solve_dirichlet(n, n, -1, 1, -1, 1, lambda X, Y: -u_exact(X, Y), u_exact)
    X, Y = np.meshgrid(x, y, indexing="ij")
    err = np.abs(U - u_exact(X, Y)).max()
    assert abs(err - ref) <= 1e-7 * ref


def test_fishpack_convergence_order():
    # test/test_finite_volume_solver.cpp:21-95: order > 1.95 between n = 256 and 512
    errs = []
    for n in (256, 512):
        U, x, y = G.solve_dirichlet(n, n, -1, 1, -1, 1, lambda X, Y: -u_exact(X, Y), u_exact)
        X, Y = np.meshgrid(x, y, indexing="ij")
        errs.append(np.abs(U - u_exact(X, Y)).max())
    order = math.log(errs[1] / errs[0]) / math.log(256 / 512)
    assert order > 1.95


def test_fishpack_and_five_point_agree():
    g = O.FiniteVolumeGrid(8, 0.0, 1.0, 8, -0.5, 0.5)
    rng = np.random.default_rng(1)
    gv, f = rng.standard_normal(32), rng.standard_normal(64)
    u1 = O.FiniteVolumeSolver(solver_type=O.FISHPACK90).solve(g, gv, f)
    u2 = O.FiniteVolumeSolver(solver_type=O.FIVE_POINT_STENCIL).solve(g, gv, f)
    np.testing.assert_allclose(u1, u2, rtol=1e-13, atol=1e-13)


def test_interpolation_operators():
    L21 = O.interpolation_fine2coarse(4)
    assert L21.shape == (4, 8) and np.allclose(L21.sum(1), 1)
    L12 = O.interpolation_coarse2fine(8)
    assert L12.shape == (8, 4)
    np.testing.assert_allclose(L12.sum(1), 1.0)          # preserves constants
    v = np.arange(4.0) * 0.3 + 1.0                      # linear data on coarse centres
    fine = L12 @ v
    xf = (np.arange(8) + 0.5) / 8
    np.testing.assert_allclose(fine, 1.0 + 0.3 * (xf * 4 - 0.5), atol=1e-14)  # exact for linears
    assert np.allclose(L21 @ L12, np.eye(4) + (L21 @ L12 - np.eye(4)))


def _run_uniform(L, n, dom, f, g):
    root = O.FiniteVolumePatch(O.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    mesh = O.Mesh().uniform(L, root)
    hps = O.HPSAlgorithm(mesh, O.FiniteVolumeSolver(solver_type=O.FISHPACK90))
    hps.buildStage()
    hps.upwardsStage(f)
    hps.solveStage(lambda s, x, y: (g(x, y), 1.0, 0.0))
    return mesh, hps


@pytest.mark.parametrize("L,n", [(1, 8), (2, 4), (3, 8)])
def test_uniform_hps_equals_global_five_point(L, n):
    dom = (-10.0, 10.0, -10.0, 10.0)
    f = lambda x, y: -u_exact(x, y)
    mesh, hps = _run_uniform(L, n, dom, f, u_exact)
    u = O.leaf_solution(hps)
    N = n * 2 ** L
    U, _, _ = G.solve_dirichlet(N, N, *dom, lambda X, Y: -u_exact(X, Y), u_exact)
    ug = G.to_leaf_order(U, L, n)
    assert np.abs(u - ug).max() <= 1e-12 * np.abs(ug).max()


@pytest.mark.parametrize("nx,ny,lam", [(64, 64, 0.0), (96, 48, -3.0)])
def test_sine_transform_direct_solve_equals_sparse_lu(nx, ny, lam):
    # the fast direct solve used at level 7 against the sparse LU of the same global system
    rng = np.random.default_rng(nx + ny)
    dom = (-1.0, 2.0, 0.5, 1.5)
    F = rng.standard_normal((nx, ny))
    gW, gE, gS, gN = rng.standard_normal(ny), rng.standard_normal(ny), rng.standard_normal(nx), rng.standard_normal(nx)
    U = G.solve_poisson_dst(F, gW, gE, gS, gN, *dom, lam=lam)
    A, cW, cE, cS, cN, x, y = G.assemble(nx, ny, *dom, lam=lambda X, Y: lam + 0.0 * X)
    R = F.copy()
    R[0, :] += -2.0 * cW[0, :] * gW
    R[-1, :] += -2.0 * cE[-1, :] * gE
    R[:, 0] += -2.0 * cS[:, 0] * gS
    R[:, -1] += -2.0 * cN[:, -1] * gN
    import scipy.sparse.linalg as spla
    Us = spla.spsolve(A.tocsc(), R.ravel())
    assert np.abs(U.ravel() - Us).max() <= 1e-12 * np.abs(Us).max()


def test_adaptive_hps_second_order():
    f = lambda x, y: -u_exact(x, y)
    errs = []
    for ml in (3, 4):
        root = O.FiniteVolumePatch(O.FiniteVolumeGrid(8, -10, 10, 8, -10, 10))
        mesh = O.Mesh().refineByFunction(lambda x, y: abs(f(x, y)) > 1.2, 1.2, 0, ml, root)
        hps = O.HPSAlgorithm(mesh, O.FiniteVolumeSolver(solver_type=O.FISHPACK90))
        hps.buildStage(); hps.upwardsStage(f)
        hps.solveStage(lambda s, x, y: (u_exact(x, y), 1.0, 0.0))
        X, Y = O.leaf_cell_centres(mesh)
        errs.append(np.abs(O.leaf_solution(hps) - u_exact(X, Y)).max())
    assert errs[1] < errs[0] / 1.5


def test_config2_adaptive_mesh_counts():
    # |-(sin x + sin y)| > 1.2 on [-10,10]^2, levels 0..7, 16x16 patches, corner balanced
    leaves = O.refine_leaves(lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2, -10, 10, -10, 10, 16, 16, 0, 7)
    levels = {}
    for l, _, _ in leaves:
        levels[l] = levels.get(l, 0) + 1
    assert len(leaves) == 7750
    assert levels == {5: 262, 6: 1568, 7: 5920}


def test_corner_balance_is_two_to_one():
    leaves = O.refine_leaves(lambda x, y: abs(x - 0.3) < 0.05 and abs(y + 0.2) < 0.05, 0, 1, 0, 1, 4, 4, 0, 7)
    ls = set(leaves)
    for (l, ix, iy) in leaves:
        n = 1 << l
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                jx, jy = ix + dx, iy + dy
                if (dx or dy) and 0 <= jx < n and 0 <= jy < n:
                    for lc in range(0, l - 1):
                        s = l - lc
                        assert (lc, jx >> s, jy >> s) not in ls
