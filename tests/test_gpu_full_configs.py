"""Parity at the full sizes of the adaptive and variable-coefficient workloads, and of one mixed block
on the uniform level-7 tree.

- Adaptive: refineByFunction(|sin x + sin y| > 1.2, min 0, max 7) on [-10, 10]^2 with 16 x 16
  leaves (7 750 leaves, 1 984 000 cells), Poisson with f = -(sin x + sin y) and Dirichlet data
  sin x + sin y.  The GPU leaf solution must match the HPS oracle (a restatement of
  HPSAlgorithm.hpp) to 1e-12 relative, and its discretisation error must be the oracle's.
- Variable coefficient: FivePointStencil, alpha = 1, beta = 1 + 0.5 sin(pi x) cos(pi y),
  lambda = -1 on [-1, 1]^2, uniform level 5 with 32 x 32 leaves (1024^2 cells), manufactured
  u = sin(2 pi x) sin(pi y).  On a uniform tree the HPS solution is the solution of the global
  cell-centred 5-point system (the leaf flux (2/d)(u - g) forces g = (u_L + u_R)/2 at every
  interface), so the GPU result is compared with a sparse direct solve of that system
  (oracle/global_fv.py) to 1e-11, its error against the manufactured solution with the direct
  solve's, and the leaf DtN maps of sample leaves with the oracle's buildD2N to 1e-12.
- Mixed block at level 7 (2048^2 cells, 16 x 16 leaves): one block of requests, one FP64
  refinement sweep, against a direct solve of the global system to 1e-10 per request (the sine
  transform that diagonalises the constant-coefficient system, pinned against a sparse LU in
  tests/test_oracle_pins.py; a sparse LU of 4.2 M unknowns takes minutes and ~6 GB).
"""
import numpy as np
import pytest

from oracle import global_fv as G
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-12
PI = np.pi


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


@pytest.fixture(scope="module")
def ef(lib):
    import ellipticforest_gb300
    return ellipticforest_gb300


# ------------------------------------------------------------------------------------------------
# adaptive, max level 7
# ------------------------------------------------------------------------------------------------
def test_adaptive_max_level_7_full_size_matches_oracle(ef):
    dom = (-10.0, 10.0, -10.0, 10.0)
    n = 16
    refine = lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2
    f = lambda x, y: -(np.sin(x) + np.sin(y))
    bc = lambda side, x, y: (np.sin(x) + np.sin(y), 1.0, 0.0)

    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    mesh = ef.Mesh().refineByFunction(refine, 0.0, 0, 7, root)
    assert mesh.num_leaves() == 7750
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.setupStage()
    hps.buildStage()
    hps.upwardsStage(f)
    hps.solveStage(bc)
    u = hps.leaf_solution()

    oroot = O.FiniteVolumePatch(O.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    om = O.Mesh().refineByFunction(refine, 0.0, 0, 7, oroot)
    oh = O.HPSAlgorithm(om, O.FiniteVolumeSolver(solver_type=O.FISHPACK90))
    oh.buildStage()
    oh.upwardsStage(f)
    oh.solveStage(lambda side, x, y: (np.sin(x) + np.sin(y), 1.0, 0.0))
    uo = O.leaf_solution(oh)

    assert u.size == uo.size == 7750 * 256
    assert rel(u, uo) <= REL
    X, Y = mesh.cell_centres()
    ue = np.sin(X) + np.sin(Y)
    err_gpu, err_orc = np.abs(u - ue).max(), np.abs(uo - ue).max()
    assert abs(err_gpu - err_orc) <= 1e-9 * err_orc   # discretisation error unchanged
    assert err_gpu < 1e-3


# ------------------------------------------------------------------------------------------------
# variable coefficient, uniform level 5, 32 x 32 leaves
# ------------------------------------------------------------------------------------------------
alpha3 = lambda x, y: 1.0 + 0.0 * x
beta3 = lambda x, y: 1.0 + 0.5 * np.sin(PI * x) * np.cos(PI * y)
lambda3 = lambda x, y: -1.0 + 0.0 * x


def u3(x, y):
    return np.sin(2 * PI * x) * np.sin(PI * y)


def f3(x, y):
    b = beta3(x, y)
    bx = 0.5 * PI * np.cos(PI * x) * np.cos(PI * y)
    by = -0.5 * PI * np.sin(PI * x) * np.sin(PI * y)
    ux = 2 * PI * np.cos(2 * PI * x) * np.sin(PI * y)
    uy = PI * np.sin(2 * PI * x) * np.cos(PI * y)
    return b * (-5 * PI ** 2) * u3(x, y) + bx * ux + by * uy - u3(x, y)


def test_variable_coefficient_L5_32_full_size_equals_global_solve(ef):
    dom = (-1.0, 1.0, -1.0, 1.0)
    n, L = 32, 5
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    mesh = ef.Mesh().uniform(L, root)
    solver = ef.FiniteVolumeSolver(alpha_function=alpha3, beta_function=beta3, lambda_function=lambda3,
                                   solver_type=ef.FivePointStencil)
    hps = ef.HPSAlgorithm(mesh, solver)
    hps.setupStage()
    hps.buildStage()
    hps.upwardsStage(f3)
    hps.solveStage(lambda side, x, y: (u3(x, y), 1.0, 0.0))
    u = hps.leaf_solution()

    N = n << L
    Ug, x, y = G.solve_dirichlet(N, N, *dom, f3, u3, alpha3, beta3, lambda3)
    us = G.to_leaf_order(Ug, L, n)
    assert u.size == us.size == N * N
    assert rel(u, us) <= 1e-11
    X, Y = mesh.cell_centres()
    ue = u3(X, Y)
    err_gpu, err_dir = np.abs(u - ue).max(), np.abs(us - ue).max()
    assert abs(err_gpu - err_dir) <= 1e-6 * err_dir   # discretisation error unchanged
    assert err_gpu < 1e-4

    # leaf DtN maps of sample leaves (corner, interior, far corner) against the oracle's buildD2N
    h = (dom[1] - dom[0]) / (1 << L)
    so = O.FiniteVolumeSolver(alpha_function=alpha3, beta_function=beta3, lambda_function=lambda3,
                              solver_type=O.FIVE_POINT_STENCIL)
    for ix, iy in ((0, 0), (13, 21), (31, 31)):
        box = (dom[0] + ix * h, dom[0] + (ix + 1) * h, dom[2] + iy * h, dom[2] + (iy + 1) * h)
        T = solver.buildD2N(ef.FiniteVolumeGrid(n, box[0], box[1], n, box[2], box[3]))
        To = so.buildD2N(O.FiniteVolumeGrid(n, box[0], box[1], n, box[2], box[3]))
        assert rel(T, To) <= REL, (ix, iy)


# ------------------------------------------------------------------------------------------------
# one mixed block on the uniform level-7 tree against the global direct solve
# ------------------------------------------------------------------------------------------------
def _requests(mesh, pts, B, seed):
    rng = np.random.default_rng(seed)
    X, Y = mesh.cell_centres()
    F, R = [], []
    for _ in range(B):
        amp, cx, cy, wd = rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(0.05, 0.3, 8)
        F.append(sum(amp[k] * np.exp(-((X - cx[k]) ** 2 + (Y - cy[k]) ** 2) / wd[k] ** 2) for k in range(8)))
        co = rng.standard_normal((4, 6))
        R.append(np.concatenate([sum(co[s, m] * np.sin((m + 1) * PI * ((yy if s < 2 else xx) + 1) / 2)
                                     for m in range(6)) for s, (xx, yy) in enumerate(pts)]))
    return np.array(F), np.array(R)


def test_mixed_block_L7_one_sweep_matches_global_direct_solve(ef):
    dom = (-1.0, 1.0, -1.0, 1.0)
    n, L, B = 16, 7, 8
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    mesh = ef.Mesh().uniform(L, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    pts = hps.boundary_points()
    F, R = _requests(mesh, pts, B, 2024)
    A = np.ones_like(R)
    hps.mixed_init(B)
    U = hps.mixed_solve(F, A, R, sweeps=1)

    N = n << L
    Ag, cW, cE, cS, cN, x, y = G.assemble(N, N, *dom)
    order = G.to_leaf_order(np.arange(N * N, dtype=float).reshape(N, N), L, n).astype(np.int64)
    M = N  # boundary points per side, in the order W, E, S, N
    for k in range(B):
        Fg = np.empty(N * N)
        Fg[order] = F[k]
        Fg = Fg.reshape(N, N)
        gW, gE, gS, gN = (R[k][s * M:(s + 1) * M] for s in range(4))
        ud = G.solve_poisson_dst(Fg, gW, gE, gS, gN, *dom).ravel()
        # the direct solve satisfies the global system (the same one the sparse LU solves)
        Rg = Fg.copy()
        Rg[0, :] += -2.0 * cW[0, :] * gW
        Rg[-1, :] += -2.0 * cE[-1, :] * gE
        Rg[:, 0] += -2.0 * cS[:, 0] * gS
        Rg[:, -1] += -2.0 * cN[:, -1] * gN
        assert np.abs(Ag @ ud - Rg.ravel()).max() <= 1e-9 * np.abs(Rg).max()
        err = rel(U[k], ud[order])
        assert err <= 1e-10, (k, err)
