"""GPU parity: the CUDA HPS path (through the C ABI) against the FP64 CPU oracle.

Tolerance: the plain FP64 GPU form must match the oracle's leaf solutions to 1e-12 relative
(max |u_gpu - u_oracle| / max |u_oracle|); DtN matrices likewise to 1e-12 relative.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import global_fv as G
from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-12
GOLD = json.loads((Path(__file__).parent / "golden" / "reference_known_answers.json").read_text())


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


def u_exact(x, y):
    return np.sin(x) + np.sin(y)


@pytest.fixture(scope="module")
def ef(lib):
    import ellipticforest_gb300
    return ellipticforest_gb300


# ------------------------------------------------------------------------------------------------
# single patch: FiniteVolumeSolver::buildD2N / solve / mapD2N
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("n,box,lam", [(4, (0, 1, 0, 1), 0.0), (8, (-1, 1, -1, 1), 0.0),
                                       (16, (-10, -7.5, 2.5, 5.0), 0.0), (16, (0, 2, 0, 1), -1.0),
                                       (32, (-1, 1, -1, 1), -3.0)])
def test_build_d2n_matches_oracle(ef, n, box, lam):
    gg = ef.FiniteVolumeGrid(n, box[0], box[1], n, box[2], box[3])
    s = ef.FiniteVolumeSolver(lambda_function=lambda x, y: lam, solver_type=ef.FISHPACK90)
    T = s.buildD2N(gg)
    og = O.FiniteVolumeGrid(n, box[0], box[1], n, box[2], box[3])
    To = O.FiniteVolumeSolver(solver_type=O.FISHPACK90, lambda_function=lambda x, y: lam).buildD2N(og)
    assert rel(T, To) <= REL


@pytest.mark.parametrize("n", [4, 8, 16, 32])
def test_patch_solve_and_map_d2n_match_oracle(ef, n):
    rng = np.random.default_rng(n)
    g, f = rng.standard_normal(4 * n), rng.standard_normal(n * n)
    gg = ef.FiniteVolumeGrid(n, -1, 2, n, 0, 3)
    og = O.FiniteVolumeGrid(n, -1, 2, n, 0, 3)
    s = ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90)
    so = O.FiniteVolumeSolver(solver_type=O.FISHPACK90)
    assert rel(s.solve(gg, g, f), so.solve(og, g, f)) <= REL
    assert rel(s.mapD2N(gg, g, f), so.mapD2N(og, g, f)) <= REL
    assert rel(s.particularNeumannData(gg, f), so.particularNeumannData(og, f)) <= REL


@pytest.mark.parametrize("n", [8, 16, 32, 64])
def test_patch_solver_readme_error_table(ef, n):
    # examples/patch-solver/README.md:17-25 reproduced by the GPU leaf solver
    ref = GOLD["patch_solver_readme"]["inf_errors"][str(n)]
    gg = ef.FiniteVolumeGrid(n, -1, 1, n, -1, 1)
    x, y = gg(0, np.arange(n)), gg(1, np.arange(n))
    g = np.concatenate([u_exact(-1, y), u_exact(1, y), u_exact(x, -1), u_exact(x, 1)])
    X, Y = np.meshgrid(x, y, indexing="ij")
    ue = u_exact(X, Y).ravel()
    u = ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90).solve(gg, g, -ue)
    err = np.abs(u - ue).max()
    assert abs(err - ref) <= 1e-8 * ref


# ------------------------------------------------------------------------------------------------
# whole HPS path
# ------------------------------------------------------------------------------------------------
def run_gpu(ef, mesh_kind, n, dom, f, bc, options=None, lam=0.0, patch_g=None):
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    if mesh_kind[0] == "uniform":
        mesh = ef.Mesh().uniform(mesh_kind[1], root)
    else:
        mesh = ef.Mesh().refineByFunction(mesh_kind[1], 0.0, mesh_kind[2], mesh_kind[3], root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(lambda_function=lambda x, y: lam, solver_type=ef.FISHPACK90), options)
    hps.setupStage()
    hps.buildStage()
    hps.upwardsStage(f)
    if patch_g is not None:
        hps.solveStage(lambda root: setattr(root, "g", patch_g(root)), patch_callback=True)
    else:
        hps.solveStage(bc)
    return mesh, hps, hps.leaf_solution()


def run_oracle(mesh_kind, n, dom, f, bc, options=None, lam=0.0, patch_g=None):
    root = O.FiniteVolumePatch(O.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    if mesh_kind[0] == "uniform":
        mesh = O.Mesh().uniform(mesh_kind[1], root)
    else:
        mesh = O.Mesh().refineByFunction(mesh_kind[1], 0.0, mesh_kind[2], mesh_kind[3], root)
    hps = O.HPSAlgorithm(mesh, O.FiniteVolumeSolver(solver_type=O.FISHPACK90,
                                                    lambda_function=lambda x, y: lam), options)
    hps.buildStage()
    hps.upwardsStage(f)
    if patch_g is not None:
        hps.solveStage(O.patch_callback(lambda root: setattr(root, "g", patch_g(root))))
    else:
        hps.solveStage(lambda s, x, y: tuple(float(np.asarray(v).ravel()[0])
                                             for v in bc(s, np.array([x]), np.array([y]))))
    return mesh, hps, O.leaf_solution(hps)


def dirichlet_exact(side, x, y):
    return u_exact(x, y), 1.0, 0.0


def test_config1_uniform_L3_matches_oracle(ef):
    # config 1: Poisson on [-10,10]^2, uniform level 3, 16x16 patches
    dom = (-10.0, 10.0, -10.0, 10.0)
    f = lambda x, y: -(np.sin(x) + np.sin(y))
    mesh, hps, u = run_gpu(ef, ("uniform", 3), 16, dom, f, dirichlet_exact)
    om, ohps, uo = run_oracle(("uniform", 3), 16, dom, f, dirichlet_exact)
    assert rel(u, uo) <= REL
    X, Y = mesh.cell_centres()
    err_gpu = np.abs(u - u_exact(X, Y)).max()
    err_orc = np.abs(uo - u_exact(X, Y)).max()
    assert abs(err_gpu - err_orc) <= 1e-9 * err_orc   # discretisation error unchanged
    assert err_gpu < 5e-3
    # patches carry the solution like the reference's leaf patches
    assert np.array_equal(mesh.patches[5].vectorU(), u[5 * 256:6 * 256])


def test_root_T_and_h_match_oracle(ef):
    dom = (-1.0, 1.0, -1.0, 1.0)
    f = lambda x, y: np.exp(x) * np.cos(3 * y)
    mesh, hps, u = run_gpu(ef, ("uniform", 2), 8, dom, f, dirichlet_exact)
    om, ohps, uo = run_oracle(("uniform", 2), 8, dom, f, dirichlet_exact)
    assert rel(hps.root_T(), ohps.mesh.quadtree.root().T) <= REL
    assert rel(hps.root_h(), ohps.mesh.quadtree.root().h) <= REL
    assert rel(u, uo) <= REL


def _random_problem(seed):
    rng = np.random.default_rng(seed)
    amp, cx, cy, wd = rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(0.05, 0.3, 8)
    co = rng.standard_normal((4, 6))

    def f(x, y):
        x = np.asarray(x, dtype=float); y = np.asarray(y, dtype=float)
        out = np.zeros(np.broadcast(x, y).shape)
        for k in range(8):
            out = out + amp[k] * np.exp(-((x - cx[k]) ** 2 + (y - cy[k]) ** 2) / wd[k] ** 2)
        return out

    def bc(side, x, y):
        t = (y if side < 2 else x)
        v = sum(co[side, m] * np.sin((m + 1) * np.pi * (t + 1) / 2) for m in range(6))
        return v, 1.0, 0.0
    return f, bc


@pytest.mark.parametrize("L,n", [(2, 8), (4, 4), (3, 16)])
def test_uniform_random_data_matches_oracle(ef, L, n):
    f, bc = _random_problem(L * 100 + n)
    dom = (-1.0, 1.0, -1.0, 1.0)
    _, _, u = run_gpu(ef, ("uniform", L), n, dom, f, bc)
    _, _, uo = run_oracle(("uniform", L), n, dom, f, bc)
    assert rel(u, uo) <= REL


ADAPTIVE_CASES = {
    "config2_small": ((lambda x, y: abs(np.sin(x) + np.sin(y)) > 1.2), (-10.0, 10.0, -10.0, 10.0), 8, 0, 4),
    "wedge": ((lambda x, y: y > 0.45 and x > 0.45), (0.0, 1.0, 0.0, 1.0), 4, 0, 6),
    "disk": ((lambda x, y: (x - 0.7) ** 2 + (y - 0.7) ** 2 < 0.04), (0.0, 1.0, 0.0, 1.0), 4, 0, 6),
    "ring": ((lambda x, y: abs(x * x + y * y - 0.5) < 0.05), (-1.0, 1.0, -1.0, 1.0), 8, 1, 5),
    # 16 x 16 leaves (register-transform leaf kernels), 88 leaves: the last 16-leaf block is ragged
    "disk16": ((lambda x, y: (x - 0.7) ** 2 + (y - 0.7) ** 2 < 0.04), (0.0, 1.0, 0.0, 1.0), 16, 0, 4),
}


@pytest.mark.parametrize("case", sorted(ADAPTIVE_CASES))
def test_adaptive_matches_oracle(ef, case):
    fn, dom, n, lo, hi = ADAPTIVE_CASES[case]
    f, bc = _random_problem(7)
    _, _, u = run_gpu(ef, ("adaptive", fn, lo, hi), n, dom, f, bc)
    om, ohps, uo = run_oracle(("adaptive", fn, lo, hi), n, dom, f, bc)
    assert rel(u, uo) <= REL


def test_adaptive_case_has_multi_step_coarsening():
    # the wedge case exercises coarsening by more than one level in one merge (tag up to 4)
    fn, dom, n, lo, hi = ADAPTIVE_CASES["wedge"]
    root = O.FiniteVolumePatch(O.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    mesh = O.Mesh().refineByFunction(fn, 0.0, lo, hi, root)
    hps = O.HPSAlgorithm(mesh, O.FiniteVolumeSolver(solver_type=O.FISHPACK90))
    hps.buildStage()
    assert max(nd.data.n_coarsens for nd in mesh.quadtree.map.values()) >= 3


def test_neumann_root_boundary_matches_oracle(ef):
    # thermal-style data: Dirichlet on W/E, Neumann (a=0, b=1) on S/N (HPSAlgorithm.hpp:402-420)
    f, _ = _random_problem(3)

    def bc(side, x, y):
        if side < 2:
            return u_exact(x, y), 1.0, 0.0
        return np.cos(y) * 0 + 0.3 * np.cos(x), 0.0, 1.0
    dom = (-1.0, 1.0, -1.0, 1.0)
    _, _, u = run_gpu(ef, ("uniform", 2), 8, dom, f, bc)
    _, _, uo = run_oracle(("uniform", 2), 8, dom, f, bc)
    assert rel(u, uo) <= REL


def test_robin_root_boundary_matches_oracle(ef):
    f, _ = _random_problem(4)

    def bc(side, x, y):
        return np.sin(2 * x + y), 1.0 + 0.0 * x, 0.25 + 0.0 * x
    dom = (0.0, 2.0, 0.0, 2.0)
    _, _, u = run_gpu(ef, ("uniform", 3), 4, dom, f, bc)
    _, _, uo = run_oracle(("uniform", 3), 4, dom, f, bc)
    assert rel(u, uo) <= REL


def test_helmholtz_lambda(ef):
    f, bc = _random_problem(5)
    dom = (-1.0, 1.0, -1.0, 1.0)
    _, _, u = run_gpu(ef, ("uniform", 3), 8, dom, f, bc, lam=-4.0)
    _, _, uo = run_oracle(("uniform", 3), 8, dom, f, bc, lam=-4.0)
    assert rel(u, uo) <= REL


def test_homogeneous_rhs_option(ef):
    f, bc = _random_problem(6)
    dom = (-1.0, 1.0, -1.0, 1.0)
    opts = {"cache-operators": False, "homogeneous-rhs": True}
    _, _, u = run_gpu(ef, ("uniform", 2), 8, dom, f, bc, options=opts)
    _, _, uo = run_oracle(("uniform", 2), 8, dom, f, bc, options=opts)
    assert rel(u, uo) <= REL


def test_cache_operators_option_uniform(ef):
    f, bc = _random_problem(8)
    dom = (-1.0, 1.0, -1.0, 1.0)
    opts = {"cache-operators": True, "homogeneous-rhs": False}
    _, _, u = run_gpu(ef, ("uniform", 3), 8, dom, f, bc, options=opts)
    _, _, uo = run_oracle(("uniform", 3), 8, dom, f, bc, options=opts)
    assert rel(u, uo) <= REL


def test_solve_stage_root_patch_callback(ef):
    f, _ = _random_problem(9)
    dom = (-1.0, 1.0, -1.0, 1.0)
    pg = lambda root: np.cos(np.arange(4 * root.grid().nx()) * 0.1)
    _, _, u = run_gpu(ef, ("uniform", 2), 8, dom, f, None, patch_g=pg)
    _, _, uo = run_oracle(("uniform", 2), 8, dom, f, None, patch_g=pg)
    assert rel(u, uo) <= REL


def test_repeated_solves_on_one_build(ef):
    # thermal-style loop: one build, several upward + solve stages
    dom = (-1.0, 1.0, -1.0, 1.0)
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, *dom[:2], 8, *dom[2:]))
    mesh = ef.Mesh().uniform(3, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    for seed in (11, 12):
        f, bc = _random_problem(seed)
        hps.upwardsStage(f)
        hps.solveStage(bc)
        _, _, uo = run_oracle(("uniform", 3), 8, dom, f, bc)
        assert rel(hps.leaf_solution(), uo) <= REL


def test_config4_size_uniform_L6_equals_global_five_point(ef):
    # config 4 size (1024^2 dofs): HPS equals the global 5-point solve (an independent oracle)
    f, bc = _random_problem(42)
    dom = (-1.0, 1.0, -1.0, 1.0)
    mesh, hps, u = run_gpu(ef, ("uniform", 6), 16, dom, f, bc)
    N = 16 * 64
    A, cW, cE, cS, cN, x, y = G.assemble(N, N, *dom)
    X, Y = np.meshgrid(x, y, indexing="ij")
    F = f(X, Y)
    gW = bc(0, np.full(N, -1.0), y)[0]; gE = bc(1, np.full(N, 1.0), y)[0]
    gS = bc(2, x, np.full(N, -1.0))[0]; gN = bc(3, x, np.full(N, 1.0))[0]
    F[0, :] += -2.0 * cW[0, :] * gW; F[-1, :] += -2.0 * cE[-1, :] * gE
    F[:, 0] += -2.0 * cS[:, 0] * gS; F[:, -1] += -2.0 * cN[:, -1] * gN
    # residual of the GPU solution in the global system (size-independent check)
    Ug = np.empty((N, N))
    order = G.to_leaf_order(np.arange(N * N, dtype=float).reshape(N, N), 6, 16).astype(np.int64)
    Ug.ravel()[order] = u
    res = A @ Ug.ravel() - F.ravel()
    assert np.abs(res).max() <= 1e-9 * np.abs(F).max()
    import scipy.sparse.linalg as spla
    Us = spla.spsolve(A.tocsc(), F.ravel())
    assert rel(Ug.ravel(), Us) <= 1e-11


def test_linearity_large(ef):
    # size-independent property at L5 x 16 (512^2 dofs): u(f1+f2, g1+g2) = u(f1,g1) + u(f2,g2)
    dom = (-1.0, 1.0, -1.0, 1.0)
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, *dom[:2], 16, *dom[2:]))
    mesh = ef.Mesh().uniform(5, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    f1, b1 = _random_problem(21)
    f2, b2 = _random_problem(22)
    sols = []
    for f, bc in ((f1, b1), (f2, b2), (lambda x, y: f1(x, y) + f2(x, y),
                                        lambda s, x, y: (b1(s, x, y)[0] + b2(s, x, y)[0], 1.0, 0.0))):
        hps.upwardsStage(f)
        hps.solveStage(bc)
        sols.append(hps.leaf_solution())
    assert rel(sols[0] + sols[1], sols[2]) <= 1e-12


def test_robin_root_lu_is_reused_while_a_b_are_unchanged(ef):
    """Repeated Robin solves on one tree: the general root matrix is factored once while (a, b) stay
    the same, each result still matches the oracle, and changing b re-factors it."""
    dom = (0.0, 2.0, 0.0, 2.0)
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(4, dom[0], dom[1], 4, dom[2], dom[3]))
    mesh = ef.Mesh().uniform(3, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    M = hps.M
    a, b = np.ones(4 * M), np.full(4 * M, 0.25)
    rng = np.random.default_rng(8)
    X, Y = mesh.cell_centres()
    base = hps.root_factorizations
    for k in range(3):
        f = np.sin(X + k) * np.cos(Y)
        r = rng.standard_normal(4 * M)
        hps.upwards_array(f)
        hps.solve_arrays(a, b, r)
        u = hps.leaf_solution()
        om = O.Mesh().uniform(3, O.FiniteVolumePatch(O.FiniteVolumeGrid(4, dom[0], dom[1], 4, dom[2], dom[3])))
        oh = O.HPSAlgorithm(om, O.FiniteVolumeSolver(solver_type=O.FISHPACK90))
        oh.buildStage()
        oh.upwards_with_data(f)
        oh.solve_with_data(a, b, r)
        assert rel(u, O.leaf_solution(oh)) <= REL
    assert hps.root_factorizations - base == 1
    hps.upwards_array(np.sin(X))
    hps.solve_arrays(a, np.full(4 * M, 0.5), rng.standard_normal(4 * M))
    assert hps.root_factorizations - base == 2


@pytest.mark.parametrize("solver", ["fishpack", "five_point"])
def test_save_load_solves_bit_identically(ef, tmp_path, solver):
    """A built tree saved to a file and loaded into a new handle solves bit for bit like the
    original, without re-merging; a damaged file is rejected."""
    if solver == "fishpack":
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, -1.0, 1.0, 8, -1.0, 1.0))
        mesh = ef.Mesh().refineByFunction(lambda x, y: x * x + y * y < 0.3, 0.0, 1, 4, root)
        hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    else:
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, -1.0, 1.0, 8, -1.0, 1.0))
        mesh = ef.Mesh().uniform(2, root)
        hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(
            beta_function=lambda x, y: 1.0 + 0.5 * np.sin(np.pi * x) * np.cos(np.pi * y),
            lambda_function=lambda x, y: -1.0 + 0.0 * x, solver_type=ef.FivePointStencil))
    hps.buildStage()
    X, Y = mesh.cell_centres()
    f = np.sin(3 * X) * np.cos(2 * Y)
    r = np.concatenate([np.cos(x + 2 * y) for x, y in hps.boundary_points()])
    a = np.ones_like(r)
    hps.upwards_array(f)
    hps.solve_arrays(a, np.zeros_like(a), r)
    u = hps.leaf_solution()
    path = tmp_path / "tree.efgb"
    hps.save(path)
    h2 = ef.HPSAlgorithm.load(path)
    assert h2.num_leaves == hps.num_leaves and h2.M == hps.M
    h2.upwards_array(f)
    h2.solve_arrays(a, np.zeros_like(a), r)
    assert np.array_equal(h2.leaf_solution(), u)
    blob = bytearray(path.read_bytes())
    blob[len(blob) // 2] ^= 0x40
    bad = tmp_path / "bad.efgb"
    bad.write_bytes(bytes(blob))
    with pytest.raises(RuntimeError):
        ef.HPSAlgorithm.load(bad)


def test_incremental_build_equals_fresh_build(ef):
    """Local re-factorisation after a mesh change: only the merges above changed leaves run, the
    others are copied from the old tree, and the result equals a fresh build bit for bit."""
    def tree(cx):
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(8, -1.0, 1.0, 8, -1.0, 1.0))
        mesh = ef.Mesh().refineByFunction(lambda x, y, cx=cx: (x - cx) ** 2 + (y + 0.5) ** 2 < 0.04, 0.0, 1, 5, root)
        return mesh, ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    _, old = tree(-0.5)
    old.buildStage()
    mesh, fresh = tree(-0.3)
    fresh.buildStage()
    _, inc = tree(-0.3)
    reused = inc.buildStageFrom(old)
    merges = mesh.num_nodes() - mesh.num_leaves()
    assert 0 < reused < merges
    X, Y = mesh.cell_centres()
    f = np.cos(2 * X) * np.sin(Y)
    r = np.concatenate([np.sin(x - y) for x, y in fresh.boundary_points()])
    a = np.ones_like(r)
    out = []
    for h in (fresh, inc):
        h.upwards_array(f)
        h.solve_arrays(a, np.zeros_like(a), r)
        out.append(h.leaf_solution())
    assert np.array_equal(out[0], out[1])
    assert np.array_equal(fresh.root_T(), inc.root_T())


def test_cooperative_lu_panel_matches_single_cta(ef):
    """The multi-CTA LU panel (matrices with >= 512 rows left: here the root X of a 256^2 tree and
    the first panels of its children's merges) gives the single-CTA factors bit for bit."""
    from ellipticforest_gb300._lib import check, load
    Ts = []
    for coop in (1, 0):
        root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -1.0, 1.0, 16, -1.0, 1.0))
        mesh = ef.Mesh().uniform(4, root)
        hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
        check(load().ef_hps_set_option(hps.handle, b"cooperative-lu", coop))
        hps.buildStage()
        Ts.append(hps.root_T())
    check(load().ef_hps_set_option(hps.handle, b"cooperative-lu", 1))
    assert np.array_equal(Ts[0], Ts[1])


def test_build_graph_replay_equals_eager(ef):
    """The merges of a build run as one captured CUDA graph from the third build of a handle on (the
    first eager, the second captured): the same kernels, and the root T and a solve bit-identical to
    an eager build."""
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(16, -1.0, 1.0, 16, -1.0, 1.0))
    mesh = ef.Mesh().uniform(4, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    f, bc = _random_problem(31)
    hps.set_graphs(False)
    hps.buildStage()
    T0 = hps.root_T()
    n0, rep0 = hps.build_info()
    hps.upwardsStage(f)
    hps.solveStage(bc)
    u0 = hps.leaf_solution()
    hps.set_graphs(True)
    for _ in range(3):
        hps.buildStage()
    n1, rep1 = hps.build_info()
    assert rep1 >= 1 and n1 == n0 > 0
    assert np.array_equal(hps.root_T(), T0)
    hps.set_graphs(False)
    hps.upwardsStage(f)
    hps.solveStage(bc)
    assert np.array_equal(hps.leaf_solution(), u0)
