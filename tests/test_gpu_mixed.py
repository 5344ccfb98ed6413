"""Mixed-precision many-RHS form: FP32 HPS passes refined against the exact residual must reach the
FP64 HPS solution to <= 1e-10 relative, on uniform and adaptive trees, and a request's result must
not depend on the other requests of its block."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def ef(lib):
    import ellipticforest_gb300
    return ellipticforest_gb300


def requests(hps, mesh, B, seed):
    rng = np.random.default_rng(seed)
    X, Y = mesh.cell_centres()
    pts = hps.boundary_points()
    F, A, R = [], [], []
    for _ in range(B):
        amp, cx, cy, wd = rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(-1, 1, 8), rng.uniform(0.05, 0.3, 8)
        f = sum(amp[k] * np.exp(-((X - cx[k]) ** 2 + (Y - cy[k]) ** 2) / wd[k] ** 2) for k in range(8))
        co = rng.standard_normal((4, 6))
        r = np.concatenate([sum(co[s, m] * np.sin((m + 1) * np.pi * ((y if s < 2 else x) + 1) / 2) for m in range(6))
                            for s, (x, y) in enumerate(pts)])
        F.append(f); A.append(np.ones_like(r)); R.append(r)
    return np.array(F), np.array(A), np.array(R)


def fp64_solutions(hps, F, A, R):
    out = []
    for f, a, r in zip(F, A, R):
        hps.upwards_array(f)
        hps.solve_arrays(a, np.zeros_like(a), r)
        out.append(hps.leaf_solution())
    return np.array(out)


def make(ef, kind, n, dom):
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    if kind[0] == "uniform":
        mesh = ef.Mesh().uniform(kind[1], root)
    else:
        mesh = ef.Mesh().refineByFunction(kind[1], 0.0, kind[2], kind[3], root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps.buildStage()
    return mesh, hps


@pytest.mark.parametrize("kind,n", [(("uniform", 4), 16), (("uniform", 5), 8)])
def test_mixed_reaches_fp64_solution_uniform(ef, kind, n):
    mesh, hps = make(ef, kind, n, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, 3, 11)
    ref = fp64_solutions(hps, F, A, R)
    hps.mixed_init(4)
    u = hps.mixed_solve(F, A, R, sweeps=2)
    for k in range(3):
        err = np.abs(u[k] - ref[k]).max() / np.abs(ref[k]).max()
        assert err <= TOL, (k, err)
    res = hps.mixed_residuals(3)
    assert np.all(res[2, :3] < res[0, :3] * 1e-8)


def test_mixed_ragged_items_16x16(ef):
    # 16 x 16 leaves run 16 items per block in the leaf and first-residual kernels: an adaptive tree
    # of 88 leaves with 3 requests leaves the last block half empty
    fn = lambda x, y: (x - 0.7) ** 2 + (y - 0.7) ** 2 < 0.04
    mesh, hps = make(ef, ("adaptive", fn, 0, 4), 16, (0.0, 1.0, 0.0, 1.0))
    B = 3
    assert (mesh.num_leaves() * B) % 16 != 0
    F, A, R = requests(hps, mesh, B, 21)
    ref = fp64_solutions(hps, F, A, R)
    hps.mixed_init(B)
    u = hps.mixed_solve(F, A, R, sweeps=2)
    for k in range(B):
        assert np.abs(u[k] - ref[k]).max() / np.abs(ref[k]).max() <= TOL


def test_mixed_reaches_fp64_solution_adaptive(ef):
    fn = lambda x, y: y > 0.45 and x > 0.45
    mesh, hps = make(ef, ("adaptive", fn, 0, 5), 8, (0.0, 1.0, 0.0, 1.0))
    F, A, R = requests(hps, mesh, 2, 5)
    ref = fp64_solutions(hps, F, A, R)
    hps.mixed_init(2)
    u = hps.mixed_solve(F, A, R, sweeps=2)
    for k in range(2):
        assert np.abs(u[k] - ref[k]).max() / np.abs(ref[k]).max() <= TOL


def test_mixed_result_same_alone_and_in_a_block(ef):
    mesh, hps = make(ef, ("uniform", 3), 16, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, 11, 23)
    hps.mixed_init(11)
    block = hps.mixed_solve(F, A, R, sweeps=1)
    for k in (0, 5, 10):
        alone = hps.mixed_solve(F[k:k + 1], A[k:k + 1], R[k:k + 1], sweeps=1)
        assert np.array_equal(alone[0], block[k])


def test_graph_replay_matches_eager(ef):
    """The captured solve sequences (plain FP64 and mixed) give the eager results bit for bit."""
    import torch
    mesh, hps = make(ef, ("uniform", 3), 16, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, 3, 31)
    f = torch.from_numpy(F[0]).cuda()
    a = torch.from_numpy(A[0]).cuda()
    b = torch.zeros_like(a)
    r = torch.from_numpy(R[0]).cuda()
    hps.set_graphs(False)
    hps.load_device_async(f.data_ptr(), a.data_ptr(), b.data_ptr(), r.data_ptr())
    hps.solve_device_async(True)
    hps.synchronize()
    eager = hps.leaf_solution().copy()
    hps.set_graphs(True)
    for _ in range(3):  # eager first call, capture, replay
        hps.load_device_async(f.data_ptr(), a.data_ptr(), b.data_ptr(), r.data_ptr())
        hps.solve_device_async(True)
        hps.synchronize()
        assert np.array_equal(hps.leaf_solution(), eager)
    hps.mixed_init(3)
    hps.set_graphs(False)
    ref = hps.mixed_solve(F, A, R, sweeps=1)
    hps.set_graphs(True)
    for _ in range(3):
        assert np.array_equal(hps.mixed_solve(F, A, R, sweeps=1), ref)


@pytest.mark.parametrize("level,n", [(3, 16), (2, 32)])
def test_mixed_five_point_variable_coefficients(ef, level, n):
    """Config-3 coefficients (alpha = 1, beta = 1 + 0.5 sin(pi x) cos(pi y), lambda = -1) on
    FivePointStencil leaves: FP32 band solves + FP64 variable-coefficient residual reach the FP64
    HPS solution, and a request's result is the same alone and in a block."""
    PI = np.pi
    solver = ef.FiniteVolumeSolver(alpha_function=lambda x, y: 1.0 + 0.0 * x,
                                   beta_function=lambda x, y: 1.0 + 0.5 * np.sin(PI * x) * np.cos(PI * y),
                                   lambda_function=lambda x, y: -1.0 + 0.0 * x,
                                   solver_type=ef.FivePointStencil)
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, -1.0, 1.0, n, -1.0, 1.0))
    mesh = ef.Mesh().uniform(level, root)
    hps = ef.HPSAlgorithm(mesh, solver)
    hps.buildStage()
    F, A, R = requests(hps, mesh, 5, 41)
    ref = fp64_solutions(hps, F, A, R)
    hps.mixed_init(5)
    u = hps.mixed_solve(F, A, R, sweeps=2)
    for k in range(5):
        err = np.abs(u[k] - ref[k]).max() / np.abs(ref[k]).max()
        assert err <= TOL, (k, err)
    alone = hps.mixed_solve(F[3:4], A[3:4], R[3:4], sweeps=2)
    assert np.array_equal(alone[0], u[3])


@pytest.mark.parametrize("kind,n,fp64_levels", [(("uniform", 4), 16, 3), (("uniform", 4), 16, 0),
                                                 (("adaptive", None, 0, 5), 8, 2)])
def test_mixed_build_reaches_fp64_solution(ef, kind, n, fp64_levels):
    """FP32 merges (interface LU of the top levels in FP64) feed the mixed solver; the FP64
    refinement still reaches the FP64 HPS solution of a separately FP64-built tree."""
    dom = (-1.0, 1.0, -1.0, 1.0) if kind[0] == "uniform" else (0.0, 1.0, 0.0, 1.0)
    if kind[0] == "adaptive":
        kind = ("adaptive", lambda x, y: y > 0.45 and x > 0.45, kind[2], kind[3])
    mesh, hps64 = make(ef, kind, n, dom)
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    mesh32 = (ef.Mesh().uniform(kind[1], root) if kind[0] == "uniform"
              else ef.Mesh().refineByFunction(kind[1], 0.0, kind[2], kind[3], root))
    hps32 = ef.HPSAlgorithm(mesh32, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90))
    hps32.buildStageMixed(fp64_levels)
    F, A, R = requests(hps64, mesh, 3, 17)
    ref = fp64_solutions(hps64, F, A, R)
    hps32.mixed_init(3)
    u = hps32.mixed_solve(F, A, R, sweeps=3)
    for k in range(3):
        err = np.abs(u[k] - ref[k]).max() / np.abs(ref[k]).max()
        assert err <= TOL, (k, err)


@pytest.mark.parametrize("dom,lam,zero_f", [((0.0, 2.0, 0.0, 1.0), 0.0, False),
                                            ((-1.0, 1.0, -1.0, 1.0), -2.5, False),
                                            ((0.0, 2.0, 0.0, 1.0), -2.5, True),
                                            ((-1.0, 1.0, -1.0, 1.0), 0.0, True)])
def test_mixed_residual_forms_one_sweep(ef, dom, lam, zero_f):
    """The leaf residual's forms: rectangular cells (cx != cy, one product per direction), a
    Helmholtz lambda (a third product), and f = 0 (Laplace data: every product exceeds the scale of f,
    so each cell sums on the scale of its largest term) -- one refinement sweep reaches the FP64
    solution."""
    n = 8
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    mesh = ef.Mesh().uniform(4, root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90,
                                                      lambda_function=lambda x, y: lam))
    hps.buildStage()
    F, A, R = requests(hps, mesh, 3, 31)
    if zero_f:
        F[:] = 0.0
    ref = fp64_solutions(hps, F, A, R)
    hps.mixed_init(3)
    u = hps.mixed_solve(F, A, R, sweeps=1)
    for k in range(3):
        assert np.abs(u[k] - ref[k]).max() / np.abs(ref[k]).max() <= TOL, k


def test_mixed_solve_blocks_matches_single_blocks(ef):
    """The pipelined two-lane form returns, block by block, exactly what one block at a time gives."""
    mesh, hps = make(ef, ("uniform", 3), 16, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, 10, 41)
    hps.mixed_init(4)
    blocks = [(F[0:4], A[0:4], R[0:4]), (F[4:8], A[4:8], R[4:8]), (F[8:10], A[8:10], R[8:10])]
    got = hps.mixed_solve_blocks(blocks, sweeps=1)
    for (f, a, r), u in zip(blocks, got):
        assert np.array_equal(u, hps.mixed_solve(f, a, r, sweeps=1))


def test_device_resident_lane_matches_lane0(ef):
    """Lane 1 (shares lane 0's FP32 operators, own stream) solves its resident block to the same bits."""
    torch = pytest.importorskip("torch")
    mesh, hps = make(ef, ("uniform", 3), 16, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, 3, 51)
    hps.mixed_init(3)
    u0 = hps.mixed_solve(F, A, R, sweeps=1)
    # the pipelined call leaves block k's inputs resident in lane k % 3: two blocks fill lanes 0, 1
    hps.mixed_solve_blocks([(F, A, R), (F, A, R)], sweeps=1)
    f1, a1, r1, u1p, st1 = hps.mixed_lane(1)
    hps.mixed_solve_async(3, 1, lane=1)
    torch.cuda.synchronize()
    n = F.shape[1]

    class _Lane1U:  # lane 1's device result, wrapped through the CUDA array interface
        __cuda_array_interface__ = {"shape": (3 * n,), "typestr": "<f8", "data": (u1p, False), "version": 3}

    out = torch.as_tensor(_Lane1U(), device="cuda").clone()
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().reshape(3, n), u0)


def _set_general_residual(hps, on):
    from ellipticforest_gb300._lib import check, load
    check(load().ef_hps_set_option(hps.handle, b"general-leaf-residual", int(on)))


@pytest.mark.parametrize("kind,dom,lam,zero_f,B", [
    (("uniform", 4), (-1.0, 1.0, -1.0, 1.0), 0.0, False, 5),     # form 0: cx = cy, lambda = 0
    (("uniform", 3), (0.0, 2.0, 0.0, 1.0), 0.0, False, 3),       # form 1: rectangular cells
    (("uniform", 3), (-1.0, 1.0, -1.0, 1.0), -2.5, False, 3),    # form 1: Helmholtz lambda
    (("uniform", 3), (-1.0, 1.0, -1.0, 1.0), 0.0, True, 2),      # f = 0: every product above f
    (("adaptive", lambda x, y: (x - 0.7) ** 2 + (y - 0.7) ** 2 < 0.04, 0, 4), (0.0, 1.0, 0.0, 1.0), 0.0,
     False, 3),                                                   # ragged last block
])
def test_residual_kernel_16_bit_identical_to_general_kernel(ef, kind, dom, lam, zero_f, B):
    """16 x 16 leaves take the exact residual through their own kernel (column, then row ownership
    of the item's fixed-point tile) and the first residual fused with the first Neumann step; the
    general leaf-size kernels, run apart, compute the same numbers, so the two give bit-identical
    solutions and residual histories."""
    n = 16
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    if kind[0] == "uniform":
        mesh = ef.Mesh().uniform(kind[1], root)
    else:
        mesh = ef.Mesh().refineByFunction(kind[1], 0.0, kind[2], kind[3], root)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(solver_type=ef.FISHPACK90,
                                                      lambda_function=lambda x, y: lam + 0.0 * x))
    hps.buildStage()
    F, A, R = requests(hps, mesh, B, 57)
    if zero_f:
        F[:] = 0.0
    F[0] *= 1.0e6   # requests of very different size share no scale
    got = []
    try:
        for general in (0, 1):
            _set_general_residual(hps, general)
            hps.mixed_init(B)
            u = hps.mixed_solve(F, A, R, sweeps=2)
            got.append((u, hps.mixed_residuals(3)[:, :B]))
    finally:
        _set_general_residual(hps, 0)
    assert np.array_equal(got[0][0], got[1][0])
    assert np.array_equal(got[0][1], got[1][1])
    ref = fp64_solutions(hps, F, A, R)
    for k in range(B):
        assert np.abs(got[0][0][k] - ref[k]).max() <= TOL * np.abs(ref[k]).max(), k


@pytest.mark.parametrize("L,n,B,robin", [(4, 16, 5, False), (3, 8, 8, False), (3, 16, 6, True)])
def test_interface_rows_in_place_bit_identical_to_per_level(ef, L, n, B, robin):
    """On a tree without coarsening steps the residual reads each leaf's Dirichlet rows where they
    live (root data, ancestors' interface states) and takes every interface mismatch straight from
    two leaf edge-flux rows; moving the rows level by level gives the same bits.  Blocks smaller
    than the solver's capacity (row stride = the block's request count) and a Robin root included."""
    from ellipticforest_gb300._lib import check, load
    mesh, hps = make(ef, ("uniform", L), n, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, B, 71)
    got = []
    try:
        for per_level in (0, 1):
            check(load().ef_hps_set_option(hps.handle, b"per-level-interface", per_level))
            hps.mixed_init(B + 3)
            if robin:
                hps.mixed_set_root(np.full(4 * hps.M, 1.0), np.full(4 * hps.M, 0.25))
            got.append([hps.mixed_solve(F[:k], A[:k], R[:k], sweeps=2) for k in (B, B - 2)])
    finally:
        check(load().ef_hps_set_option(hps.handle, b"per-level-interface", 0))
    for u0, u1 in zip(got[0], got[1]):
        assert np.array_equal(u0, u1)


def test_gemm_plan_set_instead_of_timed(ef):
    """A node-GEMM plan set through the API replaces the timing: the block solver reports it, solves
    to the FP64 solution with it, and codes the tree cannot run are refused."""
    from ellipticforest_gb300._lib import EFError
    mesh, hps = make(ef, ("uniform", 4), 16, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, 4, 81)
    ref = fp64_solutions(hps, F, A, R)
    hps.mixed_init(4)
    tuned = hps.mixed_gemm_plan()
    # every group on the CUDA-core kernel with K split 1, except the tensor-core DOWN at s >= 32
    plan = [(lv, s, 1, 1, -1 if s >= 32 else 2) for (lv, s, *_rest) in tuned]
    hps.mixed_set_gemm_plan(plan)
    hps.mixed_init(4)
    assert hps.mixed_gemm_plan() == plan
    u = hps.mixed_solve(F, A, R, sweeps=1)
    for k in range(4):
        assert np.abs(u[k] - ref[k]).max() <= TOL * np.abs(ref[k]).max(), k
    with pytest.raises(EFError):
        hps.mixed_set_gemm_plan(plan[:-1])                       # one row per group
    with pytest.raises(EFError):
        hps.mixed_set_gemm_plan([(lv, s, 1, 1, -16) for (lv, s, *_r) in plan])   # K split too large
    with pytest.raises(EFError):
        hps.mixed_set_gemm_plan([(lv, s, -1, -1, -1) for (lv, s, *_r) in plan])  # H at s = 16


def _set_tc(hps, on):
    from ellipticforest_gb300._lib import check, load
    check(load().ef_hps_set_option(hps.handle, b"tensor-cores", int(on)))


@pytest.mark.parametrize("kind,n,B", [(("uniform", 4), 16, 5), (("uniform", 5), 16, 40), (("uniform", 3), 32, 8),
                                     (("adaptive", lambda x, y: (x - 0.2) ** 2 + (y + 0.3) ** 2 < 0.1, 0, 5), 16, 6),
                                     (("uniform", 1), 16, 3)])
def test_tensor_core_gemms_match_cuda_core_gemms(ef, kind, n, B):
    """The tcgen05 node GEMMs (three-way bf16 split of the FP32 operators and requests, six tensor
    products, FP32 accumulation in TMEM) give an FP32 pass as accurate as the CUDA-core FP32 GEMMs, and
    one FP64 sweep reaches the FP64 HPS solution to 1e-10; ragged request counts (B = 5, not a
    multiple of 4; B = 40, two request blocks of 32) included, and node groups whose operator rows
    end inside a 128-row tile of the tiled bf16 planes (odd node counts on the adaptive tree; the
    single 64-row W and DOWN operators of a level-1 tree)."""
    mesh, hps = make(ef, kind, n, (-1.0, 1.0, -1.0, 1.0))
    F, A, R = requests(hps, mesh, B, 41)
    ref = fp64_solutions(hps, F, A, R)
    errs = {}
    for tc in (0, 2):  # CUDA-core GEMMs only; tensor-core GEMMs wherever supported
        _set_tc(hps, tc)
        hps.mixed_init(B)
        plan = hps.mixed_gemm_plan()
        # forced: every node GEMM the tensor-core kernel supports on it (code < 0); off: none
        supported = lambda kind, s: s >= 16 and (s & (s - 1)) == 0 and (kind != 1 or s >= 32)
        assert all((row[2 + k] < 0) == (tc == 2 and supported(k, row[1])) for row in plan for k in range(3)), plan
        if tc == 2:
            assert any(row[2 + k] < 0 for row in plan for k in range(3))
        u0 = hps.mixed_solve(F, A, R, sweeps=0)
        u1 = hps.mixed_solve(F, A, R, sweeps=1)
        e0 = max(np.abs(u0[k] - ref[k]).max() / np.abs(ref[k]).max() for k in range(B))
        e1 = max(np.abs(u1[k] - ref[k]).max() / np.abs(ref[k]).max() for k in range(B))
        errs[tc] = (e0, e1)
        assert e1 <= TOL, (tc, e0, e1)
    _set_tc(hps, 1)
    # one FP32 pass: the tensor-core products are no less accurate than the FP32 FMA chains
    assert errs[2][0] <= 2.0 * errs[0][0] + 1e-12, errs


def test_tensor_core_result_same_alone_and_in_a_block(ef):
    mesh, hps = make(ef, ("uniform", 4), 16, (-1.0, 1.0, -1.0, 1.0))
    _set_tc(hps, 2)
    F, A, R = requests(hps, mesh, 9, 17)
    hps.mixed_init(9)
    block = hps.mixed_solve(F, A, R, sweeps=1)
    for k in (0, 4, 8):
        alone = hps.mixed_solve(F[k:k + 1], A[k:k + 1], R[k:k + 1], sweeps=1)
        assert np.array_equal(alone[0], block[k])


def _root_operator(hps, pattern):
    M = hps.M
    if pattern == "thermal":  # Dirichlet on W/E, Neumann on S/N (examples/thermal/main.cpp:324-350)
        a = np.concatenate([np.ones(2 * M), np.zeros(2 * M)])
        b = np.concatenate([np.zeros(2 * M), np.ones(2 * M)])
    else:                     # Robin everywhere
        a = np.ones(4 * M)
        b = np.full(4 * M, 0.25)
    return a, b


@pytest.mark.parametrize("pattern", ["thermal", "robin"])
def test_mixed_robin_root_data_reach_fp64_solution(ef, pattern):
    """a u + b du/dn = r with b != 0 in the block solver: the root data are refined with the rest of
    the state (root condition residual, FP32 correction through (diag a + diag b T)^{-1}) and reach the
    FP64 HPS solution (general root solve, HPSAlgorithm.hpp:402-420) to 1e-10 after one sweep; a
    request's result is the same alone and in a block."""
    mesh, hps = make(ef, ("uniform", 4), 16, (-1.0, 1.0, -1.0, 1.0))
    a, b = _root_operator(hps, pattern)
    F, _, R = requests(hps, mesh, 5, 77)
    ref = []
    for f, r in zip(F, R):
        hps.upwards_array(f)
        hps.solve_arrays(a, b, r)
        ref.append(hps.leaf_solution())
    hps.mixed_init(5)
    hps.mixed_set_root(a, b)
    A = np.zeros_like(R)  # not read while b != 0
    u = hps.mixed_solve(F, A, R, sweeps=1)
    for k in range(5):
        err = np.abs(u[k] - ref[k]).max() / np.abs(ref[k]).max()
        assert err <= TOL, (k, err)
    alone = hps.mixed_solve(F[2:3], A[2:3], R[2:3], sweeps=1)
    assert np.array_equal(alone[0], u[2])
    # b = 0 returns to per-request Dirichlet data
    hps.mixed_set_root(np.ones_like(a), np.zeros_like(b))
    ud = hps.mixed_solve(F[:1], np.ones_like(R[:1]), R[:1], sweeps=1)
    hps.upwards_array(F[0])
    hps.solve_arrays(np.ones_like(a), np.zeros_like(b), R[0])
    ref_d = hps.leaf_solution()
    assert np.abs(ud[0] - ref_d).max() / np.abs(ref_d).max() <= TOL
