"""FivePointStencil (variable alpha, beta, lambda) on the GPU against the oracle's dense 5-point
operator of FiniteVolumeSolver.cpp:27-223, at 1e-12 relative; config-3 coefficients and its
manufactured solution u = sin(2 pi x) sin(pi y)."""
import numpy as np
import pytest

from oracle import hps_oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-12
PI = np.pi


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300)


# config 3: alpha = 1, beta = 1 + 0.5 sin(pi x) cos(pi y), lambda = -1
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


# a harder set: variable alpha too
alphaV = lambda x, y: 1.0 + 0.25 * np.cos(x + 2 * y)
betaV = lambda x, y: 2.0 + np.sin(3 * x) * np.cos(y)
lambdaV = lambda x, y: -2.0 - x * x


@pytest.fixture(scope="module")
def ef(lib):
    import ellipticforest_gb300
    return ellipticforest_gb300


def solvers(ef, a, b, l):
    s = ef.FiniteVolumeSolver(alpha_function=a, beta_function=b, lambda_function=l)
    so = O.FiniteVolumeSolver(alpha_function=a, beta_function=b, lambda_function=l,
                              solver_type=O.FIVE_POINT_STENCIL)
    return s, so


@pytest.mark.parametrize("n,box,coef", [(4, (0.0, 1.0, 0.0, 1.0), "3"), (8, (-1.0, 1.0, -1.0, 1.0), "3"),
                                        (16, (-0.5, 0.25, 0.0, 0.75), "V"), (12, (1.0, 2.0, -2.0, -1.0), "V")])
def test_single_patch_five_point_matches_oracle(ef, n, box, coef):
    a, b, l = (alpha3, beta3, lambda3) if coef == "3" else (alphaV, betaV, lambdaV)
    s, so = solvers(ef, a, b, l)
    g = ef.FiniteVolumeGrid(n, *box[:2], n, *box[2:])
    og = O.FiniteVolumeGrid(n, *box[:2], n, *box[2:])
    assert rel(s.buildD2N(g), so.buildD2N(og)) <= REL
    rng = np.random.default_rng(n)
    gv, f = rng.standard_normal(4 * n), rng.standard_normal(n * n)
    assert rel(s.solve(g, gv, f), so.solve(og, gv, f)) <= REL
    assert rel(s.mapD2N(g, gv, f), so.mapD2N(og, gv, f)) <= REL
    assert rel(s.particularNeumannData(g, f), so.particularNeumannData(og, f)) <= REL


def test_five_point_with_unit_coefficients_equals_fishpack(ef):
    n = 16
    g = ef.FiniteVolumeGrid(n, -1, 1, n, 0, 2)
    rng = np.random.default_rng(3)
    gv, f = rng.standard_normal(4 * n), rng.standard_normal(n * n)
    s5 = ef.FiniteVolumeSolver(lambda_function=lambda x, y: -2.0 + 0 * x)
    sf = ef.FiniteVolumeSolver(lambda_function=lambda x, y: -2.0 + 0 * x, solver_type=ef.FISHPACK90)
    assert rel(s5.solve(g, gv, f), sf.solve(g, gv, f)) <= REL
    assert rel(s5.buildD2N(g), sf.buildD2N(g)) <= REL


def _hps_pair(ef, kind, n, dom, a, b, l, f, bc):
    root = ef.FiniteVolumePatch(ef.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    oroot = O.FiniteVolumePatch(O.FiniteVolumeGrid(n, dom[0], dom[1], n, dom[2], dom[3]))
    if kind[0] == "uniform":
        mesh = ef.Mesh().uniform(kind[1], root)
        om = O.Mesh().uniform(kind[1], oroot)
    else:
        mesh = ef.Mesh().refineByFunction(kind[1], 0.0, kind[2], kind[3], root)
        om = O.Mesh().refineByFunction(kind[1], 0.0, kind[2], kind[3], oroot)
    hps = ef.HPSAlgorithm(mesh, ef.FiniteVolumeSolver(alpha_function=a, beta_function=b, lambda_function=l))
    hps.buildStage()
    hps.upwardsStage(f)
    hps.solveStage(bc)
    oh = O.HPSAlgorithm(om, O.FiniteVolumeSolver(alpha_function=a, beta_function=b, lambda_function=l,
                                                 solver_type=O.FIVE_POINT_STENCIL))
    oh.buildStage()
    oh.upwardsStage(f)
    oh.solveStage(lambda s, x, y: tuple(float(np.asarray(v).ravel()[0]) for v in bc(s, np.array([x]), np.array([y]))))
    return mesh, hps.leaf_solution(), O.leaf_solution(oh)


def test_config3_like_uniform_matches_oracle_and_converges(ef):
    dom = (-1.0, 1.0, -1.0, 1.0)
    bc = lambda s, x, y: (u3(x, y), 1.0, 0.0)
    errs = []
    for L, n in ((2, 8), (2, 16)):
        mesh, u, uo = _hps_pair(ef, ("uniform", L), n, dom, alpha3, beta3, lambda3, f3, bc)
        assert rel(u, uo) <= REL
        X, Y = mesh.cell_centres()
        errs.append(np.abs(u - u3(X, Y)).max())
    assert math_order(errs[0], errs[1]) > 1.8


def math_order(e1, e2):
    return np.log(e1 / e2) / np.log(2.0)


def test_five_point_adaptive_matches_oracle(ef):
    dom = (-1.0, 1.0, -1.0, 1.0)
    bc = lambda s, x, y: (np.cos(x) * np.exp(y), 1.0, 0.0)
    fn = lambda x, y: (x - 0.3) ** 2 + (y + 0.1) ** 2 < 0.1
    mesh, u, uo = _hps_pair(ef, ("adaptive", fn, 1, 4), 8, dom, alphaV, betaV, lambdaV,
                            lambda x, y: np.sin(3 * x + y), bc)
    assert rel(u, uo) <= REL
