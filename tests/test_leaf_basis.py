"""The 16 x 16 leaf kernels (k_mx_leaf16 in FP32, k_leaf16d in FP64) keep only rows 0..7 of the sine
basis V[i][k] = c_k sin(pi (k+1)(i+1/2)/n) and rebuild the rest from two symmetries:
V[15-i][k] = (-1)^k V[i][k] and, for the odd modes k = 2m+1, V[7-i][k] = (-1)^m V[i][k].  These CPU
tests pin the identities and restate the kernels' split transforms (analysis X = V^T x from even/odd
sums, synthesis x = V X in +- pairs and quads) against the dense products."""
import numpy as np
import pytest

N = 16


def basis(n):
    i = np.arange(n)[:, None]
    k = np.arange(n)[None, :]
    c = np.where(k == n - 1, np.sqrt(1.0 / n), np.sqrt(2.0 / n))
    return c * np.sin(np.pi * (k + 1) * (i + 0.5) / n)


def test_basis_is_orthonormal_eigenbasis():
    V = basis(N)
    assert np.allclose(V.T @ V, np.eye(N), atol=1e-14)
    # 1-D cell-centred operator with ghost 2g - u: tridiag(1, -2, 1) with -3 in both corners
    A = -2 * np.eye(N) + np.eye(N, k=1) + np.eye(N, k=-1)
    A[0, 0] = A[-1, -1] = -3
    mu = -4 * np.sin(np.pi * (np.arange(N) + 1) / (2 * N)) ** 2
    assert np.allclose(A @ V, V * mu, atol=1e-13)


def test_basis_symmetries():
    V = basis(N)
    for i in range(N):
        for k in range(N):
            assert abs(V[N - 1 - i, k] - (-1) ** k * V[i, k]) < 1e-14
    for i in range(8):
        for m in range(8):
            assert abs(V[7 - i, 2 * m + 1] - (-1) ** m * V[i, 2 * m + 1]) < 1e-14


def analysis_fp32_kernel(c, x):
    # k_mx_leaf16: X[k] = sum_{j<8} V[j][k] (x_j +- x_{15-j}), + for even k
    P, M = x[:8] + x[15:7:-1], x[:8] - x[15:7:-1]
    return np.array([sum(c[j, k] * (M[j] if k & 1 else P[j]) for j in range(8)) for k in range(N)])


def analysis_fp64_kernel(c, x):
    # k_leaf16d: the odd modes split once more over j and 7-j
    P, M = x[:8] + x[15:7:-1], x[:8] - x[15:7:-1]
    Q, R = M[:4] + M[7:3:-1], M[:4] - M[7:3:-1]
    X = np.zeros(N)
    for k in range(0, N, 2):
        X[k] = sum(c[j, k] * P[j] for j in range(8))
    for k in range(1, N, 2):
        src = R if (k >> 1) & 1 else Q
        X[k] = sum(c[j, k] * src[j] for j in range(4))
    return X


def synthesis_pairs(c, X):
    x = np.zeros(N)
    for i in range(8):
        e = sum(c[i, k] * X[k] for k in range(0, N, 2))
        o = sum(c[i, k] * X[k] for k in range(1, N, 2))
        x[i], x[15 - i] = e + o, e - o
    return x


def synthesis_quads(c, X):
    x = np.zeros(N)
    for i in range(4):
        ei = sum(c[i, k] * X[k] for k in range(0, N, 2))
        e7 = sum(c[7 - i, k] * X[k] for k in range(0, N, 2))
        oe = sum(c[i, k] * X[k] for k in range(1, N, 4))
        oo = sum(c[i, k + 2] * X[k + 2] for k in range(1, N, 4))
        x[i], x[15 - i] = ei + (oe + oo), ei - (oe + oo)
        x[7 - i], x[8 + i] = e7 + (oe - oo), e7 - (oe - oo)
    return x


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_split_transforms_match_dense(seed):
    V = basis(N)
    c = V[:8]
    rng = np.random.default_rng(seed)
    x, X = rng.standard_normal(N), rng.standard_normal(N)
    assert np.allclose(analysis_fp32_kernel(c, x), V.T @ x, atol=1e-13)
    assert np.allclose(analysis_fp64_kernel(c, x), V.T @ x, atol=1e-13)
    assert np.allclose(synthesis_pairs(c, X), V @ X, atol=1e-13)
    assert np.allclose(synthesis_quads(c, X), V @ X, atol=1e-13)


def test_patch_solve_by_split_transforms():
    # U = V [(V^T F V) ./ (mu_x + mu_y)] V^T solves the 5-point system with homogeneous Dirichlet data
    V, c = basis(N), basis(N)[:8]
    dx, dy = 0.03, 0.05
    mu = -4 * np.sin(np.pi * (np.arange(N) + 1) / (2 * N)) ** 2
    D = 1.0 / (mu[:, None] / dx ** 2 + mu[None, :] / dy ** 2)
    F = np.random.default_rng(5).standard_normal((N, N))
    A = np.array([analysis_fp32_kernel(c, F[t]) for t in range(N)])         # rows
    G = np.array([analysis_fp32_kernel(c, A[:, t]) for t in range(N)]).T    # columns
    G *= D
    C = np.array([synthesis_pairs(c, G[:, t]) for t in range(N)]).T         # columns
    U = np.array([synthesis_quads(c, C[t]) for t in range(N)])              # rows
    assert np.allclose(U, V @ (D * (V.T @ F @ V)) @ V.T, atol=1e-12)
    T = -2 * np.eye(N) + np.eye(N, k=1) + np.eye(N, k=-1)
    T[0, 0] = T[-1, -1] = -3
    assert np.allclose(T @ U / dx ** 2 + U @ T.T / dy ** 2, F, atol=1e-10)
