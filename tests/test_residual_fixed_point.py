"""CPU restatement of the integer leaf residual of the mixed block solver (k_mx_leaf_residual):
u and the ghost data on one fixed-point scale per item, exact second differences, exact 128-bit
products with 63-bit coefficient significands shifted to one per-item scale 2^sc, one exact
subtraction, one rounding to FP32.  Checked against the exact rational residual of the same FP64
inputs r = f - cx (u_W + u_E - 2 u_C) - cy (u_S + u_N - 2 u_C) - lambda u_C (ghost 2 g - u_C at
patch edges): the error must be the FP32 rounding of r plus a few units of 2^sc, where an FP64
evaluation of the stencil loses digits to cancellation."""
import math
import struct
from fractions import Fraction as Fr

import numpy as np
import pytest

M64 = (1 << 64) - 1


def bits(v):
    return struct.unpack("<Q", struct.pack("<d", float(v)))[0]


def bexp(v):
    return (bits(v) >> 52) & 0x7FF


def fx_shift(v, e_off):
    # v * 2^(1075 - e_off) truncated toward zero (the kernel's fx_shift)
    b = bits(v)
    e, m = (b >> 52) & 0x7FF, b & ((1 << 52) - 1)
    if e:
        m |= 1 << 52
    else:
        e = 1
    sh = e - e_off
    a = (m << sh) & M64 if sh >= 0 else (m >> -sh if sh > -64 else 0)
    return -a if b >> 63 else a


def significand63(c):
    # c = m * 2^(e - 63), |m| < 2^63
    if c == 0:
        return 0, 0
    fr, e = math.frexp(c)
    return int(math.ldexp(fr, 63)), e


def fx_term(s, m, d):
    # floor(s * m / 2^d) of the exact product
    return (s * m) >> d


def rn32(x):
    # the integer rounded once to FP32 (to nearest, ties to even), as __ll2float_rn
    a = abs(x)
    if a < 2 ** 24:
        return math.copysign(float(a), x)
    sh = a.bit_length() - 24
    m, rest, half = a >> sh, a & ((1 << sh) - 1), 1 << (sh - 1)
    if rest > half or (rest == half and m & 1):
        m += 1
    return math.copysign(math.ldexp(m, sh), x)


def residual_integer(u, g, f, cx, cy, lam):
    n = u.shape[0]
    eu = max([1] + [bexp(v) for v in u.ravel()] + [bexp(v) for v in g.ravel()])
    ef = max([1] + [bexp(v) for v in f.ravel()])
    cxm, ecx = significand63(cx)
    cym, ecy = significand63(cy)
    lmm, elm = significand63(lam)
    iso, has_lam = cx == cy, lmm != 0
    M = [[fx_shift(u[i, j], eu - 6) for j in range(n)] for i in range(n)]
    G = [[fx_shift(g[s, p], eu - 6) for p in range(n)] for s in range(4)]

    def diffs(i, j):
        c = M[i][j]
        xm = M[i - 1][j] if i > 0 else 2 * G[0][j] - c
        xp = M[i + 1][j] if i < n - 1 else 2 * G[1][j] - c
        ym = M[i][j - 1] if j > 0 else 2 * G[2][i] - c
        yp = M[i][j + 1] if j < n - 1 else 2 * G[3][i] - c
        sx, sy = xm + xp - 2 * c, ym + yp - 2 * c
        return (c, sx + sy, 0) if iso else (c, sx, sy)

    cells = [(i, j) for i in range(n) for j in range(n)]
    d = {ij: diffs(*ij) for ij in cells}
    # bit lengths of the largest second differences (+1, as the kernel's 65 - clz of the OR)
    bx = max(abs(v[1]).bit_length() for v in d.values()) + 1
    by = max(abs(v[2]).bit_length() for v in d.values()) + 1
    top = bx + eu - 1081 + ecx
    if not iso:
        top = max(top, by + eu - 1081 + ecy)
    if has_lam:
        top = max(top, 59 + eu - 1081 + elm)
    sc = max(ef - 1083, top - 61)
    dx, dy, dl = sc - (eu - 1144 + ecx), sc - (eu - 1144 + ecy), sc - (eu - 1144 + elm)
    r, exact_int = np.zeros((n, n)), {}
    for (i, j), (c, sx, sy) in d.items():
        R = (fx_shift(f[i, j], 1075 + sc) if bexp(f[i, j]) else 0) - fx_term(sx, cxm, dx)
        if not iso:
            R -= fx_term(sy, cym, dy)
        if has_lam:
            R -= fx_term(c, lmm, dl)
        assert abs(R) < 2 ** 63
        exact_int[i, j] = R
        r[i, j] = rn32(R) * 2.0 ** sc
    return r, sc, exact_int


def residual_exact(u, g, f, cx, cy, lam):
    n = u.shape[0]
    U = [[Fr(u[i, j]) for j in range(n)] for i in range(n)]
    Gh = [[Fr(g[s, p]) for p in range(n)] for s in range(4)]
    out = {}
    for i in range(n):
        for j in range(n):
            c = U[i][j]
            uw = U[i - 1][j] if i > 0 else 2 * Gh[0][j] - c
            ue = U[i + 1][j] if i < n - 1 else 2 * Gh[1][j] - c
            us = U[i][j - 1] if j > 0 else 2 * Gh[2][i] - c
            un = U[i][j + 1] if j < n - 1 else 2 * Gh[3][i] - c
            out[i, j] = Fr(f[i, j]) - Fr(cx) * (uw + ue - 2 * c) - Fr(cy) * (us + un - 2 * c) - Fr(lam) * c
    return out


def residual_fp64(u, g, f, cx, cy, lam):
    n = u.shape[0]
    up = np.zeros((n + 2, n + 2))
    up[1:-1, 1:-1] = u
    up[0, 1:-1], up[-1, 1:-1] = 2 * g[0] - u[0], 2 * g[1] - u[-1]
    up[1:-1, 0], up[1:-1, -1] = 2 * g[2] - u[:, 0], 2 * g[3] - u[:, -1]
    c = up[1:-1, 1:-1]
    return f - cx * (up[:-2, 1:-1] + up[2:, 1:-1] - 2 * c) - cy * (up[1:-1, :-2] + up[1:-1, 2:] - 2 * c) - lam * c


def smooth_problem(n, cx, cy, lam, scale, seed, zero_f=False):
    # u close to a discrete solution: r is many orders below the stencil terms (the hard case)
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    a, b = rng.uniform(0.5, 2.0, 2)
    u = scale * np.sin(a * X + 0.3) * np.cos(b * Y - 0.2)
    g = scale * np.array([np.sin(0.3) * np.cos(b * x - 0.2), np.sin(a + 0.3) * np.cos(b * x - 0.2),
                          np.sin(a * x + 0.3) * np.cos(-0.2), np.sin(a * x + 0.3) * np.cos(b - 0.2)])
    f = np.zeros((n, n)) if zero_f else residual_fp64(u, g, np.zeros((n, n)), cx, cy, lam) * -1.0
    f = f + scale * 1e-9 * rng.standard_normal((n, n)) if not zero_f else f
    return u, g, f


CASES = [
    ("poisson iso", (2.0 ** 20, 2.0 ** 20, 0.0), 1.0, False),
    ("anisotropic helmholtz", (1.0 / 0.03 ** 2, 1.0 / 0.05 ** 2, -1.0), 1.0, False),
    ("harmonic, f = 0", (1.0 / 0.03 ** 2, 1.0 / 0.05 ** 2, 0.0), 1.0, True),
    ("tiny scale", (1.0 / 0.01 ** 2, 1.0 / 0.01 ** 2, 0.0), 1e-30, False),
    ("huge scale", (1.0 / 0.02 ** 2, 1.0 / 0.02 ** 2, 3.0), 1e25, False),
]


@pytest.mark.parametrize("name,coef,scale,zero_f", CASES, ids=[c[0] for c in CASES])
def test_integer_residual_is_exact_to_fp32_rounding(name, coef, scale, zero_f):
    n = 8
    cx, cy, lam = coef
    u, g, f = smooth_problem(n, cx, cy, lam, scale, 3, zero_f)
    r, sc, R = residual_integer(u, g, f, cx, cy, lam)
    ex = residual_exact(u, g, f, cx, cy, lam)
    term = max(abs(float(Fr(cx) * Fr(u[i, j]))) for i in range(n) for j in range(n))
    rmax = max(abs(float(v)) for v in ex.values())
    fp64 = residual_fp64(u, g, f, cx, cy, lam)
    worst_int = worst_pre = worst_fp64 = 0.0
    for (i, j), v in ex.items():
        e_pre = abs(Fr(R[i, j]) * Fr(2) ** sc - v)
        e_int = abs(Fr(r[i, j]) - v)
        # before the output rounding: the floor shifts and truncations, a few units of 2^sc
        assert e_pre <= 8 * Fr(2) ** sc, (name, i, j)
        # after it: plus the FP32 rounding of r
        assert e_int <= abs(v) * Fr(2) ** -24 + 8 * Fr(2) ** sc, (name, i, j)
        worst_pre = max(worst_pre, float(e_pre) / rmax)
        worst_int = max(worst_int, float(e_int) / rmax)
        worst_fp64 = max(worst_fp64, float(abs(Fr(fp64[i, j]) - v)) / rmax)
    assert 2.0 ** sc <= term * 2.0 ** -56      # the fixed scale sits ~2^-59 below the largest term
    assert worst_int <= 2.0 ** -23              # the output rounding, relative to max |r|
    assert worst_pre <= worst_fp64              # the integer sums lose less than an FP64 stencil
