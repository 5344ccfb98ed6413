// Variable-coefficient leaf patches (FiniteVolumeSolverType::FivePointStencil).
//
// The reference assembles, for every patch, the dense n^2 x n^2 operator of
//     alpha div(beta grad u) + lambda u = f
// with cW = alpha_ij beta_{i-1/2,j} / dx^2, ..., cC = -alpha_ij ((beta_E + beta_W)/dx^2 +
// (beta_N + beta_S)/dy^2) + lambda_ij, subtracts c_side from the diagonal of boundary rows and adds
// -2 c_side g to their right-hand side (FiniteVolumeSolver.cpp:27-223), and LU-factors it with
// PETSc for every solve.  Here the same matrix is factored once per leaf at build time: with cell
// index j + i*n it is banded (bandwidth n); the factorisation runs in a shared-memory window of n+1
// band rows (n^4 work instead of n^6) and its band is kept in HBM for every later solve.
//
// No pivoting.  The matrix is A = D S with D = diag(alpha) and S symmetric (the face couplings
// beta/d^2 are shared by both cells of a face; S_ii = -sum beta/d^2 + lambda/alpha).  Gaussian
// elimination of D S without pivoting produces the pivots alpha_r u_rr(S), and u_rr(S) < 0 for every
// r exactly when S is negative definite -- then elimination without pivoting is backward stable (the
// Cholesky-type bound), whatever lambda's sign.  Every pivot is checked: a pivot with
// pivot * alpha_r >= 0 means S is not negative definite (lambda above the smallest eigenvalue of the
// diffusion part, alpha beta changing sign, alpha = 0), where elimination without pivoting is not
// safe; the factorisation flags it (info = -(r + 1)) and the build refuses the tree instead of
// returning results that could depart from the reference's pivoted LU.  An exact zero pivot is
// flagged as singular (info = r + 1).
//
// Coefficients arrive sampled per cell exactly as the reference samples them (cpp:66-79):
// alpha(x_i, y_j), beta at the four faces (x_i -/+ dx/2, y_j), (x_i, y_j -/+ dy/2), lambda(x_i, y_j).
#include "ef_kernels.cuh"

namespace efgb {

namespace {

// band row r holds columns r-n .. r+n at positions 0 .. 2n
__global__ void __launch_bounds__(256) k_fp_factor(const FpLeaf* __restrict__ leaves) {
    const FpLeaf lf = leaves[blockIdx.x];
    const int n = lf.n, N = n * n, w = 2 * n + 1, nslot = n + 1;
    extern __shared__ double win[];  // nslot rows x w
    double* lm = win + nslot * w;     // n multipliers
    const double dx2 = lf.dx * lf.dx, dy2 = lf.dy * lf.dy;

    // assemble band row r into its window slot (FiniteVolumeSolver.cpp:66-184)
    auto assemble = [&](int r) {
        double* row = win + (r % nslot) * w;
        for (int c = threadIdx.x; c < w; c += blockDim.x) row[c] = 0.0;
        __syncthreads();
        if (threadIdx.x == 0) {
            const int i = r / n, j = r - (r / n) * n;
            const double a = lf.alpha[r];
            const double bW = lf.beta[r], bE = lf.beta[N + r], bS = lf.beta[2 * N + r], bN = lf.beta[3 * N + r];
            const double cW = a * bW / dx2, cE = a * bE / dx2, cS = a * bS / dy2, cN = a * bN / dy2;
            const double cC = -a * ((bE + bW) / dx2 + (bN + bS) / dy2) + lf.lambda[r];
            double d = cC;
            if (i > 0) row[n - n] = cW; else d -= cW;
            if (i < n - 1) row[n + n] = cE; else d -= cE;
            if (j > 0) row[n - 1] = cS; else d -= cS;
            if (j < n - 1) row[n + 1] = cN; else d -= cN;
            row[n] = d;
            // boundary coupling coefficients for the right-hand side f_b = -2 c_side g
            if (i == 0) lf.bcoef[0 * n + j] = cW;
            if (i == n - 1) lf.bcoef[1 * n + j] = cE;
            if (j == 0) lf.bcoef[2 * n + i] = cS;
            if (j == n - 1) lf.bcoef[3 * n + i] = cN;
        }
        __syncthreads();
    };

    for (int r = 0; r <= n && r < N; ++r) assemble(r);
    for (int k = 0; k < N; ++k) {
        const double* pr = win + (k % nslot) * w;  // pivot row k
        const double piv = pr[n];
        const int rows = min(n, N - 1 - k);
        // multipliers l_i = A[k+d][k] / piv for d = 1..rows; A[k+d][k] sits at position n - d
        if (threadIdx.x < rows) {
            const int d = threadIdx.x + 1;
            double* ri = win + ((k + d) % nslot) * w;
            const double l = ri[n - d] / piv;
            lm[threadIdx.x] = l;
            ri[n - d] = l;
        }
        if (threadIdx.x == 0 && *lf.info == 0) {
            if (piv == 0.0) *lf.info = k + 1;
            else if (!(piv * lf.alpha[k] < 0.0)) *lf.info = -(k + 1);  // not (scaled) negative definite
        }
        __syncthreads();
        // A[k+d][k+e] -= l_d * A[k][k+e], e = 1..n  (positions: row k+d at n-d+e, row k at n+e)
        for (int t = threadIdx.x; t < rows * n; t += blockDim.x) {
            const int d = t / n + 1, e = t - (t / n) * n + 1;
            double* ri = win + ((k + d) % nslot) * w;
            ri[n - d + e] -= lm[d - 1] * pr[n + e];
        }
        __syncthreads();
        // row k is final: store it, then bring in row k+n+1
        for (int c = threadIdx.x; c < w; c += blockDim.x) lf.band[(long long)k * w + c] = pr[c];
        __syncthreads();
        if (k + n + 1 < N) assemble(k + n + 1);
    }
}

// One warp per (leaf, right-hand side): y = L^{-1} b, x = U^{-1} y on the stored band.
// MODE LEAF_DTN_COLUMN: g = e_unit, f = 0, write column `unit` of T; LEAF_NEUMANN: g = 0;
// LEAF_SOLVE: write u; LEAF_MAPD2N: write h.
template <int MODE>
__global__ void __launch_bounds__(256) k_fp_solve(const FpLeaf* __restrict__ leaves,
                                                  const LeafItem* __restrict__ items, int nitems) {
    const int warp = int((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (warp >= nitems) return;  // whole warp exits together
    const LeafItem it = items[warp];
    const FpLeaf lf = leaves[it.type];
    const int n = lf.n, N = n * n, w = 2 * n + 1;
    extern __shared__ double ybuf[];
    double* y = ybuf + (threadIdx.x >> 5) * N;
    const double* band = lf.band;

    auto gval = [&](int side, int pos) -> double {
        if (MODE == LEAF_DTN_COLUMN) return (it.unit == side * n + pos) ? 1.0 : 0.0;
        if (MODE == LEAF_NEUMANN) return 0.0;
        return it.g[side * n + pos];
    };
    // right-hand side f + f_boundary (FiniteVolumeSolver.cpp:96-184)
    for (int r = lane; r < N; r += 32) {
        const int i = r / n, j = r - (r / n) * n;
        double v = (MODE != LEAF_DTN_COLUMN && it.f != nullptr) ? it.f[r] : 0.0;
        if (i == 0 || i == n - 1 || j == 0 || j == n - 1) {
            double acc = 0.0;
            bool any = false;
            if (i == 0) { acc = lf.bcoef[j] * gval(0, j); any = true; }
            else if (i == n - 1) { acc = lf.bcoef[n + j] * gval(1, j); any = true; }
            if (j == 0) { const double t = lf.bcoef[2 * n + i] * gval(2, i); acc = any ? acc + t : t; }
            else if (j == n - 1) { const double t = lf.bcoef[3 * n + i] * gval(3, i); acc = any ? acc + t : t; }
            v += -2.0 * acc;
        }
        y[r] = v;
    }
    __syncwarp();
    // forward: y_k -= sum_{d=1..n} L[k][k-d] y_{k-d}
    for (int k = 1; k < N; ++k) {
        double s = 0.0;
        for (int d = lane + 1; d <= n; d += 32)
            if (k - d >= 0) s = fma(band[(long long)k * w + n - d], y[k - d], s);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) y[k] -= s;
        __syncwarp();
    }
    // backward: x_k = (y_k - sum_{e=1..n} U[k][k+e] x_{k+e}) / U[k][k]
    for (int k = N - 1; k >= 0; --k) {
        double s = 0.0;
        for (int e = lane + 1; e <= n; e += 32)
            if (k + e < N) s = fma(band[(long long)k * w + n + e], y[k + e], s);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) y[k] = (y[k] - s) / band[(long long)k * w + n];
        __syncwarp();
    }
    if (MODE == LEAF_SOLVE) {
        for (int r = lane; r < N; r += 32) it.out[r] = y[r];
    } else {
        // Neumann data of FiniteVolumeSolver.cpp:296-353
        const double dtn_x = 2.0 / lf.dx, dtn_y = 2.0 / lf.dy;
        const int m = 4 * n;
        for (int r = lane; r < m; r += 32) {
            const int side = r / n, pos = r - (r / n) * n;
            int cell;
            if (side == 0) cell = pos;
            else if (side == 1) cell = (n - 1) * n + pos;
            else if (side == 2) cell = pos * n;
            else cell = pos * n + n - 1;
            const double gv = gval(side, pos);
            double h;
            if (side == 0) h = dtn_x * (y[cell] - gv);
            else if (side == 1) h = (-dtn_x) * (y[cell] - gv);
            else if (side == 2) h = dtn_y * (y[cell] - gv);
            else h = (-dtn_y) * (y[cell] - gv);
            if (MODE == LEAF_DTN_COLUMN) it.out[(long long)r * m + it.unit] = h;
            else it.out[r] = h;
        }
    }
}

template <int MODE>
void launch_fp_solve(cudaStream_t st, const FpLeaf* leaves, const LeafItem* items, int nitems, int nmax) {
    // one n*n work vector per warp in shared memory (at most 192 KB per CTA)
    const size_t per_warp = size_t(nmax) * nmax * sizeof(double);
    int warps_per_cta = int((192 * 1024) / per_warp);
    if (warps_per_cta > 8) warps_per_cta = 8;
    if (warps_per_cta < 1) warps_per_cta = 1;
    const size_t smem = size_t(warps_per_cta) * per_warp;
    // set on every launch: the attribute is per device and per context, and the call is cheap
    cudaFuncSetAttribute(k_fp_solve<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    const unsigned blocks = unsigned((nitems + warps_per_cta - 1) / warps_per_cta);
    k_fp_solve<MODE><<<blocks, 32 * warps_per_cta, smem, st>>>(leaves, items, nitems);
    ++g_kernel_launches;
}

}  // namespace

void fp_factor(cudaStream_t st, const FpLeaf* leaves, int nleaves, int nmax) {
    if (nleaves <= 0) return;
    const size_t smem = size_t((nmax + 1) * (2 * nmax + 1) + nmax) * sizeof(double);
    cudaFuncSetAttribute(k_fp_factor, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    k_fp_factor<<<nleaves, 256, smem, st>>>(leaves);
    ++g_kernel_launches;
}

void fp_solve(cudaStream_t st, int mode, const FpLeaf* leaves, const LeafItem* items, int nitems, int nmax) {
    if (nitems <= 0) return;
    if (mode == LEAF_DTN_COLUMN) launch_fp_solve<LEAF_DTN_COLUMN>(st, leaves, items, nitems, nmax);
    else if (mode == LEAF_NEUMANN) launch_fp_solve<LEAF_NEUMANN>(st, leaves, items, nitems, nmax);
    else if (mode == LEAF_SOLVE) launch_fp_solve<LEAF_SOLVE>(st, leaves, items, nitems, nmax);
    else launch_fp_solve<LEAF_MAPD2N>(st, leaves, items, nitems, nmax);
}

}  // namespace efgb
