// Mixed-precision passes for variable-coefficient leaves (FiniteVolumeSolverType::FivePointStencil).
//
// The FP64 band LU of every leaf's 5-point operator (factored once at build time, see ef_leaf_fp.cu)
// has bandwidth n, so with the cells split into n blocks of n rows the triangular solves are
//     forward   y_j = L_jj^{-1} (q_j - L_{j,j-1} y_{j-1})
//     backward  x_j = U_jj^{-1} (y_j - U_{j,j+1} x_{j+1})
// At set-up the diagonal blocks are inverted in FP64 and the four n x n blocks of every block row
// are stored in FP32; a block of requests is then solved per leaf by 2n small GEMMs over the
// requests, with the work vectors in shared memory.  The FP64 stencil coefficients cW, cE, cS, cN,
// cC of FiniteVolumeSolver.cpp:66-100 are tabulated per cell for the residual, which uses the same
// ghost treatment as the reference's boundary rows (cpp:100-184): a missing neighbour is 2g - u_C.
#include "ef_kernels.cuh"
#include "ef_mixed_common.cuh"

namespace efgb {

namespace {

// one CTA per leaf: FP32 boundary coefficients, FP64 stencil table
__global__ void __launch_bounds__(256) k_mx_fp_convert(const FpLeaf* __restrict__ src, const MixFp* __restrict__ dst) {
    const FpLeaf lf = src[blockIdx.x];
    const MixFp mf = dst[blockIdx.x];
    const int n = lf.n, N = n * n;
    const double dx2 = lf.dx * lf.dx, dy2 = lf.dy * lf.dy;
    for (int e = threadIdx.x; e < 4 * n; e += blockDim.x) mf.bcoef[e] = float(lf.bcoef[e]);
    for (int r = threadIdx.x; r < N; r += blockDim.x) {
        const double a = lf.alpha[r];
        const double bW = lf.beta[r], bE = lf.beta[N + r], bS = lf.beta[2 * N + r], bN = lf.beta[3 * N + r];
        mf.coef[r] = a * bW / dx2;
        mf.coef[N + r] = a * bE / dx2;
        mf.coef[2 * N + r] = a * bS / dy2;
        mf.coef[3 * N + r] = a * bN / dy2;
        mf.coef[4 * N + r] = -a * ((bE + bW) / dx2 + (bN + bS) / dy2) + lf.lambda[r];
    }
}

// Block rows of the band LU (CTA = (block j, leaf), thread = column k of the n x n blocks), in FP64,
// stored FP32 as blocks[j][4][n][n] = { L_jj^{-1}, L_{j,j-1}, U_jj^{-1}, U_{j,j+1} } (row-major).
// Band row r holds columns r-n .. r+n at positions 0 .. 2n (L multipliers | U).
__global__ void k_mx_fp_blocks(const FpLeaf* __restrict__ src, const MixFp* __restrict__ dst) {
    const FpLeaf lf = src[blockIdx.y];
    const int n = lf.n, w = 2 * n + 1, j = blockIdx.x, k = threadIdx.x;
    if (k >= n) return;
    const double* band = lf.band + (long long)j * n * w;  // first row of block row j
    float* out = dst[blockIdx.y].blocks + (long long)j * 4 * n * n;
    float* Linv = out;
    float* Lsub = out + n * n;
    float* Uinv = out + 2 * n * n;
    float* Usup = out + 3 * n * n;
    // column k of L_jj^{-1} (unit lower): x_a = delta_ak - sum_{b<a} L[a][b] x_b, L[a][b] at n - (a - b)
    double x[64];
    for (int a = 0; a < n; ++a) {
        double v = (a == k) ? 1.0 : 0.0;
        if (a > k)
            for (int bb = k; bb < a; ++bb) v = fma(-band[(long long)a * w + n - (a - bb)], x[bb], v);
        x[a] = a < k ? 0.0 : v;
        Linv[a * n + k] = float(x[a]);
    }
    // column k of U_jj^{-1} (upper): x_a = (delta_ak - sum_{b>a} U[a][b] x_b) / U[a][a], U[a][b] at n + (b - a)
    for (int a = n - 1; a >= 0; --a) {
        double v = (a == k) ? 1.0 : 0.0;
        if (a < k)
            for (int bb = a + 1; bb <= k; ++bb) v = fma(-band[(long long)a * w + n + (bb - a)], x[bb], v);
        x[a] = a > k ? 0.0 : v / band[(long long)a * w + n];
        Uinv[a * n + k] = float(x[a]);
    }
    // off-diagonal blocks: L_{j,j-1}[a][b] (b >= a) at position b - a; U_{j,j+1}[a][b] (b <= a) at 2n + b - a
    for (int a = 0; a < n; ++a) {
        Lsub[a * n + k] = (j > 0 && k >= a) ? float(band[(long long)a * w + (k - a)]) : 0.0f;
        Usup[a * n + k] = (j < n - 1 && k <= a) ? float(band[(long long)a * w + 2 * n + k - a]) : 0.0f;
    }
}

// Block solve of one leaf for a group of BN requests (blockIdx.y): 2n steps, each two n x n x BN
// products with the block matrices staged in shared memory.  NEUMANN: g = 0, load q, write
// h32 = DtN(0, q).  SOLVE: load q + boundary terms of g32, add (or store, accumulate == 0) the
// solution to u64.
template <int MODE>
__global__ void __launch_bounds__(256) k_mx_fp_leaf32(const MixFp* __restrict__ fps, const MixLeaf* __restrict__ leaves,
                                                      int L, int B, int n, int BN, const float* __restrict__ q,
                                                      double* __restrict__ u64, int accumulate) {
    extern __shared__ __align__(16) float fsm[];
    const int N = n * n, ld = BN + 1;
    float* Y = fsm;                 // N x ld
    float* M1 = Y + N * ld;         // n x n
    float* M2 = M1 + n * n;         // n x n
    float* T = M2 + n * n;          // n x ld
    const int leaf = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const int b0 = blockIdx.y * BN, nb = min(BN, B - b0);
    const MixFp mf = fps[leaf];
    const MixLeaf lf = leaves[leaf];
    const long long nn = N;
    // load the group's q: cells along threads (coalesced), transposed into rows x requests
    for (int e = tid; e < N * nb; e += nt) {
        const int bb = e / N, r = e - bb * N;
        Y[r * ld + bb] = q[((long long)(b0 + bb) * L + leaf) * nn + r];
    }
    __syncthreads();
    if (MODE == LEAF_SOLVE) {
        for (int e = tid; e < 4 * n * nb; e += nt) {
            const int bb = e % nb, t = e / nb, side = t / n, pos = t - side * n;
            int r;
            if (side == 0) r = pos;
            else if (side == 1) r = (n - 1) * n + pos;
            else if (side == 2) r = pos * n;
            else r = pos * n + n - 1;
            // a corner cell gets two terms from two threads: add them in a fixed order (side 0/1 first)
            if (side >= 2 && (pos == 0 || pos == n - 1)) continue;
            float v = -2.0f * mf.bcoef[side * n + pos] * lf.g32[(long long)(side * n + pos) * B + b0 + bb];
            if (side < 2 && (pos == 0 || pos == n - 1)) {
                const int s2 = pos == 0 ? 2 : 3, p2 = side == 0 ? 0 : n - 1;
                v += -2.0f * mf.bcoef[s2 * n + p2] * lf.g32[(long long)(s2 * n + p2) * B + b0 + bb];
            }
            Y[r * ld + bb] += v;
        }
        __syncthreads();
    }
    const float* blocks = mf.blocks;
    const int outs = n * nb;
    // one product: dst[a][bb] (= base[a][bb] -) sum_c Mat[a][c] src[c][bb]
    auto gemm = [&](const float* Mat, const float* src, int src_ld, float* dst, int dst_ld, const float* base,
                    int base_ld, bool sub) {
        for (int o = tid; o < outs; o += nt) {
            const int a = o / nb, bb = o - a * nb;
            const float* mr = Mat + a * n;
            float s0 = 0.f, s1 = 0.f;
            int c = 0;
            for (; c + 1 < n; c += 2) {
                s0 = fmaf(mr[c], src[c * src_ld + bb], s0);
                s1 = fmaf(mr[c + 1], src[(c + 1) * src_ld + bb], s1);
            }
            if (c < n) s0 = fmaf(mr[c], src[c * src_ld + bb], s0);
            const float s = s0 + s1;
            dst[a * dst_ld + bb] = sub ? base[a * base_ld + bb] - s : s;
        }
    };
    auto stage = [&](const float* g1, const float* g2) {
        for (int e = tid; e < n * n; e += nt) {
            M1[e] = g1[e];
            M2[e] = g2[e];
        }
    };
    // forward sweep
    for (int j = 0; j < n; ++j) {
        const float* bj = blocks + (long long)j * 4 * n * n;
        stage(bj, bj + n * n);  // L_jj^{-1}, L_{j,j-1}
        __syncthreads();
        float* Yj = Y + j * n * ld;
        if (j > 0) gemm(M2, Yj - n * ld, ld, T, ld, Yj, ld, true);
        else
            for (int o = tid; o < outs; o += nt) { const int a = o / nb, bb = o - a * nb; T[a * ld + bb] = Yj[a * ld + bb]; }
        __syncthreads();
        gemm(M1, T, ld, Yj, ld, nullptr, 0, false);
        __syncthreads();
    }
    // backward sweep
    for (int j = n - 1; j >= 0; --j) {
        const float* bj = blocks + (long long)j * 4 * n * n;
        stage(bj + 2 * n * n, bj + 3 * n * n);  // U_jj^{-1}, U_{j,j+1}
        __syncthreads();
        float* Yj = Y + j * n * ld;
        if (j < n - 1) gemm(M2, Yj + n * ld, ld, T, ld, Yj, ld, true);
        else
            for (int o = tid; o < outs; o += nt) { const int a = o / nb, bb = o - a * nb; T[a * ld + bb] = Yj[a * ld + bb]; }
        __syncthreads();
        gemm(M1, T, ld, Yj, ld, nullptr, 0, false);
        __syncthreads();
    }
    if (MODE == LEAF_SOLVE) {
        for (int e = tid; e < N * nb; e += nt) {
            const int bb = e / N, r = e - bb * N;
            double* dst = u64 + ((long long)(b0 + bb) * L + leaf) * nn + r;
            const double v = f2d_bits(Y[r * ld + bb]);
            *dst = accumulate ? *dst + v : v;
        }
    } else {
        // Neumann data of FiniteVolumeSolver.cpp:296-353 with g = 0
        for (int e = tid; e < 4 * n * nb; e += nt) {
            const int bb = e % nb, t = e / nb, side = t / n, pos = t - side * n;
            int cell;
            if (side == 0) cell = pos;
            else if (side == 1) cell = (n - 1) * n + pos;
            else if (side == 2) cell = pos * n;
            else cell = pos * n + n - 1;
            const float dtn = float(side < 2 ? mf.dtn_x : mf.dtn_y);
            const float sg = (side == 0 || side == 2) ? 1.0f : -1.0f;
            lf.h32[(long long)(side * n + pos) * B + b0 + bb] = sg * dtn * Y[cell * ld + bb];
        }
    }
}

// FP64 residual with the tabulated stencil (see the constant-coefficient kernel in ef_mixed.cu for
// the layout and the two phases): r = f - (cW x_W + cE x_E + cS x_S + cN x_N + cC u_C).
__global__ void __launch_bounds__(256) k_mx_fp_residual(const MixFp* __restrict__ fps, const MixLeaf* __restrict__ leaves,
                                                        int L, int B, int n, int ipc, int zero_state,
                                                        const double* __restrict__ f, const double* __restrict__ u64,
                                                        float* __restrict__ q, float* __restrict__ rleaf) {
    __shared__ unsigned smax[256];
    const int nn = n * n, tpi = nn / 4;
    const int tpe = tpi < 256 ? tpi : 256;
    const int slot = threadIdx.x / tpe, lt = threadIdx.x - slot * tpe;
    const int item = blockIdx.x * ipc + slot;
    const bool act = slot < ipc && (long long)item < (long long)L * B;
    if (threadIdx.x < ipc) smax[threadIdx.x] = 0u;
    __syncthreads();
    const int leaf = act ? item / B : 0;
    const int b = act ? item - leaf * B : 0;
    const MixLeaf lf = leaves[leaf];
    const MixFp mf = fps[leaf];
    const double* cW = mf.coef;
    const double* cE = mf.coef + nn;
    const double* cS = mf.coef + 2 * nn;
    const double* cN = mf.coef + 3 * nn;
    const double* cC = mf.coef + 4 * nn;
    const long long base = ((long long)b * L + leaf) * nn;
    const double* uu = u64 + base;
    const double* ff = f + base;
    float mx = 0.f;
    if (act) {
        for (int e4 = lt; e4 < tpi; e4 += tpe) {
            const int e = 4 * e4, i = e / n, j0 = e - (e / n) * n;
            float rr[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int c = e + t, j = j0 + t;
                double r = ff[c];
                if (!zero_state) {
                    const double uc = uu[c];
                    r = fma(-cC[c], uc, r);
                    if (i > 0) r = fma(-cW[c], uu[c - n], r);
                    if (i < n - 1) r = fma(-cE[c], uu[c + n], r);
                    if (j > 0) r = fma(-cS[c], uu[c - 1], r);
                    if (j < n - 1) r = fma(-cN[c], uu[c + 1], r);
                }
                rr[t] = d2f_rn_bits(r);
            }
            const bool edge_row = i == 0 || i == n - 1;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int j = j0 + t;
                const bool interior = !edge_row && j > 0 && j < n - 1;
                mx = fmaxf(mx, interior ? fabsf(rr[t]) : 0.f);
            }
            *reinterpret_cast<float4*>(q + base + e) = make_float4(rr[0], rr[1], rr[2], rr[3]);
        }
    }
    __syncthreads();  // the boundary phase rewrites cells stored by other threads of the block
    if (act) {
        // Dirichlet data row k of the leaf
        auto gr = [&](int k) { return mx_row<const double>(lf.arena, lf.gsrc[k], B); };
        for (int k = lt; k < 4 * n - 4; k += tpe) {
            int i, j;
            if (k < n) { i = 0; j = k; }
            else if (k < 2 * n) { i = n - 1; j = k - n; }
            else { const int m = k - 2 * n; i = 1 + (m >> 1); j = (m & 1) ? n - 1 : 0; }
            const int c = i * n + j;
            const double uc = zero_state ? 0.0 : uu[c];
            const double xm = i > 0 ? (zero_state ? 0.0 : uu[c - n]) : fma(2.0, gr(j)[b], -uc);
            const double xp = i < n - 1 ? (zero_state ? 0.0 : uu[c + n]) : fma(2.0, gr(n + j)[b], -uc);
            const double ym = j > 0 ? (zero_state ? 0.0 : uu[c - 1]) : fma(2.0, gr(2 * n + i)[b], -uc);
            const double yp = j < n - 1 ? (zero_state ? 0.0 : uu[c + 1]) : fma(2.0, gr(3 * n + i)[b], -uc);
            const double r = fma(-cN[c], yp, fma(-cS[c], ym, fma(-cE[c], xp, fma(-cW[c], xm, fma(-cC[c], uc, ff[c])))));
            const float rf = d2f_rn_bits(r);
            q[base + c] = rf;
            mx = fmaxf(mx, fabsf(rf));
        }
        atomicMax(&smax[slot], __float_as_uint(mx));
        for (int r = lt; r < 4 * n; r += tpe) {
            const int side = r / n, pos = r - (r / n) * n;
            int cell;
            if (side == 0) cell = pos;
            else if (side == 1) cell = (n - 1) * n + pos;
            else if (side == 2) cell = pos * n;
            else cell = pos * n + n - 1;
            const double gv = gr(r)[b];
            const double dtn = (side == 0 || side == 2) ? (side < 2 ? mf.dtn_x : mf.dtn_y)
                                                        : -(side < 2 ? mf.dtn_x : mf.dtn_y);
            lf.h64[(long long)r * B + b] = zero_state ? -dtn * gv : dtn * (uu[cell] - gv);
        }
    }
    __syncthreads();
    if (rleaf && act && lt == 0) rleaf[(long long)b * L + leaf] = __uint_as_float(smax[slot]);
}

}  // namespace

void mx_fp_blocks(cudaStream_t st, const FpLeaf* src, const MixFp* dst, int L, int n) {
    if (L <= 0) return;
    k_mx_fp_blocks<<<dim3(unsigned(n), unsigned(L)), 32 * ((n + 31) / 32), 0, st>>>(src, dst);
    ++g_kernel_launches;
}

void mx_fp_convert(cudaStream_t st, const FpLeaf* src, const MixFp* dst, int L, int n) {
    if (L <= 0) return;
    k_mx_fp_convert<<<L, 256, 0, st>>>(src, dst);
    ++g_kernel_launches;
    mx_fp_blocks(st, src, dst, L, n);
}

int mx_fp_group(int n) { return n <= 16 ? 32 : 16; }

size_t mx_fp_leaf_smem(int n) {
    const int BN = mx_fp_group(n), ld = BN + 1;
    return (size_t(n) * n * ld + 2 * size_t(n) * n + size_t(n) * ld) * sizeof(float);
}

void mx_fp_leaf32(cudaStream_t st, int mode, const MixFp* fps, const MixLeaf* leaves, int L, int B, int n,
                  const float* q, double* u64, int accumulate) {
    const int BN = mx_fp_group(n);
    const size_t smem = mx_fp_leaf_smem(n);
    static size_t configured = 48 * 1024;
    if (smem > configured) {
        cudaFuncSetAttribute(k_mx_fp_leaf32<LEAF_NEUMANN>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        cudaFuncSetAttribute(k_mx_fp_leaf32<LEAF_SOLVE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        configured = smem;
    }
    dim3 grid(unsigned(L), unsigned((B + BN - 1) / BN));
    if (mode == LEAF_NEUMANN)
        k_mx_fp_leaf32<LEAF_NEUMANN><<<grid, 256, smem, st>>>(fps, leaves, L, B, n, BN, q, u64, 0);
    else
        k_mx_fp_leaf32<LEAF_SOLVE><<<grid, 256, smem, st>>>(fps, leaves, L, B, n, BN, q, u64, accumulate);
    ++g_kernel_launches;
}

void mx_fp_residual(cudaStream_t st, const MixFp* fps, const MixLeaf* leaves, int L, int B, int n, int zero_state,
                    const double* f, const double* u64, float* q, float* rleaf, double* rmax) {
    const int tpi = n * n / 4, tpe = tpi < 256 ? tpi : 256, ipc = 256 / tpe;
    const long long items = (long long)L * B;
    const unsigned grid = unsigned((items + ipc - 1) / ipc);
    k_mx_fp_residual<<<grid, unsigned(ipc * tpe), 0, st>>>(fps, leaves, L, B, n, ipc, zero_state, f, u64, q,
                                                           rmax ? rleaf : nullptr);
    ++g_kernel_launches;
    if (rmax) mx_rmax(st, rleaf, L, B, rmax);
}

}  // namespace efgb
