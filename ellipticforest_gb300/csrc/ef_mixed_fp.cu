// Mixed-precision passes for variable-coefficient leaves (FiniteVolumeSolverType::FivePointStencil).
//
// The FP64 band LU of every leaf's 5-point operator (factored once at build time, see ef_leaf_fp.cu)
// is copied to FP32 with the diagonal of U stored inverted, and the FP64 stencil coefficients
// cW, cE, cS, cN, cC of FiniteVolumeSolver.cpp:66-100 are tabulated per cell.  A block of B requests
// is then solved per leaf with one lane per request: the band rows are read once per leaf and
// shared by the block, the work vectors of the block live in shared memory.  The FP64 residual uses
// the tabulated coefficients with the same ghost treatment as the reference's boundary rows
// (cpp:100-184): a missing neighbour is 2g - u_C.
#include "ef_kernels.cuh"

namespace efgb {

namespace {

__device__ __forceinline__ double f2d_bits_fp(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
    if (e == 0) return __longlong_as_double((long long)sign);
    const unsigned long long e64 = e == 0xffu ? 0x7ffull : (unsigned long long)(e + 896u);
    return __longlong_as_double((long long)(sign | (e64 << 52) | ((unsigned long long)(b & 0x7fffffu) << 29)));
}
__device__ __forceinline__ float d2f_bits_fp(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = int((b >> 52) & 0x7ffull);
    const unsigned m = (unsigned)((b >> 29) & 0x7fffffull);
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));
    const int e32 = e - 896;
    if (e32 <= 0) return __uint_as_float(sign);
    if (e32 >= 255) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned)e32 << 23) | m);
}

// one CTA per leaf: FP32 band (inverted U diagonal), FP32 boundary coefficients, FP64 stencil table
__global__ void __launch_bounds__(256) k_mx_fp_convert(const FpLeaf* __restrict__ src, const MixFp* __restrict__ dst) {
    const FpLeaf lf = src[blockIdx.x];
    const MixFp mf = dst[blockIdx.x];
    const int n = lf.n, N = n * n, w = 2 * n + 1;
    const double dx2 = lf.dx * lf.dx, dy2 = lf.dy * lf.dy;
    for (long long e = threadIdx.x; e < (long long)N * w; e += blockDim.x) {
        const long long row = e / w, col = e - row * w;
        const double v = lf.band[e];
        mf.band[e] = float(col == n ? 1.0 / v : v);
        (void)row;
    }
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

constexpr int kFpLanes = 32;   // requests per CTA (one lane each)
constexpr int kFpPad = 33;     // row stride of the shared work array (conflict-free transposes)

// FP32 band solves of one leaf for up to 32 requests (blockIdx.y selects the group of 32).
// NEUMANN: g = 0, load q, write h32 = DtN(0, q).  SOLVE: load q + boundary terms of g32, add (or
// store, accumulate == 0) the solution to u64.
template <int MODE>
__global__ void __launch_bounds__(32) k_mx_fp_leaf32(const MixFp* __restrict__ fps, const MixLeaf* __restrict__ leaves,
                                                     int L, int B, int n, const float* __restrict__ q,
                                                     double* __restrict__ u64, int accumulate) {
    extern __shared__ float ys[];  // N rows x kFpPad
    const int leaf = blockIdx.x, lane = threadIdx.x;
    const int b0 = blockIdx.y * kFpLanes, nb = min(kFpLanes, B - b0);
    const int b = b0 + lane;
    const bool act = lane < nb;
    const MixFp mf = fps[leaf];
    const MixLeaf lf = leaves[leaf];
    const int N = n * n, w = 2 * n + 1;
    const long long nn = N;
    // load the block's q (coalesced along cells, transposed into rows x requests)
    for (int r0 = 0; r0 < N; r0 += 32) {
        const int r = r0 + lane;
        for (int bb = 0; bb < nb; ++bb)
            if (r < N) ys[r * kFpPad + bb] = q[((long long)(b0 + bb) * L + leaf) * nn + r];
    }
    __syncwarp();
    if (MODE == LEAF_SOLVE && act) {
        for (int side = 0; side < 4; ++side)
            for (int pos = 0; pos < n; ++pos) {
                int r;
                if (side == 0) r = pos;
                else if (side == 1) r = (n - 1) * n + pos;
                else if (side == 2) r = pos * n;
                else r = pos * n + n - 1;
                ys[r * kFpPad + lane] += -2.0f * mf.bcoef[side * n + pos] * lf.g32[(long long)(side * n + pos) * B + b];
            }
    }
    __syncwarp();
    const float* band = mf.band;
    // forward: y_k -= sum_{d=1..n} L[k][k-d] y_{k-d}
    for (int k = 1; k < N; ++k) {
        const float* row = band + (long long)k * w + n;
        float s0 = 0.f, s1 = 0.f;
        const int dmax = min(n, k);
        int d = 1;
        for (; d + 1 <= dmax; d += 2) {
            s0 = fmaf(__ldg(row - d), ys[(k - d) * kFpPad + lane], s0);
            s1 = fmaf(__ldg(row - d - 1), ys[(k - d - 1) * kFpPad + lane], s1);
        }
        if (d <= dmax) s0 = fmaf(__ldg(row - d), ys[(k - d) * kFpPad + lane], s0);
        ys[k * kFpPad + lane] -= s0 + s1;
    }
    // backward: x_k = (y_k - sum_{e=1..n} U[k][k+e] x_{k+e}) * (1 / U[k][k])
    for (int k = N - 1; k >= 0; --k) {
        const float* row = band + (long long)k * w + n;
        float s0 = 0.f, s1 = 0.f;
        const int emax = min(n, N - 1 - k);
        int e = 1;
        for (; e + 1 <= emax; e += 2) {
            s0 = fmaf(__ldg(row + e), ys[(k + e) * kFpPad + lane], s0);
            s1 = fmaf(__ldg(row + e + 1), ys[(k + e + 1) * kFpPad + lane], s1);
        }
        if (e <= emax) s0 = fmaf(__ldg(row + e), ys[(k + e) * kFpPad + lane], s0);
        ys[k * kFpPad + lane] = (ys[k * kFpPad + lane] - (s0 + s1)) * __ldg(row);
    }
    __syncwarp();
    if (MODE == LEAF_SOLVE) {
        for (int r0 = 0; r0 < N; r0 += 32) {
            const int r = r0 + lane;
            if (r >= N) continue;
            for (int bb = 0; bb < nb; ++bb) {
                double* dst = u64 + ((long long)(b0 + bb) * L + leaf) * nn + r;
                const double v = f2d_bits_fp(ys[r * kFpPad + bb]);
                *dst = accumulate ? *dst + v : v;
            }
        }
    } else if (act) {
        // Neumann data of FiniteVolumeSolver.cpp:296-353 with g = 0
        for (int side = 0; side < 4; ++side)
            for (int pos = 0; pos < n; ++pos) {
                int cell;
                if (side == 0) cell = pos;
                else if (side == 1) cell = (n - 1) * n + pos;
                else if (side == 2) cell = pos * n;
                else cell = pos * n + n - 1;
                const float dtn = float(side < 2 ? mf.dtn_x : mf.dtn_y);
                const float sg = (side == 0 || side == 2) ? 1.0f : -1.0f;
                lf.h32[(long long)(side * n + pos) * B + b] = sg * dtn * ys[cell * kFpPad + lane];
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
                rr[t] = d2f_bits_fp(r);
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
        const double* gW = lf.g64 + b;
        const double* gE = lf.g64 + (long long)n * B + b;
        const double* gS = lf.g64 + 2LL * n * B + b;
        const double* gN = lf.g64 + 3LL * n * B + b;
        for (int k = lt; k < 4 * n - 4; k += tpe) {
            int i, j;
            if (k < n) { i = 0; j = k; }
            else if (k < 2 * n) { i = n - 1; j = k - n; }
            else { const int m = k - 2 * n; i = 1 + (m >> 1); j = (m & 1) ? n - 1 : 0; }
            const int c = i * n + j;
            const double uc = zero_state ? 0.0 : uu[c];
            const double xm = i > 0 ? (zero_state ? 0.0 : uu[c - n]) : fma(2.0, gW[(long long)j * B], -uc);
            const double xp = i < n - 1 ? (zero_state ? 0.0 : uu[c + n]) : fma(2.0, gE[(long long)j * B], -uc);
            const double ym = j > 0 ? (zero_state ? 0.0 : uu[c - 1]) : fma(2.0, gS[(long long)i * B], -uc);
            const double yp = j < n - 1 ? (zero_state ? 0.0 : uu[c + 1]) : fma(2.0, gN[(long long)i * B], -uc);
            const double r = fma(-cN[c], yp, fma(-cS[c], ym, fma(-cE[c], xp, fma(-cW[c], xm, fma(-cC[c], uc, ff[c])))));
            const float rf = d2f_bits_fp(r);
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
            const double gv = lf.g64[(long long)r * B + b];
            const double dtn = (side == 0 || side == 2) ? (side < 2 ? mf.dtn_x : mf.dtn_y)
                                                        : -(side < 2 ? mf.dtn_x : mf.dtn_y);
            lf.h64[(long long)r * B + b] = zero_state ? -dtn * gv : dtn * (uu[cell] - gv);
        }
    }
    __syncthreads();
    if (rleaf && act && lt == 0) rleaf[(long long)b * L + leaf] = __uint_as_float(smax[slot]);
}

}  // namespace

void mx_fp_convert(cudaStream_t st, const FpLeaf* src, const MixFp* dst, int L) {
    if (L <= 0) return;
    k_mx_fp_convert<<<L, 256, 0, st>>>(src, dst);
    ++g_kernel_launches;
}

size_t mx_fp_leaf_smem(int n) { return size_t(n) * n * kFpPad * sizeof(float); }

void mx_fp_leaf32(cudaStream_t st, int mode, const MixFp* fps, const MixLeaf* leaves, int L, int B, int n,
                  const float* q, double* u64, int accumulate) {
    const size_t smem = mx_fp_leaf_smem(n);
    static size_t configured = 48 * 1024;
    if (smem > configured) {
        cudaFuncSetAttribute(k_mx_fp_leaf32<LEAF_NEUMANN>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        cudaFuncSetAttribute(k_mx_fp_leaf32<LEAF_SOLVE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        configured = smem;
    }
    dim3 grid(unsigned(L), unsigned((B + kFpLanes - 1) / kFpLanes));
    if (mode == LEAF_NEUMANN)
        k_mx_fp_leaf32<LEAF_NEUMANN><<<grid, kFpLanes, smem, st>>>(fps, leaves, L, B, n, q, u64, 0);
    else
        k_mx_fp_leaf32<LEAF_SOLVE><<<grid, kFpLanes, smem, st>>>(fps, leaves, L, B, n, q, u64, accumulate);
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
