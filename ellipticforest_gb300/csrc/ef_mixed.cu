// Mixed-precision, many-right-hand-side HPS passes.
//
// The plain FP64 form streams S, X^{-1} and H (3.5 GiB at level 7) with one FP64 FMA per 8 bytes
// and is capped by GB300's FP64 pipe.  Here the operators are kept a second time in FP32 and a
// block of B requests is solved at once:
//
//   state   : leaf solutions u (FP64) and the interface values u_Gamma of every merge node (FP64);
//             the leaf Dirichlet data g follow from them exactly (root data, uncoarsening, copies)
//   residual: FP64, no operator matrices -- the 5-point residual r = f + f_b(g) - A u on every leaf
//             cell (FiniteVolumeSolver.cpp:27-223) and, at every merge interface, the mismatch of
//             the coarsened leaf edge fluxes h = +-(2/d)(u_edge - g) of the two sides
//             (FiniteVolumeSolver.cpp:296-353, coarsened with L21 as in HPSAlgorithm.hpp:1024-1048)
//   pass    : one FP32 HPS solve of the correction -- leaf loads r, interface flux jumps -m,
//             homogeneous root data -- whose result is added to the FP64 state.
//
// The first pass starts from a zero state (the residual is then f plus the boundary terms), so
// every pass is the same correction pass.  Node vectors are [len][B] (batch index fastest); leaf
// cell arrays are [B][leaves][n*n].
#include "ef_kernels.cuh"

namespace efgb {

namespace {

__device__ __forceinline__ int mx_lower_child(int I) { return (I == 1) ? 1 : (I == 3 ? 2 : 0); }
__device__ __forceinline__ int mx_upper_child(int I) { return (I == 0) ? 2 : (I == 2 ? 1 : 3); }
__device__ __forceinline__ int mx_q_lower(int I, int o, int s) { return (I < 2 ? 3 * s : s) + o; }
__device__ __forceinline__ int mx_q_upper(int I, int o, int s) { return (I < 2 ? 2 * s : 0) + o; }
__device__ __forceinline__ void mx_ext_map(int p, int s, int& c, int& q) {
    const int side = p / (2 * s);
    const int r = p - side * 2 * s;
    const int hlf = r >= s ? 1 : 0;
    c = side < 2 ? side + 2 * hlf : (side == 2 ? 0 : 2) + hlf;
    q = side * s + (r - hlf * s);
}
__device__ __forceinline__ void mx_child_ifaces(int c, int& Ia, int& Ib) {
    Ia = (c == 0 || c == 2) ? 0 : 1;
    Ib = (c < 2) ? 2 : 3;
}

// ---- FP32 pass, upward ---------------------------------------------------------------------------
// hd = hc_upper - hc_lower - m  (the correction's interface jump)
__global__ void k_mx_hdiff(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int tot = 4 * s * B;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += gridDim.x * blockDim.x) {
        const int r = e / B, b = e - (e / B) * B;
        const int I = r / s, o = r - I * s;
        it.hd[e] = it.hc[mx_upper_child(I)][mx_q_upper(I, o, s) * B + b] -
                   it.hc[mx_lower_child(I)][mx_q_lower(I, o, s) * B + b] - it.m[e];
    }
}

template <int LPR>
__device__ __forceinline__ float group_sumf(float v) {
#pragma unroll
    for (int off = LPR / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// acc[k] += sum_c row[c] * x[c*B + b0 + k], k < BB, over the lanes of one group
template <int LPR, int BB>
__device__ __forceinline__ void mx_dot(const float* __restrict__ row, const float* __restrict__ x, int len,
                                       int B, int b0, int nb, int sl, float* acc) {
    for (int c = sl; c < len; c += LPR) {
        const float a = __ldcs(row + c);
        const float* xc = x + (long long)c * B + b0;
#pragma unroll
        for (int k = 0; k < BB; ++k)
            if (k < nb) acc[k] = fmaf(a, __ldg(xc + k), acc[k]);
    }
}

template <int LPR>
__device__ __forceinline__ long long mx_group_row() {
    return blockIdx.x * (long long)(256 / LPR) + threadIdx.x / LPR;
}

// w = X^{-1} hd
template <int LPR, int BB>
__global__ void __launch_bounds__(256) k_mx_gemv_w(const MixItem* __restrict__ items, int s, long long nrows, int B) {
    const int sl = threadIdx.x & (LPR - 1);
    const long long g = mx_group_row<LPR>();
    const bool ok = g < nrows;
    const int m4 = 4 * s;
    const int item = ok ? int(g / m4) : 0, r = ok ? int(g - (long long)item * m4) : 0;
    const MixItem& it = items[item];
    const int b0 = blockIdx.y * BB, nb = min(BB, B - b0);
    float acc[BB];
#pragma unroll
    for (int k = 0; k < BB; ++k) acc[k] = 0.f;
    if (ok) mx_dot<LPR, BB>(it.Xi + (long long)r * m4, it.hd, m4, B, b0, nb, sl, acc);
#pragma unroll
    for (int k = 0; k < BB; ++k) acc[k] = group_sumf<LPR>(acc[k]);
    if (ok && sl == 0)
        for (int k = 0; k < nb; ++k) it.w[(long long)r * B + b0 + k] = acc[k];
}

// h = H w + h_ext  (compact H rows, WESN order)
template <int LPR, int BB>
__global__ void __launch_bounds__(256) k_mx_gemv_h(const MixItem* __restrict__ items, int s, long long nrows, int B) {
    const int sl = threadIdx.x & (LPR - 1);
    const long long g = mx_group_row<LPR>();
    const bool ok = g < nrows;
    const int m8 = 8 * s;
    const int item = ok ? int(g / m8) : 0, p = ok ? int(g - (long long)item * m8) : 0;
    const MixItem& it = items[item];
    int c, q, Ia, Ib;
    mx_ext_map(p, s, c, q);
    mx_child_ifaces(c, Ia, Ib);
    const int b0 = blockIdx.y * BB, nb = min(BB, B - b0);
    float acc[BB];
#pragma unroll
    for (int k = 0; k < BB; ++k) acc[k] = 0.f;
    if (ok) {
        const float* row = it.H + (long long)p * (2LL * s);
        mx_dot<LPR, BB>(row, it.w + (long long)Ia * s * B, s, B, b0, nb, sl, acc);
        mx_dot<LPR, BB>(row + s, it.w + (long long)Ib * s * B, s, B, b0, nb, sl, acc);
    }
#pragma unroll
    for (int k = 0; k < BB; ++k) acc[k] = group_sumf<LPR>(acc[k]);
    if (ok && sl == 0)
        for (int k = 0; k < nb; ++k)
            it.h[(long long)p * B + b0 + k] = acc[k] + it.hc[c][(long long)q * B + b0 + k];
}

// u = S gf + w, scattered to the children's g and added to the FP64 interface state
template <int LPR, int BB>
__global__ void __launch_bounds__(256) k_mx_gemv_down(const MixItem* __restrict__ items, int s, long long nrows,
                                                      int nitems, int B) {
    const int m4 = 4 * s, m8 = 8 * s;
    if (blockIdx.y == 0) {
        const long long tot = (long long)nitems * m8 * B;
        for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
             e += (long long)gridDim.x * blockDim.x) {
            const int item = int(e / ((long long)m8 * B));
            const int rem = int(e - (long long)item * m8 * B);
            const int p = rem / B, b = rem - (rem / B) * B;
            const MixItem& it = items[item];
            int c, q;
            mx_ext_map(p, s, c, q);
            it.gc[c][q * B + b] = it.gf[rem];
        }
    }
    const int sl = threadIdx.x & (LPR - 1);
    const long long g = mx_group_row<LPR>();
    const bool ok = g < nrows;
    const int item = ok ? int(g / m4) : 0, r = ok ? int(g - (long long)item * m4) : 0;
    const MixItem& it = items[item];
    const int b0 = blockIdx.y * BB, nb = min(BB, B - b0);
    float acc[BB];
#pragma unroll
    for (int k = 0; k < BB; ++k) acc[k] = 0.f;
    if (ok) mx_dot<LPR, BB>(it.S + (long long)r * m8, it.gf, m8, B, b0, nb, sl, acc);
#pragma unroll
    for (int k = 0; k < BB; ++k) acc[k] = group_sumf<LPR>(acc[k]);
    if (ok && sl == 0) {
        const int I = r / s, o = r - I * s;
        float* gl = it.gc[mx_lower_child(I)] + (long long)mx_q_lower(I, o, s) * B;
        float* gu = it.gc[mx_upper_child(I)] + (long long)mx_q_upper(I, o, s) * B;
        for (int k = 0; k < nb; ++k) {
            const float u = acc[k] + it.w[(long long)r * B + b0 + k];
            gl[b0 + k] = u;
            gu[b0 + k] = u;
            it.uG[(long long)r * B + b0 + k] += double(u);
        }
    }
}

// ---- FP64 residual -------------------------------------------------------------------------------
// children's exact Dirichlet data: exterior from the parent, interfaces from the FP64 state
__global__ void k_mx_scatter64(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int m4 = 4 * s, m8 = 8 * s;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < (m8 + m4) * B; e += gridDim.x * blockDim.x) {
        if (e < m8 * B) {
            const int p = e / B, b = e - (e / B) * B;
            int c, q;
            mx_ext_map(p, s, c, q);
            it.gc64[c][q * B + b] = it.gf64[e];
        } else {
            const int f = e - m8 * B;
            const int r = f / B, b = f - (f / B) * B;
            const int I = r / s, o = r - I * s;
            const double v = it.uG[f];
            it.gc64[mx_lower_child(I)][mx_q_lower(I, o, s) * B + b] = v;
            it.gc64[mx_upper_child(I)][mx_q_upper(I, o, s) * B + b] = v;
        }
    }
}

// interface flux mismatch (becomes the next pass's jump) and the node's boundary flux
__global__ void k_mx_flux_up(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int m4 = 4 * s, m8 = 8 * s;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < (m8 + m4) * B; e += gridDim.x * blockDim.x) {
        if (e < m8 * B) {
            const int p = e / B, b = e - (e / B) * B;
            int c, q;
            mx_ext_map(p, s, c, q);
            it.h64[e] = it.hc64[c][q * B + b];
        } else {
            const int f = e - m8 * B;
            const int r = f / B, b = f - (f / B) * B;
            const int I = r / s, o = r - I * s;
            const double ml = it.hc64[mx_lower_child(I)][mx_q_lower(I, o, s) * B + b];
            const double mu = it.hc64[mx_upper_child(I)][mx_q_upper(I, o, s) * B + b];
            it.mout[f] = float(ml - mu);
        }
    }
}

// ---- batched (un)coarsening, [len][B] vectors --------------------------------------------------
template <typename T>
__global__ void k_mx_coarsen(const T* const* vin, T* const* vout, int nf, int B) {
    const T* a = vin[blockIdx.y];
    T* o = vout[blockIdx.y];
    const int nc = nf / 2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 4 * nc * B; e += gridDim.x * blockDim.x) {
        const int r = e / B, b = e - (e / B) * B;
        const int side = r / nc, i = r - side * nc;
        o[e] = T(0.5) * a[(side * nf + 2 * i) * B + b] + T(0.5) * a[(side * nf + 2 * i + 1) * B + b];
    }
}

template <typename T>
__global__ void k_mx_uncoarsen(const T* const* vin, T* const* vout, int nf, int B) {
    const T* a = vin[blockIdx.y];
    T* o = vout[blockIdx.y];
    const int nc = nf / 2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 4 * nf * B; e += gridDim.x * blockDim.x) {
        const int r = e / B, b = e - (e / B) * B;
        const int side = r / nf, c = r - side * nf;
        const T* y = a + side * nc * B + b;
        T v;
        if (c == 0) v = T(1.40625) * y[0] + T(-0.5625) * y[B] + T(0.15625) * y[2 * B];
        else if (c == nf - 1) v = T(0.15625) * y[(nc - 3) * B] + T(-0.5625) * y[(nc - 2) * B] + T(1.40625) * y[(nc - 1) * B];
        else if (c & 1) { const int jp = (c - 1) / 2; v = T(0.75) * y[jp * B] + T(0.25) * y[(jp + 1) * B]; }
        else { const int jp = (c - 2) / 2; v = T(0.25) * y[jp * B] + T(0.75) * y[(jp + 1) * B]; }
        o[e] = v;
    }
}

// ---- leaves --------------------------------------------------------------------------------------
// FP32 eigenbasis leaf pass for (leaf, b): NEUMANN writes h32 = DtN(0, q); SOLVE adds the solution
// of (g32, q) to the FP64 state u64.
template <int MODE>
__global__ void __launch_bounds__(256) k_mx_leaf32(const LeafType32* __restrict__ types,
                                                   const MixLeaf* __restrict__ leaves, int L, int B,
                                                   const float* __restrict__ q, double* __restrict__ u64) {
    const int leaf = blockIdx.x, b = blockIdx.y;
    const MixLeaf lf = leaves[leaf];
    const LeafType32 ty = types[lf.type];
    const int n = ty.n, nn = n * n;
    extern __shared__ float smf[];
    float* V = smf;
    float* F = smf + nn;
    float* W = smf + 2 * nn;
    const int tid = threadIdx.x, nt = blockDim.x;
    const float cx = 1.0f / (ty.dx * ty.dx), cy = 1.0f / (ty.dy * ty.dy);
    const float* qq = q + ((long long)b * L + leaf) * nn;
    for (int e = tid; e < nn; e += nt) {
        V[e] = ty.V[e];
        const int i = e / n, j = e - (e / n) * n;
        float v = qq[e];
        if (MODE == LEAF_SOLVE && (i == 0 || i == n - 1 || j == 0 || j == n - 1)) {
            float acc = 0.f;
            if (i == 0) acc += cx * lf.g32[(0 * n + j) * B + b];
            else if (i == n - 1) acc += cx * lf.g32[(1 * n + j) * B + b];
            if (j == 0) acc += cy * lf.g32[(2 * n + i) * B + b];
            else if (j == n - 1) acc += cy * lf.g32[(3 * n + i) * B + b];
            v += -2.0f * acc;
        }
        F[e] = v;
    }
    __syncthreads();
    for (int e = tid; e < nn; e += nt) {
        const int k = e / n, j = e - (e / n) * n;
        float acc = 0.f;
        for (int i = 0; i < n; ++i) acc = fmaf(V[i * n + k], F[i * n + j], acc);
        W[e] = acc;
    }
    __syncthreads();
    for (int e = tid; e < nn; e += nt) {
        const int k = e / n, l = e - (e / n) * n;
        float acc = 0.f;
        for (int j = 0; j < n; ++j) acc = fmaf(W[k * n + j], V[j * n + l], acc);
        F[e] = acc * ty.Dinv[e];
    }
    __syncthreads();
    for (int e = tid; e < nn; e += nt) {
        const int i = e / n, l = e - (e / n) * n;
        float acc = 0.f;
        for (int k = 0; k < n; ++k) acc = fmaf(V[i * n + k], F[k * n + l], acc);
        W[e] = acc;
    }
    __syncthreads();
    if (MODE == LEAF_SOLVE) {
        double* uu = u64 + ((long long)b * L + leaf) * nn;
        for (int e = tid; e < nn; e += nt) {
            const int i = e / n, j = e - (e / n) * n;
            float acc = 0.f;
            for (int l = 0; l < n; ++l) acc = fmaf(W[i * n + l], V[j * n + l], acc);
            uu[e] += double(acc);
        }
    } else {
        const float dtn_x = 2.0f / ty.dx, dtn_y = 2.0f / ty.dy;
        for (int r = tid; r < 4 * n; r += nt) {
            const int side = r / n, pos = r - (r / n) * n;
            int i, j;
            if (side == 0) { i = 0; j = pos; }
            else if (side == 1) { i = n - 1; j = pos; }
            else if (side == 2) { i = pos; j = 0; }
            else { i = pos; j = n - 1; }
            float u = 0.f;
            for (int l = 0; l < n; ++l) u = fmaf(W[i * n + l], V[j * n + l], u);
            const float sg = (side == 0 || side == 2) ? 1.0f : -1.0f;
            lf.h32[r * B + b] = sg * (side < 2 ? dtn_x : dtn_y) * u;
        }
    }
}

// FP64 leaf residual r = f + f_b(g) - A u (stored as the next pass's FP32 load) and the leaf's edge
// fluxes h = +-(2/d)(u_edge - g) (FP64), for the constant-coefficient operator of FISHPACK90.
__global__ void __launch_bounds__(256) k_mx_leaf_residual(const LeafType* __restrict__ types,
                                                          const MixLeaf* __restrict__ leaves, int L, int B,
                                                          double lambda, const double* __restrict__ f,
                                                          const double* __restrict__ u64, float* __restrict__ q,
                                                          double* __restrict__ rmax) {
    const int leaf = blockIdx.x, b = blockIdx.y;
    const MixLeaf lf = leaves[leaf];
    const LeafType ty = types[lf.type];
    const int n = ty.n, nn = n * n;
    const double cx = 1.0 / (ty.dx * ty.dx), cy = 1.0 / (ty.dy * ty.dy);
    const double cc = -(2.0 * cx + 2.0 * cy) + lambda;
    const long long base = ((long long)b * L + leaf) * nn;
    const double* uu = u64 + base;
    const double* ff = f + base;
    double mx = 0.0;
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        const int i = e / n, j = e - (e / n) * n;
        double d = cc, au = 0.0, fb = 0.0;
        if (i > 0) au = fma(cx, uu[e - n], au); else { d -= cx; fb = fma(cx, lf.g64[(0 * n + j) * B + b], fb); }
        if (i < n - 1) au = fma(cx, uu[e + n], au); else { d -= cx; fb = fma(cx, lf.g64[(1 * n + j) * B + b], fb); }
        if (j > 0) au = fma(cy, uu[e - 1], au); else { d -= cy; fb = fma(cy, lf.g64[(2 * n + i) * B + b], fb); }
        if (j < n - 1) au = fma(cy, uu[e + 1], au); else { d -= cy; fb = fma(cy, lf.g64[(3 * n + i) * B + b], fb); }
        au = fma(d, uu[e], au);
        const double r = ff[e] - 2.0 * fb - au;
        q[base + e] = float(r);
        mx = fmax(mx, fabs(r));
    }
    if (rmax) {
        for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
        if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned long long*>(rmax + b),
                                               __double_as_longlong(mx));
    }
    const double dtn_x = 2.0 / ty.dx, dtn_y = 2.0 / ty.dy;
    for (int r = threadIdx.x; r < 4 * n; r += blockDim.x) {
        const int side = r / n, pos = r - (r / n) * n;
        int cell;
        if (side == 0) cell = pos;
        else if (side == 1) cell = (n - 1) * n + pos;
        else if (side == 2) cell = pos * n;
        else cell = pos * n + n - 1;
        const double gv = lf.g64[r * B + b];
        double h;
        if (side == 0) h = dtn_x * (uu[cell] - gv);
        else if (side == 1) h = (-dtn_x) * (uu[cell] - gv);
        else if (side == 2) h = dtn_y * (uu[cell] - gv);
        else h = (-dtn_y) * (uu[cell] - gv);
        lf.h64[r * B + b] = h;
    }
}

// FP32 copies of S (RHS columns [0,8s)), X^{-1} (RHS columns [8s,12s)) and the compact H
__global__ void k_mx_convert(const MixConv* __restrict__ items, int s) {
    const MixConv& it = items[blockIdx.y];
    const long long m4 = 4LL * s, m12 = 12LL * s;
    const long long nS = m4 * 8 * s, nX = m4 * m4, nH = 16LL * s * s;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nS + nX + nH;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < nS) {
            const long long r = e / (8 * s), c = e - r * (8 * s);
            it.S[e] = float(it.RHS[r * m12 + c]);
        } else if (e < nS + nX) {
            const long long f = e - nS, r = f / m4, c = f - r * m4;
            it.Xi[f] = float(it.RHS[r * m12 + 8 * s + c]);
        } else {
            const long long f = e - nS - nX;
            it.H32[f] = float(it.H[f]);
        }
    }
}

// root Dirichlet data (b == 0): g = r / a per request, [4M][B]
__global__ void k_mx_root(int m, int B, const double* a, const double* r, double* g) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * B; e += gridDim.x * blockDim.x) {
        const int i = e / B, b = e - (e / B) * B;
        g[e] = r[(long long)b * m + i] / a[(long long)b * m + i];
    }
}

inline int mx_pick_lpr(int len) {
    if (len >= 256) return 32;
    if (len >= 64) return 16;
    if (len >= 16) return 8;
    return 4;
}

inline unsigned mx_grid(long long tot) {
    long long b = (tot + 255) / 256;
    if (b > 8192) b = 8192;
    return unsigned(b < 1 ? 1 : b);
}

constexpr int kBB = 8;  // requests accumulated per pass over a matrix row

#define EF_MX_DISPATCH(KERNEL, LPR, GRID, ...)                                        \
    do {                                                                              \
        if (LPR == 32) KERNEL<32, kBB><<<GRID, 256, 0, st>>>(__VA_ARGS__);            \
        else if (LPR == 16) KERNEL<16, kBB><<<GRID, 256, 0, st>>>(__VA_ARGS__);       \
        else if (LPR == 8) KERNEL<8, kBB><<<GRID, 256, 0, st>>>(__VA_ARGS__);         \
        else KERNEL<4, kBB><<<GRID, 256, 0, st>>>(__VA_ARGS__);                       \
    } while (0)

}  // namespace

void mx_up(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    dim3 g1(mx_grid(4LL * s * B), nitems);
    k_mx_hdiff<<<g1, 256, 0, st>>>(items, s, B);
    const int chunks = (B + kBB - 1) / kBB;
    {
        const long long rows = (long long)nitems * 4 * s;
        const int lpr = mx_pick_lpr(4 * s);
        dim3 g((unsigned)((rows * lpr + 255) / 256), chunks);
        EF_MX_DISPATCH(k_mx_gemv_w, lpr, g, items, s, rows, B);
    }
    {
        const long long rows = (long long)nitems * 8 * s;
        const int lpr = mx_pick_lpr(s);
        dim3 g((unsigned)((rows * lpr + 255) / 256), chunks);
        EF_MX_DISPATCH(k_mx_gemv_h, lpr, g, items, s, rows, B);
    }
    g_kernel_launches += 3;
}

void mx_down(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    const int chunks = (B + kBB - 1) / kBB;
    const long long rows = (long long)nitems * 4 * s;
    const int lpr = mx_pick_lpr(8 * s);
    long long blocks = (rows * lpr + 255) / 256;
    if (blocks < 1) blocks = 1;
    dim3 g((unsigned)blocks, chunks);
    EF_MX_DISPATCH(k_mx_gemv_down, lpr, g, items, s, rows, nitems, B);
    ++g_kernel_launches;
}

void mx_scatter64(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    dim3 g(mx_grid(12LL * s * B), nitems);
    k_mx_scatter64<<<g, 256, 0, st>>>(items, s, B);
    ++g_kernel_launches;
}

void mx_flux_up(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    dim3 g(mx_grid(12LL * s * B), nitems);
    k_mx_flux_up<<<g, 256, 0, st>>>(items, s, B);
    ++g_kernel_launches;
}

void mx_coarsen(cudaStream_t st, bool fp64, const void* const* in, void* const* out, int count, int nf, int B) {
    dim3 g(mx_grid(2LL * nf * B), count);
    if (fp64) k_mx_coarsen<double><<<g, 256, 0, st>>>((const double* const*)in, (double* const*)out, nf, B);
    else k_mx_coarsen<float><<<g, 256, 0, st>>>((const float* const*)in, (float* const*)out, nf, B);
    ++g_kernel_launches;
}

void mx_uncoarsen(cudaStream_t st, bool fp64, const void* const* in, void* const* out, int count, int nf, int B) {
    dim3 g(mx_grid(4LL * nf * B), count);
    if (fp64) k_mx_uncoarsen<double><<<g, 256, 0, st>>>((const double* const*)in, (double* const*)out, nf, B);
    else k_mx_uncoarsen<float><<<g, 256, 0, st>>>((const float* const*)in, (float* const*)out, nf, B);
    ++g_kernel_launches;
}

void mx_convert(cudaStream_t st, const MixConv* items, int nitems, int s) {
    dim3 g(mx_grid(36LL * s * s), nitems);
    k_mx_convert<<<g, 256, 0, st>>>(items, s);
    ++g_kernel_launches;
}

void mx_leaf32(cudaStream_t st, int mode, const LeafType32* types, const MixLeaf* leaves, int L, int B, int n,
               const float* q, double* u64) {
    const size_t smem = size_t(3) * n * n * sizeof(float);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_mx_leaf32<LEAF_NEUMANN>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(k_mx_leaf32<LEAF_SOLVE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        configured = true;
    }
    dim3 g(L, B);
    if (mode == LEAF_NEUMANN) k_mx_leaf32<LEAF_NEUMANN><<<g, 256, smem, st>>>(types, leaves, L, B, q, u64);
    else k_mx_leaf32<LEAF_SOLVE><<<g, 256, smem, st>>>(types, leaves, L, B, q, u64);
    ++g_kernel_launches;
}

void mx_leaf_residual(cudaStream_t st, const LeafType* types, const MixLeaf* leaves, int L, int B, double lambda,
                      const double* f, const double* u64, float* q, double* rmax) {
    dim3 g(L, B);
    k_mx_leaf_residual<<<g, 256, 0, st>>>(types, leaves, L, B, lambda, f, u64, q, rmax);
    ++g_kernel_launches;
}

void mx_root(cudaStream_t st, int m, int B, const double* a, const double* r, double* g) {
    k_mx_root<<<mx_grid((long long)m * B), 256, 0, st>>>(m, B, a, r, g);
    ++g_kernel_launches;
}

}  // namespace efgb
