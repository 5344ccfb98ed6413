// Merge (build), upward and downward kernels of the HPS tree, grouped per tree level.
//
// Index maps (see ef_kernels.cuh): interfaces I0..I3 = alpha|gamma, beta|omega, alpha|beta,
// gamma|omega (HPSAlgorithm.hpp:752-788); the lower child of I sees it on its N (I0, I1) or E
// (I2, I3) side, the upper child on its S or W side.  Parent exterior points are WESN with
// W = [alpha_W; gamma_W], E = [beta_E; omega_E], S = [alpha_S; beta_S], N = [gamma_N; omega_N]
// (the pi_WESN = {0,4,2,6,1,3,5,7} reorder of HPSAlgorithm.hpp:979-993).
#include <algorithm>

#include "ef_kernels.cuh"

namespace efgb {

namespace {

__device__ __forceinline__ int lower_child(int I) { return (I == 1) ? 1 : (I == 3 ? 2 : 0); }
__device__ __forceinline__ int upper_child(int I) { return (I == 0) ? 2 : (I == 2 ? 1 : 3); }
__device__ __forceinline__ int q_lower(int I, int o, int s) { return (I < 2 ? 3 * s : s) + o; }
__device__ __forceinline__ int q_upper(int I, int o, int s) { return (I < 2 ? 2 * s : 0) + o; }

// parent exterior index p in [0, 8s) -> (child, child side index)
__device__ __forceinline__ void ext_map(int p, int s, int& c, int& q) {
    const int side = p / (2 * s);
    const int r = p - side * 2 * s;
    const int hlf = r >= s ? 1 : 0;
    const int o = r - hlf * s;
    // W: alpha, gamma; E: beta, omega; S: alpha, beta; N: gamma, omega
    c = side < 2 ? side + 2 * hlf : (side == 2 ? 0 : 2) + hlf;
    q = side * s + o;
}

// child-side index of interface point (I, o) on child c, or -1 if c is not adjacent to I.
__device__ __forceinline__ int iface_q(int c, int I, int o, int s, double& sigma) {
    if (c == lower_child(I)) { sigma = -1.0; return q_lower(I, o, s); }
    if (c == upper_child(I)) { sigma = 1.0; return q_upper(I, o, s); }
    return -1;
}

// the two interfaces adjacent to child c
__device__ __forceinline__ void child_ifaces(int c, int& Ia, int& Ib) {
    // alpha: I0, I2; beta: I1, I2; gamma: I0, I3; omega: I1, I3
    Ia = (c == 0 || c == 2) ? 0 : 1;
    Ib = (c < 2) ? 2 : 3;
}

template <class Real>
__global__ void k_gather_xht(const MergeItemT<Real>* __restrict__ items, int s) {
    const MergeItemT<Real>& it = items[blockIdx.y];
    const long long m2 = 2LL * s, m4 = 4LL * s, m8 = 8LL * s;
    const long long nX = m4 * m4, nH = m8 * m2, nT = m8 * m8;
    const long long tot = nX + nH + nT;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        if (e < nX) {
            const int r = int(e / m4), cc = int(e - (e / m4) * m4);
            const int I = r / s, o = r - I * s, J = cc / s, oj = cc - J * s;
            Real v = Real(0);
            // X(I,J) = -sum_c sigma(I,c) Tc[q(c,I)][q(c,J)]
            const int cl = lower_child(I), cu = upper_child(I);
            double sj;
            int qj = iface_q(cl, J, oj, s, sj);
            if (qj >= 0) v += it.Tc[cl][(long long)q_lower(I, o, s) * m4 + qj];
            qj = iface_q(cu, J, oj, s, sj);
            if (qj >= 0) v -= it.Tc[cu][(long long)q_upper(I, o, s) * m4 + qj];
            it.X[e] = v;
        } else if (e < nX + nH) {
            // compact H: columns [0,s) <-> interface Ia(c(p)), [s,2s) <-> Ib(c(p))
            const long long f = e - nX;
            const int p = int(f / m2), col = int(f - (f / m2) * m2);
            const int seg = col >= s ? 1 : 0, o = col - seg * s;
            int c, q, Ia, Ib;
            ext_map(p, s, c, q);
            child_ifaces(c, Ia, Ib);
            double sg;
            const int qi = iface_q(c, seg ? Ib : Ia, o, s, sg);
            it.H[f] = it.Tc[c][(long long)q * m4 + qi];
        } else {
            const long long f = e - nX - nH;
            const int p = int(f / m8), pp = int(f - (f / m8) * m8);
            int c, q, c2, q2;
            ext_map(p, s, c, q);
            ext_map(pp, s, c2, q2);
            it.T[f] = (c == c2) ? it.Tc[c][(long long)q * m4 + q2] : Real(0);
        }
    }
}

template <class Real>
__global__ void k_gather_rhs(const MergeItemT<Real>* __restrict__ items, int s) {
    const MergeItemT<Real>& it = items[blockIdx.y];
    const long long m4 = 4LL * s, m12 = 12LL * s;
    const long long tot = m4 * m12;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = int(e / m12), col = int(e - (e / m12) * m12);
        const int src = it.perm[r];
        Real v;
        if (col < 8 * s) {
            const int I = src / s, o = src - I * s;
            int c, q;
            ext_map(col, s, c, q);
            double sg;
            const int qi = iface_q(c, I, o, s, sg);
            v = (qi >= 0) ? Real(sg) * it.Tc[c][(long long)qi * m4 + q] : Real(0);
        } else {
            v = (col - 8 * s == src) ? Real(1) : Real(0);
        }
        it.RHS[e] = v;
    }
}

// L12 column j (coarse index) of InterpolationMatrixCoarse2Fine(nf): fine rows and weights.
__device__ __forceinline__ int l12_col(int j, int nf, int* rows, double* w) {
    const int nc = nf / 2;
    int k = 0;
    if (j <= 2) {
        rows[k] = 0;
        w[k++] = (j == 0) ? 1.40625 : (j == 1 ? -0.5625 : 0.15625);
    }
    if (j >= 1) { rows[k] = 2 * j - 1; w[k++] = 0.25; rows[k] = 2 * j; w[k++] = 0.75; }
    if (j <= nc - 2) { rows[k] = 2 * j + 1; w[k++] = 0.75; rows[k] = 2 * j + 2; w[k++] = 0.25; }
    if (j >= nc - 3) {
        rows[k] = nf - 1;
        w[k++] = (j == nc - 3) ? 0.15625 : (j == nc - 2 ? -0.5625 : 1.40625);
    }
    return k;
}

template <class Real>
__global__ void k_coarsen_T(const Real* const* Tin, Real* const* Tout, int nf) {
    const Real* __restrict__ A = Tin[blockIdx.y];
    Real* __restrict__ B = Tout[blockIdx.y];
    const int nc = nf / 2, mf = 4 * nf, mc = 4 * nc;
    const long long tot = (long long)mc * mc;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const int R = int(e / mc), C = int(e - (e / mc) * mc);
        const int a = R / nc, i = R - a * nc, b = C / nc, j = C - b * nc;
        int rows[6];
        double w[6];
        const int k = l12_col(j, nf, rows, w);
        Real acc = Real(0);
        for (int rr = 0; rr < 2; ++rr) {
            const Real* row = A + (long long)(a * nf + 2 * i + rr) * mf + b * nf;
            Real t = Real(0);
            for (int q = 0; q < k; ++q) t = fma(row[rows[q]], Real(w[q]), t);
            acc = fma(Real(0.5), t, acc);
        }
        B[e] = acc;
    }
}

template <class In, class Out>
__global__ void k_convert_batched(const In* const* in, Out* const* out, long long len) {
    const In* a = in[blockIdx.y];
    Out* b = out[blockIdx.y];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len; e += (long long)gridDim.x * blockDim.x)
        b[e] = Out(a[e]);
}

__global__ void k_coarsen_vec(const double* const* vin, double* const* vout, int nf) {
    const double* __restrict__ a = vin[blockIdx.y];
    double* __restrict__ b = vout[blockIdx.y];
    const int nc = nf / 2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 4 * nc; e += gridDim.x * blockDim.x) {
        const int side = e / nc, i = e - side * nc;
        b[e] = 0.5 * a[side * nf + 2 * i] + 0.5 * a[side * nf + 2 * i + 1];
    }
}

__global__ void k_uncoarsen_vec(const double* const* vin, double* const* vout, int nf) {
    const double* __restrict__ a = vin[blockIdx.y];
    double* __restrict__ b = vout[blockIdx.y];
    const int nc = nf / 2;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 4 * nf; e += gridDim.x * blockDim.x) {
        const int side = e / nf, c = e - side * nf;
        const double* y = a + side * nc;
        double v;
        if (c == 0) v = 1.40625 * y[0] + (-0.5625) * y[1] + 0.15625 * y[2];
        else if (c == nf - 1) v = 0.15625 * y[nc - 3] + (-0.5625) * y[nc - 2] + 1.40625 * y[nc - 1];
        else if (c & 1) { const int jp = (c - 1) / 2; v = 0.75 * y[jp] + 0.25 * y[jp + 1]; }
        else { const int jp = (c - 2) / 2; v = 0.25 * y[jp] + 0.75 * y[jp + 1]; }
        b[e] = v;
    }
}

// threads per CTA of the interface GEMVs
constexpr int kGemvThreads = 128;

// Group dot products: LPR consecutive lanes (LPR in {4, 8, 16, 32}) share one matrix row; the
// row is streamed with evict-first loads, the vector is read through L1.
template <int LPR>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
    for (int off = LPR / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// This lane's share of row[0:len) . x[0:len) for one group of LPR lanes (sl = lane within the
// group), where x[i] = xa[i] for i < split and xb[i - split] after (split even when VEC).  Eight
// independent row loads per lane and step keep enough bytes in flight at the occupancy these
// kernels run at (a vector load serving four rows, with four times the registers, ran slower).
// VEC: row, xa and xb 16-byte aligned and len even -> double2 loads.
template <bool VEC, int LPR>
__device__ __forceinline__ double group_dot(const double* __restrict__ row, const double* __restrict__ xa,
                                             const double* __restrict__ xb, int split, int len, int sl) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (VEC) {
        const double2* r2 = reinterpret_cast<const double2*>(row);
        const double2* xa2 = reinterpret_cast<const double2*>(xa);
        const double2* xb2 = reinterpret_cast<const double2*>(xb) - (split >> 1);
        const int n2 = len >> 1, s2 = split >> 1;
        int i = sl;
        for (; i + 7 * LPR < n2; i += 8 * LPR) {
            double2 m[8], v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) m[u] = __ldcs(r2 + i + u * LPR);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = i + u * LPR;
                v[u] = __ldg((k < s2 ? xa2 : xb2) + k);
            }
#pragma unroll
            for (int u = 0; u < 8; u += 4) {
                a0 = fma(m[u].x, v[u].x, a0); a0 = fma(m[u].y, v[u].y, a0);
                a1 = fma(m[u + 1].x, v[u + 1].x, a1); a1 = fma(m[u + 1].y, v[u + 1].y, a1);
                a2 = fma(m[u + 2].x, v[u + 2].x, a2); a2 = fma(m[u + 2].y, v[u + 2].y, a2);
                a3 = fma(m[u + 3].x, v[u + 3].x, a3); a3 = fma(m[u + 3].y, v[u + 3].y, a3);
            }
        }
#pragma unroll 7
        for (; i < n2; i += LPR) {
            const double2 m0 = __ldcs(r2 + i), v0 = __ldg((i < s2 ? xa2 : xb2) + i);
            a0 = fma(m0.x, v0.x, a0); a0 = fma(m0.y, v0.y, a0);
        }
    } else {
        const double* xbs = xb - split;
        int i = sl;
        for (; i + 7 * LPR < len; i += 8 * LPR) {
            double m[8], v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) m[u] = __ldcs(row + i + u * LPR);
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int k = i + u * LPR;
                v[u] = __ldg((k < split ? xa : xbs) + k);
            }
#pragma unroll
            for (int u = 0; u < 8; u += 4) {
                a0 = fma(m[u], v[u], a0);
                a1 = fma(m[u + 1], v[u + 1], a1);
                a2 = fma(m[u + 2], v[u + 2], a2);
                a3 = fma(m[u + 3], v[u + 3], a3);
            }
        }
#pragma unroll 7
        for (; i < len; i += LPR) a0 = fma(__ldcs(row + i), __ldg((i < split ? xa : xbs) + i), a0);
    }
    return (a0 + a1) + (a2 + a3);
}

// hDiff = h_upper - h_lower per interface point (HPSAlgorithm.hpp:1061-1081)
__global__ void k_hdiff(const MergeItem* __restrict__ items, int s) {
    const long long m4 = 4LL * s;
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (e >= m4) return;
    const MergeItem& it = items[b];
    const int r = int(e), I = r / s, o = r - I * s;
    it.hd[r] = it.hc[upper_child(I)][q_upper(I, o, s)] - it.hc[lower_child(I)][q_lower(I, o, s)];
}

// Row handled by this thread's lane group; groups never leave early (full-warp shuffles).
template <int LPR>
__device__ __forceinline__ long long group_row() {
    return blockIdx.x * (long long)(kGemvThreads / LPR) + threadIdx.x / LPR;
}

// w = X^{-1} hDiff (the X^{-1} block of RHS, columns [8s, 12s))
template <bool VEC, int LPR>
__global__ void __launch_bounds__(kGemvThreads) k_gemv_w(const MergeItem* __restrict__ items, int s, long long nrows) {
    const int sl = threadIdx.x & (LPR - 1);
    const long long g = group_row<LPR>();
    const bool ok = g < nrows;
    const int m4 = 4 * s;
    const int item = ok ? int(g / m4) : 0, r = ok ? int(g - (long long)item * m4) : 0;
    const MergeItem& it = items[item];
    const double part = ok ? group_dot<VEC, LPR>(it.RHS + (long long)r * (12LL * s) + 8 * s, it.hd, it.hd, m4, m4, sl) : 0.0;
    const double acc = group_sum<LPR>(part);
    if (ok && sl == 0) it.w[r] = acc;
}

// h = H w + h_update (HPSAlgorithm.hpp:1098-1117), compact H rows already in WESN order; the
// compact H row p is contiguous: its first s entries multiply w on interface Ia, the rest Ib
template <bool VEC, int LPR>
__global__ void __launch_bounds__(kGemvThreads) k_gemv_h(const MergeItem* __restrict__ items, int s, long long nrows) {
    const int sl = threadIdx.x & (LPR - 1);
    const long long g = group_row<LPR>();
    const bool ok = g < nrows;
    const int m8 = 8 * s;
    const int item = ok ? int(g / m8) : 0, p = ok ? int(g - (long long)item * m8) : 0;
    const MergeItem& it = items[item];
    int c, q, Ia, Ib;
    ext_map(p, s, c, q);
    child_ifaces(c, Ia, Ib);
    const double part = ok ? group_dot<VEC, LPR>(it.H + (long long)p * (2LL * s), it.w + Ia * s, it.w + Ib * s, s, 2 * s, sl) : 0.0;
    const double acc = group_sum<LPR>(part);
    if (ok && sl == 0) it.h[p] = acc + it.hc[c][q];
}

// u_Gamma = S g + w (HPSAlgorithm.hpp:1197-1204) scattered to the children's interface data; the
// leading threads also copy the exterior data of the children (HPSAlgorithm.hpp:1214-1227)
template <bool VEC, int LPR>
__global__ void __launch_bounds__(kGemvThreads) k_gemv_down(const MergeItem* __restrict__ items, int s,
                                                            long long nrows, int nitems, int add_w) {
    const int m4 = 4 * s, m8 = 8 * s;
    const long long ext = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (ext < (long long)nitems * m8) {
        const int item = int(ext / m8), p = int(ext - (long long)item * m8);
        const MergeItem& it = items[item];
        int c, q;
        ext_map(p, s, c, q);
        it.gc[c][q] = it.gf[p];
    }
    const int sl = threadIdx.x & (LPR - 1);
    const long long g = group_row<LPR>();
    const bool ok = g < nrows;
    const int item = ok ? int(g / m4) : 0, r = ok ? int(g - (long long)item * m4) : 0;
    const MergeItem& it = items[item];
    const double part = ok ? group_dot<VEC, LPR>(it.RHS + (long long)r * (12LL * s), it.gf, it.gf, m8, m8, sl) : 0.0;
    const double acc = group_sum<LPR>(part);
    if (ok && sl == 0) {
        const double u = add_w ? acc + it.w[r] : acc;
        const int I = r / s, o = r - I * s;
        it.gc[lower_child(I)][q_lower(I, o, s)] = u;
        it.gc[upper_child(I)][q_upper(I, o, s)] = u;
    }
}

// lanes per row for a row of `len` doubles: eight loads per lane where the row allows
inline int pick_lpr(int len, bool vec) {
    const int units = vec ? len / 2 : len;
    if (units >= 256) return 32;
    if (units >= 128) return 16;
    if (units >= 64) return 8;
    return 4;
}

#define EF_LPR_DISPATCH(KERNEL, VEC, LPR, GRID, ...)                                       \
    do {                                                                                    \
        if (LPR == 32) KERNEL<VEC, 32><<<GRID, kGemvThreads, 0, st>>>(__VA_ARGS__);         \
        else if (LPR == 16) KERNEL<VEC, 16><<<GRID, kGemvThreads, 0, st>>>(__VA_ARGS__);    \
        else if (LPR == 8) KERNEL<VEC, 8><<<GRID, kGemvThreads, 0, st>>>(__VA_ARGS__);      \
        else KERNEL<VEC, 4><<<GRID, kGemvThreads, 0, st>>>(__VA_ARGS__);                    \
    } while (0)

__global__ void k_root_diag(int m, const double* a, const double* b, const double* r,
                            const double* h, double* g) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const double bh = (h != nullptr) ? b[i] * h[i] : 0.0;
        g[i] = (r[i] - bh) / a[i];
    }
}

__global__ void k_root_assemble(int m, const double* a, const double* b, const double* T, double* A) {
    const long long tot = (long long)m * m;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = int(e / m), j = int(e - (e / m) * m);
        const double v = b[i] * T[e];
        A[e] = (i == j) ? a[i] + v : v;
    }
}

__global__ void k_root_rhs(int m, const double* b, const double* r, const double* h, const int* perm,
                           double* rhs) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
        const int k = perm[i];
        const double bh = (h != nullptr) ? b[k] * h[k] : 0.0;
        rhs[i] = r[k] - bh;
    }
}

__global__ void k_root_same(int m, const double* a, const double* b, const double* a0, const double* b0,
                            int* flag) {
    __shared__ int diff;
    if (threadIdx.x == 0) diff = 0;
    __syncthreads();
    int d = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x)
        d |= (__double_as_longlong(a[i]) != __double_as_longlong(a0[i])) |
             (__double_as_longlong(b[i]) != __double_as_longlong(b0[i]));
    if (d) atomicOr(&diff, 1);
    __syncthreads();
    if (threadIdx.x == 0) *flag = diff ? 0 : 1;
}

__global__ void k_copy_batched(const double* const* src, double* const* dst, const long long* len) {
    const double* a = src[blockIdx.y];
    double* b = dst[blockIdx.y];
    const long long n = len[blockIdx.y];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        b[e] = a[e];
}

__global__ void k_fill_zero(double* p, long long n) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        p[e] = 0.0;
}

inline int grid_for(long long tot, int per_item_items) {
    long long b = (tot + 255) / 256;
    if (b > 4096) b = 4096;
    if (b < 1) b = 1;
    (void)per_item_items;
    return int(b);
}

}  // namespace

template <class Real>
void gather_xht_t(cudaStream_t st, const MergeItemT<Real>* items, int nitems, int s) {
    const long long tot = 16LL * s * s + 32LL * s * s + 64LL * s * s;
    dim3 g(grid_for(tot, nitems), nitems);
    k_gather_xht<Real><<<g, 256, 0, st>>>(items, s);
    ++g_kernel_launches;
}

template <class Real>
void gather_rhs_t(cudaStream_t st, const MergeItemT<Real>* items, int nitems, int s) {
    const long long tot = 48LL * s * s;
    dim3 g(grid_for(tot, nitems), nitems);
    k_gather_rhs<Real><<<g, 256, 0, st>>>(items, s);
    ++g_kernel_launches;
}

template <class Real>
void coarsen_T_t(cudaStream_t st, const Real* const* Tin, Real* const* Tout, int nitems, int nf) {
    const long long tot = 4LL * nf * 4LL * nf / 4;
    dim3 g(grid_for(tot, nitems), nitems);
    k_coarsen_T<Real><<<g, 256, 0, st>>>(Tin, Tout, nf);
    ++g_kernel_launches;
}

void merge_gather_xht(cudaStream_t st, const MergeItem* items, int nitems, int s) { gather_xht_t(st, items, nitems, s); }
void merge_gather_rhs(cudaStream_t st, const MergeItem* items, int nitems, int s) { gather_rhs_t(st, items, nitems, s); }
void coarsen_T(cudaStream_t st, const double* const* Tin, double* const* Tout, int nitems, int nf) {
    coarsen_T_t(st, Tin, Tout, nitems, nf);
}
void merge_gather_xht32(cudaStream_t st, const MergeItem32* items, int nitems, int s) {
    gather_xht_t(st, items, nitems, s);
}
void merge_gather_rhs32(cudaStream_t st, const MergeItem32* items, int nitems, int s) {
    gather_rhs_t(st, items, nitems, s);
}
void coarsen_T32(cudaStream_t st, const float* const* Tin, float* const* Tout, int nitems, int nf) {
    coarsen_T_t(st, Tin, Tout, nitems, nf);
}
void widen_batched(cudaStream_t st, const float* const* in, double* const* out, long long len, int count) {
    if (count <= 0) return;
    k_convert_batched<float, double><<<dim3(grid_for(len, count), count), 256, 0, st>>>(in, out, len);
    ++g_kernel_launches;
}
void narrow_batched(cudaStream_t st, const double* const* in, float* const* out, long long len, int count) {
    if (count <= 0) return;
    k_convert_batched<double, float><<<dim3(grid_for(len, count), count), 256, 0, st>>>(in, out, len);
    ++g_kernel_launches;
}

void coarsen_vec(cudaStream_t st, const double* const* vin, double* const* vout, int nitems, int nf) {
    dim3 g((2 * nf + 255) / 256, nitems);
    k_coarsen_vec<<<g, 256, 0, st>>>(vin, vout, nf);
    ++g_kernel_launches;
}

void uncoarsen_vec(cudaStream_t st, const double* const* vin, double* const* vout, int nitems, int nf) {
    dim3 g((4 * nf + 255) / 256, nitems);
    k_uncoarsen_vec<<<g, 256, 0, st>>>(vin, vout, nf);
    ++g_kernel_launches;
}

void upward_hdiff(cudaStream_t st, const MergeItem* items, int nitems, int s) {
    dim3 g((4 * s + 255) / 256, nitems);
    k_hdiff<<<g, 256, 0, st>>>(items, s);
    ++g_kernel_launches;
}

inline unsigned gemv_blocks(long long threads) {
    return unsigned(std::max(1LL, (threads + kGemvThreads - 1) / kGemvThreads));
}

void upward_w(cudaStream_t st, const MergeItem* items, int nitems, int s) {
    const long long rows = (long long)nitems * 4 * s;
    const bool vec = (s % 2 == 0);
    const int lpr = pick_lpr(4 * s, vec);
    if (vec) EF_LPR_DISPATCH(k_gemv_w, true, lpr, gemv_blocks(rows * lpr), items, s, rows);
    else EF_LPR_DISPATCH(k_gemv_w, false, lpr, gemv_blocks(rows * lpr), items, s, rows);
    ++g_kernel_launches;
}

void upward_h(cudaStream_t st, const MergeItem* items, int nitems, int s) {
    const long long rows = (long long)nitems * 8 * s;
    const bool vec = (s % 2 == 0);
    const int lpr = pick_lpr(2 * s, vec);
    if (vec) EF_LPR_DISPATCH(k_gemv_h, true, lpr, gemv_blocks(rows * lpr), items, s, rows);
    else EF_LPR_DISPATCH(k_gemv_h, false, lpr, gemv_blocks(rows * lpr), items, s, rows);
    ++g_kernel_launches;
}

// the grid also covers the exterior copy (one element per thread)
void downward(cudaStream_t st, const MergeItem* items, int nitems, int s, int add_w) {
    const long long rows = (long long)nitems * 4 * s;
    const bool vec = (s % 2 == 0);
    const int lpr = pick_lpr(8 * s, vec);
    const unsigned nb = gemv_blocks(std::max(rows * lpr, (long long)nitems * 8 * s));
    if (vec) EF_LPR_DISPATCH(k_gemv_down, true, lpr, nb, items, s, rows, nitems, add_w);
    else EF_LPR_DISPATCH(k_gemv_down, false, lpr, nb, items, s, rows, nitems, add_w);
    ++g_kernel_launches;
}

void root_diag(cudaStream_t st, int m, const double* a, const double* b, const double* r,
               const double* h, double* g) {
    k_root_diag<<<(m + 255) / 256, 256, 0, st>>>(m, a, b, r, h, g);
    ++g_kernel_launches;
}

void root_assemble(cudaStream_t st, int m, const double* a, const double* b, const double* T, double* A) {
    k_root_assemble<<<grid_for((long long)m * m, 1), 256, 0, st>>>(m, a, b, T, A);
    ++g_kernel_launches;
}

void root_rhs(cudaStream_t st, int m, const double* b, const double* r, const double* h,
              const int* perm, double* rhs) {
    k_root_rhs<<<(m + 255) / 256, 256, 0, st>>>(m, b, r, h, perm, rhs);
    ++g_kernel_launches;
}

void root_same(cudaStream_t st, int m, const double* a, const double* b, const double* a0, const double* b0,
               int* flag) {
    k_root_same<<<1, 1024, 0, st>>>(m, a, b, a0, b0, flag);
    ++g_kernel_launches;
}

void copy_batched(cudaStream_t st, const double* const* src, double* const* dst, const long long* len, int count) {
    for (int k0 = 0; k0 < count; k0 += 65535) {
        const int c = count - k0 < 65535 ? count - k0 : 65535;
        k_copy_batched<<<dim3(64, c), 256, 0, st>>>(src + k0, dst + k0, len + k0);
        ++g_kernel_launches;
    }
}

void fill_zero(cudaStream_t st, double* p, long long n) {
    if (n > 0) {
        k_fill_zero<<<grid_for(n, 1), 256, 0, st>>>(p, n);
        ++g_kernel_launches;
    }
}

}  // namespace efgb
