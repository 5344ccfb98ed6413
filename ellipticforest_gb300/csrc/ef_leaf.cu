// Leaf patch kernels: batched fast solves of the cell-centred 5-point Helmholtz system
//     u_xx + u_yy + lambda u = f   on an n x n patch, Dirichlet data g on the cell faces,
// i.e. the system FISHPACK90 hstcrt_ solves for FiniteVolumeSolver (FiniteVolumeSolver.cpp:224-290)
// and that the FivePointStencil branch assembles with alpha = beta = 1 (cpp:27-223): interior
// 5-point stencil, ghost value u_ghost = 2g - u, boundary right-hand side f -= 2 c_side g.
//
// With the ghost rule the 1-D operator (1/h^2) tridiag(1,-2,1) with -3 in both corners has the
// orthonormal eigenvectors V[i][k] = c_k sin(pi (k+1) (i+1/2) / n) and eigenvalues
// mu_k = -(4/h^2) sin^2(pi (k+1) / (2n)), so the patch solve is four dense n x n contractions:
//     U = V [ (V^T F V) ./ (mu_x[k] + mu_y[l] + lambda) ] V^T.
// The Neumann data follow FiniteVolumeSolver.cpp:296-353: h_W = (2/dx)(u_W - g_W),
// h_E = -(2/dx)(u_E - g_E), h_S = (2/dy)(u_S - g_S), h_N = -(2/dy)(u_N - g_N).
#include <cmath>
#include <stdexcept>

#include "ef_kernels.cuh"

namespace efgb {

namespace {

template <int MODE>
__global__ void __launch_bounds__(256) k_leaf_eigen(const LeafType* __restrict__ types,
                                                    const LeafItem* __restrict__ items) {
    const LeafItem it = items[blockIdx.x];
    const LeafType ty = types[it.type];
    const int n = ty.n, nn = n * n;
    extern __shared__ double sm[];
    double* V = sm;
    double* F = sm + nn;
    double* W = sm + 2 * nn;
    const int tid = threadIdx.x, nt = blockDim.x;
    const double cx = 1.0 / (ty.dx * ty.dx), cy = 1.0 / (ty.dy * ty.dy);

    // boundary value of side `side` at position `pos` (WESN)
    auto gval = [&](int side, int pos) -> double {
        if (MODE == LEAF_DTN_COLUMN) return (it.unit == side * n + pos) ? 1.0 : 0.0;
        if (MODE == LEAF_NEUMANN) return 0.0;
        return it.g[side * n + pos];
    };

    for (int e = tid; e < nn; e += nt) {
        V[e] = ty.V[e];
        const int i = e / n, j = e - (e / n) * n;
        double v = (MODE != LEAF_DTN_COLUMN && it.f != nullptr) ? it.f[e] : 0.0;
        if (MODE != LEAF_NEUMANN && (i == 0 || i == n - 1 || j == 0 || j == n - 1)) {
            // f_boundary = -2 (c_x g_x + c_y g_y)  (FiniteVolumeSolver.cpp:100-184)
            double acc = 0.0;
            bool any = false;
            if (i == 0) { acc = cx * gval(0, j); any = true; }
            else if (i == n - 1) { acc = cx * gval(1, j); any = true; }
            if (j == 0) { const double t = cy * gval(2, i); acc = any ? acc + t : t; }
            else if (j == n - 1) { const double t = cy * gval(3, i); acc = any ? acc + t : t; }
            v += -2.0 * acc;
        }
        F[e] = v;
    }
    __syncthreads();
    // W = V^T F
    for (int e = tid; e < nn; e += nt) {
        const int k = e / n, j = e - (e / n) * n;
        double acc = 0.0;
        for (int i = 0; i < n; ++i) acc = fma(V[i * n + k], F[i * n + j], acc);
        W[e] = acc;
    }
    __syncthreads();
    // F = (W V) ./ D
    for (int e = tid; e < nn; e += nt) {
        const int k = e / n, l = e - (e / n) * n;
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc = fma(W[k * n + j], V[j * n + l], acc);
        F[e] = acc * ty.Dinv[e];
    }
    __syncthreads();
    // W = V F
    for (int e = tid; e < nn; e += nt) {
        const int i = e / n, l = e - (e / n) * n;
        double acc = 0.0;
        for (int k = 0; k < n; ++k) acc = fma(V[i * n + k], F[k * n + l], acc);
        W[e] = acc;
    }
    __syncthreads();
    if (MODE == LEAF_SOLVE) {
        // U = W V^T
        for (int e = tid; e < nn; e += nt) {
            const int i = e / n, j = e - (e / n) * n;
            double acc = 0.0;
            for (int l = 0; l < n; ++l) acc = fma(W[i * n + l], V[j * n + l], acc);
            it.out[e] = acc;
        }
    } else {
        // edge cells only: u[0][j], u[n-1][j], u[i][0], u[i][n-1]
        const double dtn_x = 2.0 / ty.dx, dtn_y = 2.0 / ty.dy;
        const int m = 4 * n;
        for (int r = tid; r < m; r += nt) {
            const int side = r / n, pos = r - (r / n) * n;
            int i, j;
            if (side == 0) { i = 0; j = pos; }
            else if (side == 1) { i = n - 1; j = pos; }
            else if (side == 2) { i = pos; j = 0; }
            else { i = pos; j = n - 1; }
            double u = 0.0;
            for (int l = 0; l < n; ++l) u = fma(W[i * n + l], V[j * n + l], u);
            const double gv = gval(side, pos);
            double h;
            if (side == 0) h = dtn_x * (u - gv);
            else if (side == 1) h = (-dtn_x) * (u - gv);
            else if (side == 2) h = dtn_y * (u - gv);
            else h = (-dtn_y) * (u - gv);
            if (MODE == LEAF_DTN_COLUMN) it.out[(long long)r * m + it.unit] = h;
            else it.out[r] = h;
        }
    }
}

// ---- 16 x 16 leaves: register-resident sine transforms in FP64 ---------------------------------------
// V[15 - i][k] = (-1)^k V[i][k], and for the odd modes k = 2m + 1 also V[7 - i][k] = (-1)^m V[i][k]
// (those columns are the 8-point basis), so rows 0..7 of V (constant memory: the FMA's constant
// operand) define the basis and a 16-point transform costs 96 FMAs and 24 additions instead of 256
// FMAs: the FP64 pipe (about 2 FMAs per clock per SM) bounds these passes.
__constant__ double c_V16d[8 * 16];

// X[k] = sum_j V[j][k] x[j]; out(k, X[k])
template <class Out>
__device__ __forceinline__ void dst16d_fwd(const double (&x)[16], Out&& out) {
    double P[8], M[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        P[j] = x[j] + x[15 - j];
        M[j] = x[j] - x[15 - j];
    }
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
        double a = 0.0;
#pragma unroll
        for (int j = 0; j < 8; ++j) a = fma(c_V16d[j * 16 + k], P[j], a);
        out(k, a);
    }
    double Q[4], R[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        Q[j] = M[j] + M[7 - j];
        R[j] = M[j] - M[7 - j];
    }
#pragma unroll
    for (int k = 1; k < 16; k += 2) {
        const bool modd = ((k >> 1) & 1) != 0;  // k = 2m + 1 with m odd
        double a = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) a = fma(c_V16d[j * 16 + k], modd ? R[j] : Q[j], a);
        out(k, a);
    }
}
// x[i], x[15 - i], x[7 - i], x[8 + i] (i < 4) of x = V X
__device__ __forceinline__ void dst16d_quad(const double (&X)[16], int i, double& a, double& b, double& c,
                                            double& d) {
    double ei = 0.0, e7 = 0.0, oe = 0.0, oo = 0.0;
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
        ei = fma(c_V16d[i * 16 + k], X[k], ei);
        e7 = fma(c_V16d[(7 - i) * 16 + k], X[k], e7);
    }
#pragma unroll
    for (int k = 1; k < 16; k += 4) {
        oe = fma(c_V16d[i * 16 + k], X[k], oe);
        oo = fma(c_V16d[i * 16 + k + 2], X[k + 2], oo);
    }
    const double oi = oe + oo, o7 = oe - oo;
    a = ei + oi;
    b = ei - oi;
    c = e7 + o7;
    d = e7 - o7;
}

// Plain FP64 leaf pass for n = 16 (NEUMANN, SOLVE): 16 threads per item, thread t owning row t;
// the same contractions as k_leaf_eigen, U = V [(V^T F V) ./ D] V^T, with two transposes through
// a 16 x 17 shared buffer under __syncwarp.
template <int MODE>
__global__ void __launch_bounds__(256) k_leaf16d(const LeafType* __restrict__ types,
                                                 const LeafItem* __restrict__ items, int nitems) {
    __shared__ double buf[16 * 272];
    __shared__ double Vs[16 * 17];
    const int tid = threadIdx.x, slot = tid >> 4, t = tid & 15;
    const int idx = blockIdx.x * 16 + slot;
    const bool act = idx < nitems;
    const LeafItem it = items[act ? idx : 0];
    const LeafType ty = types[it.type];
    double* bf = buf + slot * 272;
    if (MODE == LEAF_NEUMANN) {
        const int i = tid >> 4, k = tid & 15;
        const double v = c_V16d[(i < 8 ? i : 15 - i) * 16 + k];
        Vs[i * 17 + k] = (i >= 8 && (k & 1)) ? -v : v;
        __syncthreads();
    }
    double x[16], X[16];
    // (1) row t of f; the solve adds -2 (cx g_x + cy g_y) on the edge cells
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = (act && it.f != nullptr) ? it.f[t * 16 + j] : 0.0;
    if (MODE == LEAF_SOLVE && act && it.g != nullptr) {
        const double cx = 1.0 / (ty.dx * ty.dx), cy = 1.0 / (ty.dy * ty.dy);
        const double gs = it.g[2 * 16 + t], gn = it.g[3 * 16 + t];
        if (t == 0 || t == 15) {
            const int side = t == 0 ? 0 : 16;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                double acc = cx * it.g[side + j];
                if (j == 0) acc = acc + cy * gs;
                else if (j == 15) acc = acc + cy * gn;
                x[j] += -2.0 * acc;
            }
        } else {
            x[0] += -2.0 * (cy * gs);
            x[15] += -2.0 * (cy * gn);
        }
    }
    // (2) A = F V by rows; transpose
    dst16d_fwd(x, [&](int l, double v) { bf[t * 17 + l] = v; });
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = bf[i * 17 + t];
    // (3) G[k][t] = Dinv[k][t] (V^T A)[k][t]
    dst16d_fwd(x, [&](int k, double v) { X[k] = v * __ldg(ty.Dinv + k * 16 + t); });
    // (4) C = V G by columns; transpose back (buffer row t = column t of C)
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        double a, b, c, d;
        dst16d_quad(X, i, a, b, c, d);
        bf[t * 17 + i] = a;
        bf[t * 17 + 15 - i] = b;
        bf[t * 17 + 7 - i] = c;
        bf[t * 17 + 8 + i] = d;
    }
    __syncwarp();
    if (MODE == LEAF_SOLVE) {
        // (5) U[t][j] = sum_l C[t][l] V[j][l], staged, then written coalesced
#pragma unroll
        for (int l = 0; l < 16; ++l) X[l] = bf[l * 17 + t];
        __syncwarp();
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            double a, b, c, d;
            dst16d_quad(X, i, a, b, c, d);
            bf[t * 17 + i] = a;
            bf[t * 17 + 15 - i] = b;
            bf[t * 17 + 7 - i] = c;
            bf[t * 17 + 8 + i] = d;
        }
        __syncwarp();
        if (act)
#pragma unroll
            for (int m = 0; m < 16; ++m) {
                const int e = t + 16 * m;
                it.out[e] = bf[(e >> 4) * 17 + (e & 15)];
            }
    } else {
        // (5) edge values: S/N at i = t (row t of C), W/E at j = t (rows 0 and 15 of C)
        double e = 0.0, o = 0.0, uw = 0.0, ue = 0.0;
#pragma unroll
        for (int l = 0; l < 16; l += 2) {
            e = fma(c_V16d[l], bf[l * 17 + t], e);
            o = fma(c_V16d[l + 1], bf[(l + 1) * 17 + t], o);
        }
#pragma unroll
        for (int l = 0; l < 16; ++l) {
            const double v = Vs[t * 17 + l];
            uw = fma(bf[l * 17], v, uw);
            ue = fma(bf[l * 17 + 15], v, ue);
        }
        if (act) {
            const double dtn_x = 2.0 / ty.dx, dtn_y = 2.0 / ty.dy;
            it.out[0 * 16 + t] = dtn_x * uw;
            it.out[1 * 16 + t] = (-dtn_x) * ue;
            it.out[2 * 16 + t] = dtn_y * (e + o);
            it.out[3 * 16 + t] = (-dtn_y) * (e - o);
        }
    }
}

template <int MODE>
void launch_leaf(cudaStream_t st, const LeafType* types, const LeafItem* items, int nitems, int nmax) {
    const size_t smem = size_t(3) * nmax * nmax * sizeof(double);
    // set on every call (cheap, and the current device may change between calls); a once-only flag
    // would be shared unsynchronised by host threads
    cudaFuncSetAttribute(k_leaf_eigen<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    k_leaf_eigen<MODE><<<nitems, 256, smem, st>>>(types, items);
    ++g_kernel_launches;
}

}  // namespace

void leaf_set_basis16(cudaStream_t st) {
    // uploaded by every tree set-up and single-patch call (1 KB): the values never change, and a
    // context reset by the caller cannot leave the table empty
    double V[8 * 16];
    for (int i = 0; i < 8; ++i)
        for (int k = 0; k < 16; ++k) {
            const double c = (k == 15) ? std::sqrt(1.0 / 16) : std::sqrt(2.0 / 16);
            V[i * 16 + k] = c * std::sin(M_PI * (k + 1) * (i + 0.5) / 16);
        }
    if (cudaMemcpyToSymbolAsync(c_V16d, V, sizeof(V), 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        throw std::runtime_error("leaf basis upload failed");
}

void leaf_eigen(cudaStream_t st, int mode, const LeafType* types, const LeafItem* items, int nitems,
                int nmax) {
    if (nitems <= 0) return;
    if (nmax == 16 && (mode == LEAF_NEUMANN || mode == LEAF_SOLVE)) {
        const unsigned grid = unsigned((nitems + 15) / 16);
        if (mode == LEAF_NEUMANN) k_leaf16d<LEAF_NEUMANN><<<grid, 256, 0, st>>>(types, items, nitems);
        else k_leaf16d<LEAF_SOLVE><<<grid, 256, 0, st>>>(types, items, nitems);
        ++g_kernel_launches;
        return;
    }
    leaf_eigen_tables(st, mode, types, items, nitems, nmax);
}

void leaf_eigen_tables(cudaStream_t st, int mode, const LeafType* types, const LeafItem* items, int nitems,
                       int nmax) {
    if (nitems <= 0) return;
    if (mode == LEAF_DTN_COLUMN) launch_leaf<LEAF_DTN_COLUMN>(st, types, items, nitems, nmax);
    else if (mode == LEAF_NEUMANN) launch_leaf<LEAF_NEUMANN>(st, types, items, nitems, nmax);
    else if (mode == LEAF_SOLVE) launch_leaf<LEAF_SOLVE>(st, types, items, nitems, nmax);
    else launch_leaf<LEAF_MAPD2N>(st, types, items, nitems, nmax);
}

}  // namespace efgb
