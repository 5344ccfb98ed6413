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

template <int MODE>
void launch_leaf(cudaStream_t st, const LeafType* types, const LeafItem* items, int nitems, int nmax) {
    const size_t smem = size_t(3) * nmax * nmax * sizeof(double);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_leaf_eigen<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        configured = true;
    }
    k_leaf_eigen<MODE><<<nitems, 256, smem, st>>>(types, items);
    ++g_kernel_launches;
}

}  // namespace

void leaf_eigen(cudaStream_t st, int mode, const LeafType* types, const LeafItem* items, int nitems,
                int nmax) {
    if (nitems <= 0) return;
    if (mode == LEAF_DTN_COLUMN) launch_leaf<LEAF_DTN_COLUMN>(st, types, items, nitems, nmax);
    else if (mode == LEAF_NEUMANN) launch_leaf<LEAF_NEUMANN>(st, types, items, nitems, nmax);
    else if (mode == LEAF_SOLVE) launch_leaf<LEAF_SOLVE>(st, types, items, nitems, nmax);
    else launch_leaf<LEAF_MAPD2N>(st, types, items, nitems, nmax);
}

}  // namespace efgb
