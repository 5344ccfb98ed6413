// Leaf Dirichlet-to-Neumann maps of the constant-coefficient (FISHPACK90) leaf types by a pivoted
// dense LU of the 5-point operator (FiniteVolumeSolver::buildD2N, FiniteVolumeSolver.cpp:355-455).
//
// Column j of T is mapD2N(e_j, f = 0): the solve of A u = -2 c_side e_j at the edge cell of boundary
// point j, then h = +-(2/d)(u_edge - g) (cpp:296-353).  The sine eigenbasis solves the same system,
// but its rounding spreads over every mode, and the DtN applied to smooth data cancels to O(1) from
// entries of O(1/d): HPS trees built on eigenbasis DtN maps drifted from the LU-based solution by
// ~N^2 eps at the leaf solutions (1.2e-11 at 1024^2 cells, against 2.6e-13 with an LU).  A tree has
// one DtN per distinct leaf geometry (n, dx, dy), so the n^2 x n^2 LU costs little: the batched
// pivoted LU and triangular solves of the merges (ef_linalg.cu) factor every type at once.
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "ef_kernels.cuh"

namespace efgb {

namespace {

// A (nn x nn, row-major, cell index j + i n) of u_xx + u_yy + lambda u with the Dirichlet ghost
// 2g - u at the patch faces, as the oracle's five_point_matrix builds it (cpp:66-200 with
// alpha = beta = 1): cW = cE = 1/dx^2, cS = cN = 1/dy^2, cC = -(2/dx^2 + 2/dy^2) + lambda, and the
// ghost moves -c_side onto the diagonal at the faces.
__global__ void k_dtn_assemble(int n, const double* __restrict__ dxs, const double* __restrict__ dys,
                               double lambda, double* const* A) {
    const long long nn = (long long)n * n, tot = nn * nn;
    const int t = blockIdx.y;
    const double dx = dxs[t], dy = dys[t];
    const double cx = 1.0 * 1.0 / (dx * dx), cy = 1.0 * 1.0 / (dy * dy);
    const double cC = -1.0 * ((1.0 + 1.0) / (dx * dx) + (1.0 + 1.0) / (dy * dy)) + lambda;
    double* __restrict__ a = A[t];
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const int r = int(e / nn), c = int(e - (e / nn) * nn);
        const int i = r / n, j = r - (r / n) * n;
        double v = 0.0;
        if (c == r) {
            double d = cC;
            if (i == 0) d -= cx;
            if (i == n - 1) d -= cx;
            if (j == 0) d -= cy;
            if (j == n - 1) d -= cy;
            v = d;
        } else if (c == r - n && i > 0) {
            v = cx;
        } else if (c == r + n && i < n - 1) {
            v = cx;
        } else if (c == r - 1 && j > 0) {
            v = cy;
        } else if (c == r + 1 && j < n - 1) {
            v = cy;
        }
        a[e] = v;
    }
}

// edge cell (j + i n) next to boundary point p in WESN order
__device__ __forceinline__ int edge_cell(int p, int n) {
    const int side = p / n, k = p - (p / n) * n;
    if (side == 0) return k;                  // W: i = 0, j = k
    if (side == 1) return (n - 1) * n + k;    // E: i = n-1
    if (side == 2) return k * n;              // S: j = 0, i = k
    return k * n + n - 1;                     // N: j = n-1
}

// right-hand sides of the 4n unit Dirichlet data, rows already permuted by the LU's row order:
// B[r][p] = f_boundary(e_p)[perm[r]] = -2 c_side(p) at the edge cell of p (cpp:96-184)
__global__ void k_dtn_rhs(int n, const double* __restrict__ dxs, const double* __restrict__ dys,
                          const int* const* perm, double* const* B) {
    const int nn = n * n, m = 4 * n;
    const int t = blockIdx.y;
    const double cx = 1.0 * 1.0 / (dxs[t] * dxs[t]), cy = 1.0 * 1.0 / (dys[t] * dys[t]);
    const int* __restrict__ pm = perm[t];
    double* __restrict__ b = B[t];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nn * m; e += gridDim.x * blockDim.x) {
        const int r = e / m, p = e - (e / m) * m;
        const int src = pm[r];
        b[e] = (src == edge_cell(p, n)) ? -2.0 * (p < 2 * n ? cx : cy) : 0.0;
    }
}

// T[q][p] = s_q (2/d_q)(u_p[edge_cell(q)] - delta_qp): W +2/dx, E -2/dx, S +2/dy, N -2/dy
__global__ void k_dtn_extract(int n, const double* __restrict__ dxs, const double* __restrict__ dys,
                              const double* const* U, double* const* T) {
    const int m = 4 * n;
    const int t = blockIdx.y;
    const double dtn_x = 2.0 / dxs[t], dtn_y = 2.0 / dys[t];
    const double* __restrict__ u = U[t];
    double* __restrict__ out = T[t];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * m; e += gridDim.x * blockDim.x) {
        const int q = e / m, p = e - (e / m) * m;
        const int side = q / n;
        const double diff = u[(long long)edge_cell(q, n) * m + p] - (q == p ? 1.0 : 0.0);
        const double scale = side == 0 ? dtn_x : side == 1 ? -dtn_x : side == 2 ? dtn_y : -dtn_y;
        out[e] = scale * diff;
    }
}

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

}  // namespace

int leaf_dtn_lu(cudaStream_t st, int n, double lambda, const std::vector<double>& dx, const std::vector<double>& dy,
                const std::vector<double*>& T) {
    const int nt = int(dx.size());
    if (nt == 0) return 0;
    if (int(dy.size()) != nt || int(T.size()) != nt) throw std::invalid_argument("leaf_dtn_lu: table sizes differ");
    const size_t nn = size_t(n) * n, m = 4 * size_t(n);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t oA = 0, oB = oA + up(nt * nn * nn * 8), oP = oB + up(nt * nn * m * 8),
                 oQ = oP + up(nt * nn * 4), oI = oQ + up(nt * nn * 4), oDx = oI + up(nt * 4),
                 oDy = oDx + up(nt * 8), oArr = oDy + up(nt * 8), total = oArr + up(6 * nt * sizeof(void*));
    char* buf = nullptr;
    ck(cudaMalloc(&buf, total), "cudaMalloc(leaf DtN LU)");
    std::vector<void*> arr(6 * nt);
    for (int t = 0; t < nt; ++t) {
        arr[0 * nt + t] = buf + oA + t * nn * nn * 8;  // A (LU in place)
        arr[1 * nt + t] = buf + oB + t * nn * m * 8;   // B -> U
        arr[2 * nt + t] = buf + oP + t * nn * 4;       // piv
        arr[3 * nt + t] = buf + oQ + t * nn * 4;       // perm
        arr[4 * nt + t] = T[t];                        // T out
        arr[5 * nt + t] = nullptr;
    }
    int bad = 0;
    try {
        ck(cudaMemcpyAsync(buf + oDx, dx.data(), nt * 8, cudaMemcpyHostToDevice, st), "dx");
        ck(cudaMemcpyAsync(buf + oDy, dy.data(), nt * 8, cudaMemcpyHostToDevice, st), "dy");
        ck(cudaMemcpyAsync(buf + oArr, arr.data(), arr.size() * sizeof(void*), cudaMemcpyHostToDevice, st), "arrays");
        ck(cudaMemsetAsync(buf + oI, 0, nt * 4, st), "info");
        auto** dA = reinterpret_cast<double**>(buf + oArr);
        auto** dB = dA + nt;
        auto** dP = reinterpret_cast<int**>(dA + 2 * nt);
        auto** dQ = reinterpret_cast<int**>(dA + 3 * nt);
        auto** dT = dA + 4 * nt;
        const double* ddx = reinterpret_cast<const double*>(buf + oDx);
        const double* ddy = reinterpret_cast<const double*>(buf + oDy);
        int* dinfo = reinterpret_cast<int*>(buf + oI);
        const int ga = int(std::min<size_t>((nn * nn + 255) / 256, 4096));
        k_dtn_assemble<<<dim3(ga, nt), 256, 0, st>>>(n, ddx, ddy, lambda, dA);
        ++g_kernel_launches;
        dgetrf_batched(st, int(nn), dA, int(nn), dP, dinfo, nt);
        piv_to_perm(st, int(nn), dP, dQ, nt);
        const int gb = int(std::min<size_t>((nn * m + 255) / 256, 4096));
        k_dtn_rhs<<<dim3(gb, nt), 256, 0, st>>>(n, ddx, ddy, dQ, dB);
        ++g_kernel_launches;
        dlu_solve_permuted(st, int(nn), int(m), (const double* const*)dA, int(nn), dB, int(m), nt);
        const int gt = int(std::min<size_t>((m * m + 255) / 256, 4096));
        k_dtn_extract<<<dim3(gt, nt), 256, 0, st>>>(n, ddx, ddy, (const double* const*)dB, dT);
        ++g_kernel_launches;
        ck(cudaGetLastError(), "leaf DtN launch");
        std::vector<int> info(nt);
        ck(cudaMemcpyAsync(info.data(), dinfo, nt * 4, cudaMemcpyDeviceToHost, st), "info");
        ck(cudaStreamSynchronize(st), "leaf DtN sync");
        for (int v : info) bad += (v != 0);
    } catch (...) {
        cudaStreamSynchronize(st);
        cudaFree(buf);
        throw;
    }
    cudaFree(buf);
    return bad;
}

}  // namespace efgb
