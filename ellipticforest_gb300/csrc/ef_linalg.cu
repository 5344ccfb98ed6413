// Batched dense linear algebra for the HPS merges: FP64 (plain form) and FP32 (mixed build).
//
// Replaces the reference's per-node LAPACK/BLAS calls (Matrix.hpp:789-952: dgemv, dgemm and dgesv
// on transposed copies) with grouped launches over every merge of one tree level.  On GB300 the
// FP64 pipe, not HBM, bounds these kernels; they are tiled for register reuse.
#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>
#include <climits>

#include "ef_kernels.cuh"

namespace efgb {

std::atomic<long long> g_kernel_launches{0};
std::atomic<bool> g_cooperative_lu{true};

namespace {

constexpr int TM = 64, TN = 64, TK = 16;
constexpr int NB = 32;  // LU / triangular-solve block size

template <class Real>
__global__ void __launch_bounds__(256) k_dgemm(int M, int N, int K, Real alpha, GemmArgsT<Real> a,
                                               Real beta, int b0) {
    const int b = b0 + blockIdx.z;
    const Real* __restrict__ A = a.A[b] + a.offA;
    const Real* __restrict__ B = a.B[b] + a.offB;
    const Real* __restrict__ B2 = a.B2 ? a.B2[b] + a.offB2 : B;
    const int kb = a.B2 ? a.kb : (1 << 30);
    Real* C = a.C[b] + a.offC;
    const int m0 = blockIdx.y * TM, n0 = blockIdx.x * TN;
    __shared__ Real As[TK][TM + 1];
    __shared__ Real Bs[TK][TN];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    Real acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = Real(0);

    for (int k0 = 0; k0 < K; k0 += TK) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int e = tid + 256 * r;
            const int row = e >> 4, kk = e & 15;
            const int gm = m0 + row, gk = k0 + kk;
            As[kk][row] = (gm < M && gk < K) ? A[(long long)gm * a.lda + gk] : Real(0);
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int e = tid + 256 * r;
            const int kk = e >> 6, col = e & 63;
            const int gk = k0 + kk, gn = n0 + col;
            Bs[kk][col] = (gk < K && gn < N)
                              ? (gk < kb ? B[(long long)gk * a.ldb + gn] : B2[(long long)(gk - kb) * a.ldb + gn])
                              : Real(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            Real av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int row = m0 + ty + 16 * i;
        if (row >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int col = n0 + tx + 16 * j;
            if (col >= N) continue;
            Real* c = C + (long long)row * a.ldc + col;
            *c = (beta == Real(0)) ? alpha * acc[i][j] : fma(alpha, acc[i][j], beta * *c);
        }
    }
}

// Unblocked LU with partial pivoting of the panel A[k:n, k:k+jb] (LAPACK dgetf2 on a panel).
// One CTA per matrix.  Row swaps are applied inside the panel columns only.
template <class Real>
__global__ void __launch_bounds__(1024) k_getf2_panel(int n, int k, int jb, Real* const* Aarr,
                                                      int lda, int* const* pivarr, int* info) {
    Real* __restrict__ A = Aarr[blockIdx.x];
    int* __restrict__ piv = pivarr[blockIdx.x];
    __shared__ Real s_val[32];
    __shared__ int s_idx[32];
    __shared__ int s_p;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    for (int j = k; j < k + jb; ++j) {
        Real best = Real(-1);
        int bi = INT_MAX;
        for (int i = j + tid; i < n; i += blockDim.x) {
            const Real v = fabs(A[(long long)i * lda + j]);
            if (v > best) { best = v; bi = i; }
            else if (bi == INT_MAX) { bi = i; }
        }
        // (value, index) reduction: the larger value wins, ties go to the smaller index (idamax).
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const Real ov = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, bi, off);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { s_val[wid] = best; s_idx[wid] = bi; }
        __syncthreads();
        if (wid == 0) {
            best = (lane < nw) ? s_val[lane] : Real(-2);
            bi = (lane < nw) ? s_idx[lane] : INT_MAX;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const Real ov = __shfl_down_sync(0xffffffffu, best, off);
                const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (lane == 0) {
                const int p = (bi >= j && bi < n) ? bi : j;
                s_p = p;
                piv[j] = p;
                if (!(A[(long long)p * lda + j] != Real(0)) && info[blockIdx.x] == 0) info[blockIdx.x] = j + 1;
            }
        }
        __syncthreads();
        const int p = s_p;
        if (p != j) {
            for (int c = tid; c < jb; c += blockDim.x) {
                Real* a = A + (long long)j * lda + k + c;
                Real* b = A + (long long)p * lda + k + c;
                const Real t = *a; *a = *b; *b = t;
            }
        }
        __syncthreads();
        const Real pv = A[(long long)j * lda + j];
        if (pv != Real(0)) {
            if (fabs(pv) >= (sizeof(Real) == 8 ? Real(DBL_MIN) : Real(FLT_MIN))) {
                const Real r = Real(1) / pv;
                for (int i = j + 1 + tid; i < n; i += blockDim.x) A[(long long)i * lda + j] *= r;
            } else {
                for (int i = j + 1 + tid; i < n; i += blockDim.x) A[(long long)i * lda + j] /= pv;
            }
        }
        __syncthreads();
        const int nc = k + jb - j - 1;
        if (nc > 0) {
            const long long tot = (long long)(n - j - 1) * nc;
            for (long long e = tid; e < tot; e += blockDim.x) {
                const int i = j + 1 + int(e / nc);
                const int c = j + 1 + int(e % nc);
                A[(long long)i * lda + c] -= A[(long long)i * lda + j] * A[(long long)j * lda + c];
            }
        }
        __syncthreads();
    }
}

// Panel LU of large matrices spread over P CTAs per matrix (cooperative launch, one grid-wide barrier
// per column).  Rows are not moved during the panel: every CTA owns a slice of the physical rows and
// keeps their logical positions and "not yet a pivot" flags, so the pivot search, the scaling and the
// rank-1 updates are those of the single-CTA kernel (ties go to the smaller logical index, as in
// idamax); piv holds the LAPACK swap sequence, applied to the panel columns afterwards.
constexpr int kCoopRows = 1024;  // rows per CTA at most (shared memory for their bookkeeping)

template <class Real>
__global__ void __launch_bounds__(256) k_getf2_coop(int n, int k, int jb, Real* const* Aarr, int lda,
                                                    int* const* pivarr, int* info, int P, Real* pval, int* ppos) {
    namespace cg = cooperative_groups;
    cg::grid_group grid = cg::this_grid();
    const int mat = blockIdx.x / P, part = blockIdx.x - mat * P;
    Real* __restrict__ A = Aarr[mat];
    int* __restrict__ piv = pivarr[mat];
    const int rows = n - k, per = (rows + P - 1) / P;
    const int r0 = k + part * per, r1 = min(n, r0 + per);
    __shared__ int lpos[kCoopRows];
    __shared__ unsigned char act[kCoopRows];
    __shared__ Real s_val[32];
    __shared__ int s_idx[32];
    __shared__ int s_phys[32];
    __shared__ Real s_prow[32];
    __shared__ int s_pphys, s_plog;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    for (int r = r0 + tid; r < r1; r += blockDim.x) {
        lpos[r - r0] = r;
        act[r - r0] = 1;
    }
    __syncthreads();
    // (value, logical index) of the largest |A[r][j]| over this CTA's active rows
    // (value, logical index, physical row) of the largest |A[r][j]| over this CTA's active rows, to
    // the candidate tables (logical indices in ppos slots 0/1, physical rows in slots 2/3)
    auto local_max = [&](int j, int slot) {
        Real best = Real(-1);
        int bi = INT_MAX, bp = -1;
        for (int r = r0 + tid; r < r1; r += blockDim.x) {
            if (!act[r - r0]) continue;
            const Real v = fabs(A[(long long)r * lda + j]);
            const int li = lpos[r - r0];
            if (v > best || (v == best && li < bi)) { best = v; bi = li; bp = r; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const Real ov = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, bi, off);
            const int op = __shfl_down_sync(0xffffffffu, bp, off);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; bp = op; }
        }
        if (lane == 0) { s_val[wid] = best; s_idx[wid] = bi; s_phys[wid] = bp; }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < nw; ++w)
                if (s_val[w] > best || (s_val[w] == best && s_idx[w] < bi)) { best = s_val[w]; bi = s_idx[w]; bp = s_phys[w]; }
            pval[((long long)slot * gridDim.x) + blockIdx.x] = best;
            ppos[((long long)slot * gridDim.x) + blockIdx.x] = bi;
            ppos[((long long)(2 + slot) * gridDim.x) + blockIdx.x] = bp;
        }
        __syncthreads();
    };
    local_max(k, 0);
    for (int j = k; j < k + jb; ++j) {
        const int slot = (j - k) & 1;
        grid.sync();
        // every CTA of the matrix reduces the P candidates the same way; the owner of the pivot row
        // publishes its physical index through the candidate table
        if (tid == 0) {
            Real best = Real(-1);
            int bi = INT_MAX, bp = -1;
            for (int t = 0; t < P; ++t) {
                const Real v = pval[(long long)slot * gridDim.x + mat * P + t];
                const int li = ppos[(long long)slot * gridDim.x + mat * P + t];
                if (v > best || (v == best && li < bi)) {
                    best = v;
                    bi = li;
                    bp = ppos[(long long)(2 + slot) * gridDim.x + mat * P + t];
                }
            }
            s_plog = bi;
            s_pphys = bp;
        }
        __syncthreads();
        const int plog = s_plog, pphys = s_pphys;
        if (part == 0 && tid == 0) {
            piv[j] = plog;
            if (!(A[(long long)pphys * lda + j] != Real(0)) && info[mat] == 0) info[mat] = j + 1;
        }
        // the pivot row leaves the active set; the row at logical position j moves to plog
        for (int r = r0 + tid; r < r1; r += blockDim.x) {
            const int l = r - r0;
            if (r == pphys) { act[l] = 0; lpos[l] = j; }
            else if (act[l] && lpos[l] == j) lpos[l] = plog;
        }
        for (int c = tid; c < k + jb - j; c += blockDim.x) s_prow[c] = A[(long long)pphys * lda + j + c];
        __syncthreads();
        const Real pv = s_prow[0];
        const bool big = fabs(pv) >= (sizeof(Real) == 8 ? Real(DBL_MIN) : Real(FLT_MIN));
        const Real rinv = Real(1) / pv;
        const int nc = k + jb - j - 1;
        for (int r = r0 + tid; r < r1; r += blockDim.x) {
            if (!act[r - r0]) continue;
            Real* row = A + (long long)r * lda;
            Real l = row[j];
            if (pv != Real(0)) l = big ? l * rinv : l / pv;
            row[j] = l;
            for (int c = 1; c <= nc; ++c) row[j + c] -= l * s_prow[c];
        }
        __syncthreads();
        if (j + 1 < k + jb) local_max(j + 1, (j + 1 - k) & 1);
    }
}

// Apply the swaps piv[k..k+jb) to the columns [c0, c0 + ncols) (LAPACK dlaswp).
// Panel LU of a large matrix on a thread-block cluster of P CTAs (P <= 8) per matrix: CTA c holds the
// panel rows [c R, (c+1) R) of A[k:n, k:k+jb] in its shared memory, so a column costs two cluster
// barriers instead of grid-wide ones.  Per column: every CTA offers the largest |a| of its rows (ties
// to the smaller row) -> barrier -> every CTA combines the P candidates read through distributed
// shared memory (the same winner everywhere), copies the pivot row, and the owner of the pivot row
// keeps the old row j -> barrier -> the two owners write the exchanged rows, every CTA scales its
// rows below j and applies the rank-1 update with its copy of the pivot row.  The element operations
// and their order are those of k_getf2_panel (bit-identical factors and pivots); rows are exchanged
// in shared memory and written back at the end, so only the columns outside the panel still need
// the row swaps.
template <class Real>
__global__ void __launch_bounds__(256) k_getf2_cluster(int n, int k, int jb, Real* const* Aarr, int lda,
                                                       int* const* pivarr, int* info, int P, int R) {
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    extern __shared__ __align__(16) unsigned char cl_smem[];
    Real* rows = reinterpret_cast<Real*>(cl_smem);  // R x jb, row-major
    Real* prow = rows + (size_t)R * jb;            // copy of the pivot row
    Real* jrow = prow + jb;                        // old row j (owner of the pivot row)
    __shared__ Real s_val[32];
    __shared__ int s_idx[32];
    __shared__ Real c_val;
    __shared__ int c_idx;
    const int mat = blockIdx.x / P;
    const int c = int(cluster.block_rank());
    Real* __restrict__ A = Aarr[mat];
    int* __restrict__ piv = pivarr[mat];
    const int m = n - k;                  // panel height
    const int r0 = c * R, r1 = min(m, r0 + R);
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
    for (int e = tid; e < (r1 - r0) * jb; e += blockDim.x) {
        const int i = e / jb, cc = e - i * jb;
        rows[e] = A[(long long)(k + r0 + i) * lda + k + cc];
    }
    __syncthreads();
    for (int j = 0; j < jb; ++j) {
        // (1) this CTA's candidate among its rows i >= j
        Real best = Real(-1);
        int bi = INT_MAX;
        for (int i = max(j, r0) + tid; i < r1; i += blockDim.x) {
            const Real v = fabs(rows[(size_t)(i - r0) * jb + j]);
            if (v > best) { best = v; bi = i; }
            else if (bi == INT_MAX) { bi = i; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const Real ov = __shfl_down_sync(0xffffffffu, best, off);
            const int oi = __shfl_down_sync(0xffffffffu, bi, off);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if (lane == 0) { s_val[wid] = best; s_idx[wid] = bi; }
        __syncthreads();
        if (wid == 0) {
            best = (lane < nw) ? s_val[lane] : Real(-2);
            bi = (lane < nw) ? s_idx[lane] : INT_MAX;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const Real ov = __shfl_down_sync(0xffffffffu, best, off);
                const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (lane == 0) { c_val = best; c_idx = bi; }
        }
        cluster.sync();
        // (2) the winner, the pivot row and (its owner) the old row j
        if (wid == 0) {
            best = (lane < P) ? *cluster.map_shared_rank(&c_val, lane) : Real(-2);
            bi = (lane < P) ? *cluster.map_shared_rank(&c_idx, lane) : INT_MAX;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const Real ov = __shfl_down_sync(0xffffffffu, best, off);
                const int oi = __shfl_down_sync(0xffffffffu, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (lane == 0) s_idx[0] = (bi >= j && bi < m) ? bi : j;
        }
        __syncthreads();
        const int p = s_idx[0];
        const int cp = p / R, cj = j / R;
        const Real* prem = cluster.map_shared_rank(rows, cp) + (size_t)(p - cp * R) * jb;
        for (int cc = tid; cc < jb; cc += blockDim.x) prow[cc] = prem[cc];
        if (c == cp && p != j) {
            const Real* jrem = cluster.map_shared_rank(rows, cj) + (size_t)(j - cj * R) * jb;
            for (int cc = tid; cc < jb; cc += blockDim.x) jrow[cc] = jrem[cc];
        }
        if (c == 0 && tid == 0) {
            piv[k + j] = k + p;
            if (!(prem[j] != Real(0)) && info[mat] == 0) info[mat] = k + j + 1;
        }
        cluster.sync();
        if (p != j) {
            if (c == cj)
                for (int cc = tid; cc < jb; cc += blockDim.x) rows[(size_t)(j - r0) * jb + cc] = prow[cc];
            if (c == cp)
                for (int cc = tid; cc < jb; cc += blockDim.x) rows[(size_t)(p - r0) * jb + cc] = jrow[cc];
        }
        __syncthreads();
        // (3) scale the column below the pivot, (4) rank-1 update of the panel's later columns
        const Real pv = prow[j];
        const int lo = max(j + 1, r0);
        if (pv != Real(0)) {
            if (fabs(pv) >= (sizeof(Real) == 8 ? Real(DBL_MIN) : Real(FLT_MIN))) {
                const Real rcp = Real(1) / pv;
                for (int i = lo + tid; i < r1; i += blockDim.x) rows[(size_t)(i - r0) * jb + j] *= rcp;
            } else {
                for (int i = lo + tid; i < r1; i += blockDim.x) rows[(size_t)(i - r0) * jb + j] /= pv;
            }
        }
        __syncthreads();
        const int nc = jb - j - 1;
        if (nc > 0 && lo < r1) {
            const int tot = (r1 - lo) * nc;
            for (int e = tid; e < tot; e += blockDim.x) {
                const int i = lo + e / nc, cc = j + 1 + e % nc;
                Real* a = rows + (size_t)(i - r0) * jb;
                a[cc] -= a[j] * prow[cc];
            }
        }
        __syncthreads();
    }
    for (int e = tid; e < (r1 - r0) * jb; e += blockDim.x) {
        const int i = e / jb, cc = e - i * jb;
        A[(long long)(k + r0 + i) * lda + k + cc] = rows[e];
    }
    cluster.sync();  // no CTA leaves while another may still read its shared memory
}

template <class Real>
__global__ void k_laswp_cols(int k, int jb, Real* const* Aarr, int lda, int* const* pivarr, int c0, int ncols) {
    Real* __restrict__ A = Aarr[blockIdx.y];
    const int* __restrict__ piv = pivarr[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncols) return;
    const int c = c0 + t;
    for (int j = k; j < k + jb; ++j) {
        const int p = piv[j];
        if (p != j) {
            Real* a = A + (long long)j * lda + c;
            Real* b = A + (long long)p * lda + c;
            const Real tmp = *a; *a = *b; *b = tmp;
        }
    }
}

// Apply the swaps piv[k..k+jb) to the columns outside the panel (LAPACK dlaswp).
template <class Real>
__global__ void k_laswp_outside(int n, int k, int jb, Real* const* Aarr, int lda,
                                int* const* pivarr) {
    Real* __restrict__ A = Aarr[blockIdx.y];
    const int* __restrict__ piv = pivarr[blockIdx.y];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n - jb) return;
    const int c = (t < k) ? t : t + jb;
    for (int j = k; j < k + jb; ++j) {
        const int p = piv[j];
        if (p != j) {
            Real* a = A + (long long)j * lda + c;
            Real* b = A + (long long)p * lda + c;
            const Real tmp = *a; *a = *b; *b = tmp;
        }
    }
}

// Triangular solve of the jb rows [brow0, brow0+jb) x columns [bcol0, bcol0+ncols) of B with the
// jb x jb diagonal block of LU at (k, k).  LOWER: unit lower, forward substitution;
// !LOWER: upper non-unit, backward substitution.  One thread per column.
template <class Real, bool LOWER>
__global__ void __launch_bounds__(256) k_trsm_block(int k, int jb, const Real* const* LUarr,
                                                    int lda, Real* const* Barr, int ldb,
                                                    int brow0, int bcol0, int ncols) {
    const Real* __restrict__ LU = LUarr[blockIdx.y];
    Real* __restrict__ B = Barr[blockIdx.y];
    __shared__ Real L[NB][NB + 1];
    for (int e = threadIdx.x; e < jb * jb; e += blockDim.x) {
        const int r = e / jb, c = e % jb;
        L[r][c] = LU[(long long)(k + r) * lda + k + c];
    }
    __syncthreads();
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= ncols) return;
    Real* Bc = B + (long long)brow0 * ldb + bcol0 + col;
    Real x[NB];
#pragma unroll
    for (int i = 0; i < NB; ++i) x[i] = (i < jb) ? Bc[(long long)i * ldb] : Real(0);
    if (LOWER) {
#pragma unroll
        for (int i = 1; i < NB; ++i) {
            Real acc = x[i];
#pragma unroll
            for (int t = 0; t < i; ++t) acc -= L[i][t] * x[t];
            x[i] = (i < jb) ? acc : Real(0);
        }
    } else {
#pragma unroll
        for (int i = NB - 1; i >= 0; --i) {
            if (i < jb) {
                Real acc = x[i];
#pragma unroll
                for (int t = i + 1; t < NB; ++t) acc -= (t < jb ? L[i][t] : Real(0)) * x[t];
                x[i] = acc / L[i][i];
            }
        }
    }
#pragma unroll
    for (int i = 0; i < NB; ++i)
        if (i < jb) Bc[(long long)i * ldb] = x[i];
}

__global__ void k_piv_to_perm(int n, int* const* pivarr, int* const* permarr) {
    extern __shared__ int sp[];
    const int* piv = pivarr[blockIdx.x];
    int* perm = permarr[blockIdx.x];
    for (int i = threadIdx.x; i < n; i += blockDim.x) sp[i] = i;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < n; ++j) {
            const int p = piv[j];
            if (p != j && p >= 0 && p < n) { const int t = sp[j]; sp[j] = sp[p]; sp[p] = t; }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}


template <class Real>
void gemm_batched_t(cudaStream_t st, int M, int N, int K, Real alpha, const GemmArgsT<Real>& a, Real beta,
                    int batch) {
    if (M <= 0 || N <= 0 || batch <= 0) return;
    if (K <= 0 && beta == Real(1)) return;
    for (int b0 = 0; b0 < batch; b0 += 65535) {
        const int nb = batch - b0 < 65535 ? batch - b0 : 65535;
        dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM, nb);
        k_dgemm<Real><<<grid, 256, 0, st>>>(M, N, K, alpha, a, beta, b0);
        ++g_kernel_launches;
    }
}

// CTAs per matrix for the cooperative panel of a matrix with `rows` rows left (0: single-CTA panel)
template <class Real>
int coop_parts(int rows, int batch) {
    static int capacity = -1;
    if (capacity < 0) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_getf2_coop<Real>, 256, 0);
        capacity = coop ? sms * per : 0;
    }
    if (rows < 512 || capacity <= 0 || !g_cooperative_lu.load()) return 0;
    int P = std::min(capacity / batch, (rows + 31) / 32);
    while ((rows + P - 1) / P > kCoopRows) ++P;
    if (P < 2 || P * batch > capacity) return 0;
    return P;
}

// CTAs per matrix for the cluster panel of a matrix with `rows` rows left: the smallest power of two
// (2..8) that keeps a CTA's slice at <= 512 rows (FP64) / 1024 rows (FP32) -- 128 KB of shared
// memory with a 32-column panel; 0 when the cluster panel does not apply
template <class Real>
int cluster_parts(int rows) {
    if (rows < 512 || !g_cooperative_lu.load()) return 0;
    const int rmax = sizeof(Real) == 8 ? 512 : 1024;
    for (int P = 2; P <= 8; P *= 2)
        if ((rows + P - 1) / P <= rmax) return P;
    return 0;
}

template <class Real>
bool launch_cluster_panel(cudaStream_t st, int n, int k, int jb, Real* const* A, int lda, int* const* piv,
                          int* info, int batch, int P) {
    const int R = (n - k + P - 1) / P;
    const size_t smem = (size_t(R) * jb + 2 * size_t(jb)) * sizeof(Real);
    static size_t configured = 0;
    if (smem > configured) {
        if (cudaFuncSetAttribute(k_getf2_cluster<Real>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) !=
            cudaSuccess) {
            (void)cudaGetLastError();
            return false;
        }
        configured = smem;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(P * batch));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(P);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (cudaLaunchKernelEx(&cfg, k_getf2_cluster<Real>, n, k, jb, A, lda, piv, info, P, R) != cudaSuccess) {
        (void)cudaGetLastError();  // refused (cluster shape): the other panels
        return false;
    }
    return true;
}

template <class Real>
struct CoopScratch {  // candidate tables of the cooperative panel: 4 slots x grid
    Real* val = nullptr;
    int* pos = nullptr;
    int size = 0;
};

template <class Real>
void getrf_batched_t(cudaStream_t st, int n, Real* const* A, int lda, int* const* piv, int* info, int batch) {
    static CoopScratch<Real> scratch;
    for (int k = 0; k < n; k += NB) {
        const int jb = (n - k < NB) ? n - k : NB;
        const int Pc = cluster_parts<Real>(n - k);
        if (Pc > 0 && launch_cluster_panel<Real>(st, n, k, jb, A, lda, piv, info, batch, Pc)) {
            ++g_kernel_launches;  // rows exchanged in shared memory: no k_laswp_cols
        } else if (const int P = coop_parts<Real>(n - k, batch); P > 0) {
            const int grid = P * batch;
            if (scratch.size < grid) {
                cudaStreamSynchronize(st);
                if (scratch.val) cudaFree(scratch.val);
                if (scratch.pos) cudaFree(scratch.pos);
                cudaMalloc(&scratch.val, 4 * size_t(grid) * sizeof(Real));
                cudaMalloc(&scratch.pos, 4 * size_t(grid) * sizeof(int));
                scratch.size = grid;
            }
            int nn = n, kk = k, jj = jb, ld = lda, PP = P;
            Real* const* AA = A;
            int* const* pp = piv;
            int* inf = info;
            Real* pv = scratch.val;
            int* ps = scratch.pos;
            void* args[] = {&nn, &kk, &jj, (void*)&AA, &ld, (void*)&pp, &inf, &PP, &pv, &ps};
            if (cudaLaunchCooperativeKernel((const void*)k_getf2_coop<Real>, dim3(grid), dim3(256), args, 0, st) ==
                cudaSuccess) {
                ++g_kernel_launches;
                dim3 gp((jb + 31) / 32, batch);
                k_laswp_cols<Real><<<gp, 32, 0, st>>>(k, jb, A, lda, piv, k, jb);
                ++g_kernel_launches;
            } else {
                (void)cudaGetLastError();  // refused (co-residency): the single-CTA panel
                k_getf2_panel<Real><<<batch, 1024, 0, st>>>(n, k, jb, A, lda, piv, info);
                ++g_kernel_launches;
            }
        } else {
            const int threads = (n - k >= 512) ? 1024 : 256;
            k_getf2_panel<Real><<<batch, threads, 0, st>>>(n, k, jb, A, lda, piv, info);
            ++g_kernel_launches;
        }
        if (n - jb > 0) {
            dim3 g((n - jb + 255) / 256, batch);
            k_laswp_outside<Real><<<g, 256, 0, st>>>(n, k, jb, A, lda, piv);
            ++g_kernel_launches;
        }
        const int rest = n - k - jb;
        if (rest > 0) {
            // U12 = L11^{-1} A12
            dim3 g((rest + 255) / 256, batch);
            k_trsm_block<Real, true><<<g, 256, 0, st>>>(k, jb, (const Real* const*)A, lda, A, lda, k, k + jb, rest);
            ++g_kernel_launches;
            // A22 -= L21 U12
            GemmArgsT<Real> ga{(const Real* const*)A, (long long)(k + jb) * lda + k, lda,
                               (const Real* const*)A, (long long)k * lda + k + jb, lda,
                               A, (long long)(k + jb) * lda + k + jb, lda};
            gemm_batched_t<Real>(st, rest, rest, jb, Real(-1), ga, Real(1), batch);
        }
    }
}

template <class Real>
void lu_solve_permuted_t(cudaStream_t st, int n, int nrhs, const Real* const* LU, int lda, Real* const* B, int ldb,
                         int batch) {
    // forward: L y = P b
    for (int k = 0; k < n; k += NB) {
        const int jb = (n - k < NB) ? n - k : NB;
        dim3 g((nrhs + 255) / 256, batch);
        k_trsm_block<Real, true><<<g, 256, 0, st>>>(k, jb, LU, lda, B, ldb, k, 0, nrhs);
        ++g_kernel_launches;
        const int rest = n - k - jb;
        if (rest > 0) {
            GemmArgsT<Real> ga{LU, (long long)(k + jb) * lda + k, lda,
                               (const Real* const*)B, (long long)k * ldb, ldb,
                               B, (long long)(k + jb) * ldb, ldb};
            gemm_batched_t<Real>(st, rest, nrhs, jb, Real(-1), ga, Real(1), batch);
        }
    }
    // backward: U x = y
    const int last = ((n - 1) / NB) * NB;
    for (int k = last; k >= 0; k -= NB) {
        const int jb = (n - k < NB) ? n - k : NB;
        dim3 g((nrhs + 255) / 256, batch);
        k_trsm_block<Real, false><<<g, 256, 0, st>>>(k, jb, LU, lda, B, ldb, k, 0, nrhs);
        ++g_kernel_launches;
        if (k > 0) {
            GemmArgsT<Real> ga{LU, (long long)k, lda,
                               (const Real* const*)B, (long long)k * ldb, ldb,
                               B, 0, ldb};
            gemm_batched_t<Real>(st, k, nrhs, jb, Real(-1), ga, Real(1), batch);
        }
    }
}

}  // namespace

void dgemm_batched(cudaStream_t st, int M, int N, int K, double alpha, const GemmArgs& a, double beta, int batch) {
    gemm_batched_t<double>(st, M, N, K, alpha, a, beta, batch);
}
void sgemm_batched(cudaStream_t st, int M, int N, int K, float alpha, const GemmArgs32& a, float beta, int batch) {
    gemm_batched_t<float>(st, M, N, K, alpha, a, beta, batch);
}
void dgetrf_batched(cudaStream_t st, int n, double* const* A, int lda, int* const* piv, int* info, int batch) {
    getrf_batched_t<double>(st, n, A, lda, piv, info, batch);
}
void sgetrf_batched(cudaStream_t st, int n, float* const* A, int lda, int* const* piv, int* info, int batch) {
    getrf_batched_t<float>(st, n, A, lda, piv, info, batch);
}
void dlu_solve_permuted(cudaStream_t st, int n, int nrhs, const double* const* LU, int lda, double* const* B,
                        int ldb, int batch) {
    lu_solve_permuted_t<double>(st, n, nrhs, LU, lda, B, ldb, batch);
}
void slu_solve_permuted(cudaStream_t st, int n, int nrhs, const float* const* LU, int lda, float* const* B,
                        int ldb, int batch) {
    lu_solve_permuted_t<float>(st, n, nrhs, LU, lda, B, ldb, batch);
}

void piv_to_perm(cudaStream_t st, int n, int* const* piv, int* const* perm, int batch) {
    k_piv_to_perm<<<batch, 256, n * sizeof(int), st>>>(n, piv, perm);
    ++g_kernel_launches;
}

}  // namespace efgb
