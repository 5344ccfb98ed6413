// Device kernels of the GB300 HPS solver (FP64 plain form) and their host launch wrappers.
//
// Conventions (shared with the reference, src/HPSAlgorithm.hpp and FiniteVolumeSolver.cpp):
//   * every matrix is row-major with an explicit leading dimension;
//   * boundary vectors are WESN-stacked, each side `n` long (W,E run along y; S,N along x);
//   * a patch's cell (i, j) (x-index i, y-index j) is stored at j + i*n;
//   * children of a node are 0=alpha (SW), 1=beta (SE), 2=gamma (NW), 3=omega (NE).
//
// The merge of four children with (coarsened) side s uses the interface order of
// HPSAlgorithm.hpp:870-895: I0 = alpha|gamma, I1 = beta|omega, I2 = alpha|beta, I3 = gamma|omega.
// Each interface has a "lower" child (alpha, beta, alpha, gamma) and an "upper" child (gamma,
// omega, beta, omega); with sigma(lower) = -1, sigma(upper) = +1 the reference's blocks are
//   X(I,I')  = -sum_c sigma(I,c) Tc[q(c,I)][q(c,I')]
//   S_RHS(I,p) = sigma(I,c(p)) Tc(p)[q(c,I)][q(p)]          (c(p) adjacent to I)
//   H(p,I)   = Tc(p)[q(p)][q(c(p),I)]                        (c(p) adjacent to I)
//   T_LHS(p,p') = Tc[q(p)][q(p')]                             (c(p) == c(p'))
// where p runs over the parent's exterior points already in WESN order, i.e. the permutation
// pi_WESN = {0,4,2,6,1,3,5,7} of HPSAlgorithm.hpp:979-993 is applied while gathering.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <atomic>
#include <vector>
#include <cstdint>

namespace efgb {

// Number of kernels this library has launched (all handles, all streams).
extern std::atomic<long long> g_kernel_launches;
// LU panels of matrices with >= 512 rows left use the cooperative multi-CTA panel (default on)
extern std::atomic<bool> g_cooperative_lu;
// 16 x 16 leaves take the exact residual through the general leaf-size kernel (default off; the
// kernel for 16 x 16 leaves gives bit-identical results)
extern std::atomic<bool> g_general_residual;
// mixed block solvers created while set run the residual's interface rows level by level on every
// tree (default off: trees without coarsening steps read and difference the rows in place)
extern std::atomic<bool> g_level_interface;

// ------------------------------------------------------------------------------------------------
// Batched FP64 dense linear algebra (pointer arrays, uniform shapes and offsets per launch)
// ------------------------------------------------------------------------------------------------
template <class Real>
struct GemmArgsT {
    const Real* const* A; long long offA; int lda;
    const Real* const* B; long long offB; int ldb;
    Real* const* C; long long offC; int ldc;
    // optional: rows k >= kb of B come from B2 (row k - kb, same ldb)
    const Real* const* B2 = nullptr;
    long long offB2 = 0;
    int kb = 1 << 30;
};
using GemmArgs = GemmArgsT<double>;
using GemmArgs32 = GemmArgsT<float>;

// C = alpha*A*B + beta*C for each batch item (row-major); FP64 (plain form) and FP32 (mixed build).
void dgemm_batched(cudaStream_t st, int M, int N, int K, double alpha, const GemmArgs& a,
                   double beta, int batch);
void sgemm_batched(cudaStream_t st, int M, int N, int K, float alpha, const GemmArgs32& a, float beta,
                   int batch);

// In-place LU with partial pivoting of the square n x n matrices A[b] (row-major, lda).
// piv[b][j] is the 0-based row swapped with row j (LAPACK dgetrf semantics, 0-based);
// info[b] = first zero pivot (1-based) or 0.  A, piv: device arrays of device pointers.
void dgetrf_batched(cudaStream_t st, int n, double* const* A, int lda, int* const* piv, int* info,
                    int batch);
void sgetrf_batched(cudaStream_t st, int n, float* const* A, int lda, int* const* piv, int* info, int batch);

// perm[b][i] = original row that ends at position i after applying piv[b][0..n).
void piv_to_perm(cudaStream_t st, int n, int* const* piv, int* const* perm, int batch);

// B[b] <- U^{-1} L^{-1} B[b]  (B already row-permuted), n x nrhs, ldb.
void dlu_solve_permuted(cudaStream_t st, int n, int nrhs, const double* const* LU, int lda,
                        double* const* B, int ldb, int batch);
void slu_solve_permuted(cudaStream_t st, int n, int nrhs, const float* const* LU, int lda, float* const* B,
                        int ldb, int batch);

// ------------------------------------------------------------------------------------------------
// Leaf patch kernels (constant-coefficient Helmholtz u_xx + u_yy + lambda u = f, Dirichlet data on
// cell faces with ghost u = 2g - u; the discrete system of FiniteVolumeSolver.cpp:27-290)
// ------------------------------------------------------------------------------------------------
struct LeafType {
    int n;
    double dx, dy;
    const double* V;     // n x n orthonormal sine basis, V[i][k]
    const double* Dinv;  // n x n, 1 / (mu_x[k] + mu_y[l] + lambda)
};

enum LeafMode : int {
    LEAF_DTN_COLUMN = 0,  // g = e_unit, f = 0, write column `unit` of T (4n x 4n, row-major)
    LEAF_NEUMANN = 1,     // g = 0, f given, write h (4n)
    LEAF_SOLVE = 2,       // f (nullable = 0) and g given, write u (n*n)
    LEAF_MAPD2N = 3,      // f (nullable = 0) and g given, write h (4n)
};

struct LeafItem {
    int type;
    int unit;
    const double* f;
    const double* g;
    double* out;
};

void leaf_eigen(cudaStream_t st, int mode, const LeafType* types_dev, const LeafItem* items_dev,
                int nitems, int nmax);
// same as leaf_eigen, but every size runs the contraction kernel that reads the basis V from the
// LeafType table (never the constant-memory 16 x 16 basis): for callers that cannot upload it
void leaf_eigen_tables(cudaStream_t st, int mode, const LeafType* types_dev, const LeafItem* items_dev,
                       int nitems, int nmax);
// Leaf DtN maps T[t] (4n x 4n, row-major, WESN) of the constant-coefficient leaf geometries
// (dx[t], dy[t]) by a pivoted dense LU of their 5-point operators (ef_leaf_dtn.cu); synchronous,
// returns the number of singular operators (zero pivot)
int leaf_dtn_lu(cudaStream_t st, int n, double lambda, const std::vector<double>& dx, const std::vector<double>& dy,
                const std::vector<double*>& T);
// rows 0..7 of the 16 x 16 sine basis into constant memory (ordered on st, synchronous); required
// before leaf_eigen runs NEUMANN or SOLVE on 16 x 16 leaves
void leaf_set_basis16(cudaStream_t st);

// Variable-coefficient leaf (FivePointStencil): coefficients sampled per cell, banded LU of the
// 5-point operator (bandwidth n, no pivoting), triangular solves one warp per (leaf, RHS).
struct FpLeaf {
    int n;
    double dx, dy;
    const double* alpha;   // n*n, alpha(x_i, y_j)
    const double* beta;    // 4*n*n: beta at the W, E, S, N face of every cell
    const double* lambda;  // n*n
    double* band;          // n*n rows x (2n+1): row r holds columns r-n .. r+n (L multipliers | U)
    double* bcoef;         // 4n boundary coupling coefficients c_side (WESN)
    int* info;             // first zero pivot (1-based) or 0
};
void fp_factor(cudaStream_t st, const FpLeaf* leaves, int nleaves, int nmax);
// items[k].type indexes `leaves`; modes as for leaf_eigen
void fp_solve(cudaStream_t st, int mode, const FpLeaf* leaves, const LeafItem* items, int nitems,
              int nmax);

// ------------------------------------------------------------------------------------------------
// Mixed-precision many-RHS passes (ef_mixed.cu).  Node vectors are [len][B], leaf cells [B][L][n*n].
// ------------------------------------------------------------------------------------------------
struct LeafType32 {
    int n;
    float dx, dy;
    const float* V;
    const float* Dinv;
};

// A [B]-row of a mixed solver's arena: its buffer (byte offset / 256 from the arena's base) and row;
// the address depends on the block's request count B, the row stride of every buffer
struct MxRow {
    unsigned buf, row;
};
template <class T>
__host__ __device__ inline T* mx_row(const char* arena, MxRow r, int B) {
    return reinterpret_cast<T*>(const_cast<char*>(arena) + size_t(r.buf) * 256) + size_t(r.row) * size_t(B);
}

struct MixLeaf {
    int type;
    float* g32;   // [4n][B] Dirichlet data of the FP32 pass
    float* h32;   // [4n][B] particular flux of the FP32 pass
    double* g64;  // [4n][B] exact Dirichlet data of the state
    double* h64;  // [4n][B] edge flux of the state
    // the 4n rows of the exact Dirichlet data where they live: rows of g64, or, on a tree without
    // coarsening steps, rows of the root data and of the ancestors' interface states
    const MxRow* gsrc;
    const char* arena;  // base of the rows
};

// Merge index maps of a 4-to-1 node (the mixed kernels and the host tables that trace them).
// Interface I (0..3) of a node with child interfaces of s points: its lower and upper children and
// their rows; exterior row p of the node (8s rows, 2s per side): child c and its row q.
__host__ __device__ inline int mx_lower_child(int I) { return (I == 1) ? 1 : (I == 3 ? 2 : 0); }
__host__ __device__ inline int mx_upper_child(int I) { return (I == 0) ? 2 : (I == 2 ? 1 : 3); }
__host__ __device__ inline int mx_q_lower(int I, int o, int s) { return (I < 2 ? 3 * s : s) + o; }
__host__ __device__ inline int mx_q_upper(int I, int o, int s) { return (I < 2 ? 2 * s : 0) + o; }
__host__ __device__ inline void mx_ext_map(int p, int s, int& c, int& q) {
    const int side = p / (2 * s);
    const int r = p - side * 2 * s;
    const int hlf = r >= s ? 1 : 0;
    c = side < 2 ? side + 2 * hlf : (side == 2 ? 0 : 2) + hlf;
    q = side * s + (r - hlf * s);
}

// one interface row of the residual's flux mismatch: out[b] = FP32(lo[b] - up[b]), lo and up the
// edge-flux rows of the leaves on the interface's two sides
struct MxMis {
    MxRow out, lo, up;
};
void mx_mismatch(cudaStream_t st, const char* arena, const MxMis* rows, long long nrows, int B);
// one interface row of the FP64 state update of a pass: ug[b] += FP64(u[b]), u the pass's FP32
// interface values as the DOWN GEMM wrote them into the lower child's Dirichlet rows
struct MxAdd {
    MxRow ug, u;
};
void mx_state_add(cudaStream_t st, const char* arena, const MxAdd* rows, long long nrows, int B);
// dst row e ([B], rows contiguous) = row src[e]
void mx_gather_rows64(cudaStream_t st, const char* arena, const MxRow* src, double* dst, int nrows, int B);

struct MixItem {
    const float* S;       // 4s x 8s
    const float* Xi;      // 4s x 4s
    const float* H;       // 8s x 2s (compact)
    const float* hc[4];   // children's coarsened particular flux [4s][B]
    float* h;             // [8s][B]
    float* hd;            // [4s][B]
    float* w;             // [4s][B]
    const float* m;       // [4s][B] interface flux mismatch of the state
    const float* gf;      // [8s][B] own full-size Dirichlet data of the pass
    float* gc[4];         // children's Dirichlet data of the pass [4s][B]
    double* uG;           // [4s][B] interface values of the state
    const double* gf64;   // [8s][B] own full-size exact Dirichlet data
    double* gc64[4];      // children's exact Dirichlet data [4s][B]
    const double* hc64[4];// children's coarsened edge flux [4s][B]
    double* h64;          // [8s][B] own edge flux
    float* mout;          // = m, written by the residual
};

struct MixConv {  // operators -> FP32 copies in the group layout
    const double* RHS;    // FP64-built [S | X^-1] (or null)
    const double* H;      // FP64-built compact H (or null)
    float* S;
    float* Xi;
    float* H32;
    const float* RHS32;   // FP32-built [S | X^-1] (used when non-null)
    const float* Hsrc32;  // FP32-built compact H
};

// Rows per tile of the FP32 node GEMMs (kind 0: X^{-1} and S, 4s rows per node; kind 1: compact H,
// whose tiles stay inside one run of s rows): the largest of 64, 32, 16, 8, 4 dividing the run.
inline int mx_tile_rows(int kind, int s) {
    const int run = kind == 1 ? s : 4 * s;
    for (int rt = 64; rt >= 4; rt /= 2)
        if (run % rt == 0) return rt;
    return 0;
}

void mx_convert(cudaStream_t st, const MixConv* items, int nitems, int s);
// hd = hc_upper - hc_lower - m (the correction's interface jump)
void mx_hdiff(cudaStream_t st, const MixItem* items, int nitems, int s, int B);
// FP32 node GEMM of one group: kind 0  w = X^{-1} hd;  kind 1  h = H w + hc;  kind 2  u = S gf + w
// (scattered to the children and added to u_Gamma).  The group's operators are contiguous row-major
// matrices read through the TMA tensor map tm (32 columns x mx_tile_rows rows per box, 128-byte
// swizzle); err is set when a TMA wait times out.
// ksplit: CTAs of the thread-block cluster that split K for one tile (0: a heuristic from the tile
// count; the choice never depends on B, so a request's sums are grouped the same way in any block)
void mx_gemm(cudaStream_t st, int kind, const CUtensorMap& tm, const MixItem* items, int nitems, int s, int B,
             int* err, int ksplit);
// largest K split worth trying for a GEMM kind at interface size s (every CTA keeps >= 2 chunks)
int mx_gemm_max_split(int kind, int s);
// Tensor-core (tcgen05) form of the same node GEMMs (ef_mixed_tc.cu).  The group's operators are
// three bf16 planes whose sum is the FP32 operator (mx_tc_split, compact H rows in the child-major
// order of the kernel), stored as 16 KB blocks of 128 rows x 64 columns in the order of their
// shared-memory image with the 128-byte swizzle (mx_tc_plane_elems elements for the three planes,
// zeroed before the split).  Supported for interface sizes s that are powers of two >= 16.
bool mx_tc_supported(int kind, int s);
int mx_tc_max_split(int kind, int s);
long long mx_tc_plane_elems(long long rows, int K);
void mx_tc_split(cudaStream_t st, int kind, const float* src, void* dst, long long rows, int K, int s);
// failure-path test switch of both GEMM forms (process-wide): every CTA's first wait runs out
void mx_set_inject_timeout(int on);
void mx_tc_set_inject_timeout(int on);
void mx_gemm_tc(cudaStream_t st, int kind, const void* planes, const MixItem* items, int nitems, int s, int B,
                int* err, int ksplit);
void mx_scatter64(cudaStream_t st, const MixItem* items, int nitems, int s, int B);
// the pass's exterior rows of every node of a group to its children (gf -> gc)
void mx_ext32(cudaStream_t st, const MixItem* items, int nitems, int s, int B);
void mx_flux_up(cudaStream_t st, const MixItem* items, int nitems, int s, int B);
void mx_coarsen(cudaStream_t st, bool fp64, const void* const* in, void* const* out, int count, int nf, int B);
void mx_uncoarsen(cudaStream_t st, bool fp64, const void* const* in, void* const* out, int count, int nf, int B);
// rows 0..7 of the 16 x 16 leaf eigenbasis (row-major, FP32) for the n = 16 leaf passes
void mx_set_basis16(cudaStream_t st, const float* V);
void mx_leaf32(cudaStream_t st, int mode, const LeafType32* types, const MixLeaf* leaves, int L, int B, int n,
               const float* q, double* u64, int accumulate);
// Stencil constants of a leaf type for the residual: cx = 1/dx^2, cy = 1/dy^2 and lambda as signed
// 63-bit significands m (|m| in [2^62, 2^63)) with c = m 2^(e - 63) (lmm = 0 when lambda = 0), iso
// when cx == cy; FP32 copies of cx, cy for the first residual; the FP64 edge-flux factors 2/dx, 2/dy
struct MixCoef {
    double dtn_x, dtn_y;
    long long cxm, cym, lmm;
    int ecx, ecy, elm, iso;
    float cx32, cy32;
};
// Residual of every leaf (n % 4 == 0, n <= 64): exact fixed-point second differences and 128-bit
// integer products (more accurate than an FP64 stencil); form 0 when every leaf type has cx = cy and lambda = 0, else 1;
// zero_state when u is identically zero; rleaf [B][L]
// scratch for the per-request maximum rmax (may be null)
// (gsrc, arena: the leaves' Dirichlet row tables, MixLeaf::gsrc of leaf k = gsrc + 4 n k, and their arena)
void mx_leaf_residual(cudaStream_t st, const MixCoef* coefs, int form, const MixLeaf* leaves, int L, int B, int n,
                      int zero_state, const double* f, const double* u64, float* q, float* rleaf, double* rmax,
                      const MxRow* gsrc, const char* arena);
void mx_root(cudaStream_t st, int m, int B, const double* a, const double* r, double* g);
// Robin root data in the mixed form (fixed a, b per block solver; r per request, [B][m]):
// rho = r - a g64 - b h64 (FP64 -> FP32); rhs = rho - b h32; g64 += dg
void mx_root_residual(cudaStream_t st, int m, int B, const double* a, const double* b, const double* r,
                      const double* g64, const double* h64, float* rho);
void mx_root_rhs(cudaStream_t st, int m, int B, const float* b32, const float* rho, const float* h32, float* rhs);
void mx_root_update(cudaStream_t st, int m, int B, const float* dg, double* g64);
// Z = P I for the row order perm of an LU (its solve then gives the inverse)
void mx_perm_identity(cudaStream_t st, int m, const int* perm, double* Z);
// rmax[b] = max over leaves of rleaf[b][leaf]
void mx_rmax(cudaStream_t st, const float* rleaf, int L, int B, double* rmax);
// 16 x 16 constant-coefficient leaves: the zero-state residual (as mx_leaf_residual with zero_state)
// fused with the first pass's Neumann step (as mx_leaf32 LEAF_NEUMANN on its output)
void mx_leaf16_first(cudaStream_t st, const LeafType32* types, const MixCoef* coefs, const MixLeaf* leaves, int L,
                     int B, const double* f, float* q, float* rleaf, double* rmax, const MxRow* gsrc,
                     const char* arena);
// 16 x 16 leaves of residual form 0: the exact residual (as mx_leaf_residual) fused with the next
// pass's Neumann step
void mx_leaf16_residual_neumann(cudaStream_t st, const LeafType32* types, const MixCoef* coefs, const MixLeaf* leaves,
                                int L, int B, const double* f, const double* u64, float* q, float* rleaf, double* rmax,
                                const MxRow* gsrc, const char* arena);

// Variable-coefficient (FivePointStencil) leaves of the mixed form (ef_mixed_fp.cu), indexed by leaf.
struct MixFp {
    float* blocks;  // n block rows x {L_jj^-1, L_j,j-1, U_jj^-1, U_j,j+1} (n x n each) of the band LU, FP32
    float* bcoef;   // 4n boundary coupling coefficients (WESN)
    double* coef;   // 5 x n*n FP64 stencil coefficients cW, cE, cS, cN, cC
    double dtn_x, dtn_y;
};
// stencil table, FP32 boundary coefficients and the block rows of the band LU (from the FP64 factors)
void mx_fp_convert(cudaStream_t st, const FpLeaf* src, const MixFp* dst, int L, int n);
size_t mx_fp_leaf_smem(int n);
// block triangular solves, one CTA per (leaf, group of requests); modes LEAF_NEUMANN / LEAF_SOLVE
void mx_fp_leaf32(cudaStream_t st, int mode, const MixFp* fps, const MixLeaf* leaves, int L, int B, int n,
                  const float* q, double* u64, int accumulate);
void mx_fp_residual(cudaStream_t st, const MixFp* fps, const MixLeaf* leaves, int L, int B, int n, int zero_state,
                    const double* f, const double* u64, float* q, float* rleaf, double* rmax);

// ------------------------------------------------------------------------------------------------
// Merge / upward / downward kernels
// ------------------------------------------------------------------------------------------------
template <class Real>
struct MergeItemT {
    const Real* Tc[4];  // children's (coarsened) T, 4s x 4s
    Real* X;            // 4s x 4s (LU in place)
    int* piv;           // 4s
    int* perm;          // 4s
    Real* RHS;          // 4s x 12s  = [S (WESN columns) | X^{-1}]
    Real* H;            // 8s x 2s compact: row p holds the two interface blocks adjacent to c(p)
    Real* T;            // 8s x 8s, WESN
    const Real* hc[4];  // children's (coarsened) h, 4s
    Real* h;            // own h, 8s
    Real* hd;           // 4s, interface differences of the children's h
    Real* w;            // 4s
    const Real* gf;     // own full-size g, 8s
    Real* gc[4];        // children's g (at coarsened size), 4s
};
using MergeItem = MergeItemT<double>;
using MergeItem32 = MergeItemT<float>;

// X, H and T (= T_LHS) from the children (build, step 1).
void merge_gather_xht(cudaStream_t st, const MergeItem* items, int nitems, int s);
// RHS = P [S_RHS | I] with the row permutation of the LU of X (build, step 3).
void merge_gather_rhs(cudaStream_t st, const MergeItem* items, int nitems, int s);

// Per-side coarsening of T (4nf x 4nf -> 4nc x 4nc): L21 T L12  (SpecialMatrices.hpp:93-173).
void coarsen_T(cudaStream_t st, const double* const* Tin, double* const* Tout, int nitems, int nf);
// FP32 versions of the build gathers for the mixed-precision build
void merge_gather_xht32(cudaStream_t st, const MergeItem32* items, int nitems, int s);
void merge_gather_rhs32(cudaStream_t st, const MergeItem32* items, int nitems, int s);
void coarsen_T32(cudaStream_t st, const float* const* Tin, float* const* Tout, int nitems, int nf);
// element-wise precision changes of `count` items of `len` values each
void widen_batched(cudaStream_t st, const float* const* in, double* const* out, long long len, int count);
void narrow_batched(cudaStream_t st, const double* const* in, float* const* out, long long len, int count);
// Per-side fine-to-coarse averaging of h (4nf -> 4nc).
void coarsen_vec(cudaStream_t st, const double* const* vin, double* const* vout, int nitems, int nf);
// Per-side coarse-to-fine interpolation of g (4nc -> 4nf).
void uncoarsen_vec(cudaStream_t st, const double* const* vin, double* const* vout, int nitems, int nf);

// hdiff = h_upper - h_lower gathered from the children (upward, step 1).
void upward_hdiff(cudaStream_t st, const MergeItem* items, int nitems, int s);
// w = X^{-1} hdiff (upward, step 2): one warp per row, streamed double2 loads.
void upward_w(cudaStream_t st, const MergeItem* items, int nitems, int s);
// h = H w + h_ext (upward, step 3).
void upward_h(cudaStream_t st, const MergeItem* items, int nitems, int s);
// u_Gamma = S gf (+ w) and scatter of the children's Dirichlet data (downward).
void downward(cudaStream_t st, const MergeItem* items, int nitems, int s, int add_w);

// Root Dirichlet data.  diag: g = (r - b.h) / a.  general: A = diag(a) + diag(b) T; rhs = r - b.h
void root_diag(cudaStream_t st, int m, const double* a, const double* b, const double* r,
               const double* h, double* g);
void root_assemble(cudaStream_t st, int m, const double* a, const double* b, const double* T,
                   double* A);
void root_rhs(cudaStream_t st, int m, const double* b, const double* r, const double* h,
              const int* perm, double* rhs);
// flag = 1 when (a, b) equal (a0, b0) bit for bit, else 0
void root_same(cudaStream_t st, int m, const double* a, const double* b, const double* a0, const double* b0,
               int* flag);

void fill_zero(cudaStream_t st, double* p, long long n);
// dst[k][0..len[k]) = src[k][0..len[k]) for k < count
void copy_batched(cudaStream_t st, const double* const* src, double* const* dst, const long long* len, int count);

}  // namespace efgb
