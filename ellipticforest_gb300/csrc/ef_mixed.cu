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
#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <stdexcept>

#include "ef_kernels.cuh"
#include "ef_mixed_common.cuh"

namespace cg = cooperative_groups;

namespace efgb {

std::atomic<bool> g_general_residual{false};
std::atomic<bool> g_level_interface{false};

namespace {

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

// the same with four requests per thread (B % 4 == 0): three float4 loads in flight, a quarter of
// the threads and blocks
__global__ void k_mx_hdiff4(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int B4 = B >> 2, tot = 4 * s * B4;
    for (int e4 = blockIdx.x * blockDim.x + threadIdx.x; e4 < tot; e4 += gridDim.x * blockDim.x) {
        const int r = e4 / B4, b = (e4 - r * B4) * 4;
        const int I = r / s, o = r - I * s;
        const long long rb = (long long)r * B + b;
        const float4 hu = *reinterpret_cast<const float4*>(it.hc[mx_upper_child(I)] + (long long)mx_q_upper(I, o, s) * B + b);
        const float4 hl = *reinterpret_cast<const float4*>(it.hc[mx_lower_child(I)] + (long long)mx_q_lower(I, o, s) * B + b);
        const float4 m = *reinterpret_cast<const float4*>(it.m + rb);
        *reinterpret_cast<float4*>(it.hd + rb) =
            make_float4(hu.x - hl.x - m.x, hu.y - hl.y - m.y, hu.z - hl.z - m.z, hu.w - hl.w - m.w);
    }
}

// ---- FP32 node GEMMs: Y[rows][B] = A[rows][K] X[K][B] over all nodes of one group -----------------
//
// The operators of a group are stored back to back (one row-major matrix of cnt * rows_item rows)
// and streamed by TMA in tiles of RT rows x 32 columns with the 128-byte swizzle; the request block
// X (batch index fastest) is staged by cp.async.  Every thread owns 4 rows x 4 requests and reads
// both operands as float4 from shared memory.  Top levels, whose few long rows would leave most SMs
// idle, split K over the CTAs of a thread-block cluster and add the partial tiles through
// distributed shared memory in rank order (deterministic).
//   W    : w  = X^{-1} hd          rows 4s, K 4s
//   H    : h  = H [w_Ia; w_Ib] + hc rows 8s, K 2s (compact H; a tile never spans two children)
//   DOWN : u  = S gf + w           rows 4s, K 8s; u goes to both children and into u_Gamma (FP64)
constexpr int kKC = 32;      // K columns per stage (128 bytes of FP32: one swizzle row)
constexpr int kStages = 3;

// floats per A stage: rt rows of 32, rounded up to a 1024-byte multiple
__host__ __device__ __forceinline__ int mx_astage_floats(int rt) { return ((rt * kKC * 4 + 1023) / 1024) * 256; }
inline size_t mx_gemm_smem(int rt, int BN) {
    return 1024 + size_t(kStages) * mx_astage_floats(rt) * 4 + size_t(kStages) * kKC * BN * 4 + (kStages + 1) * 8;
}

// one tile of rt rows: its node, its row offset and the rows of X it multiplies
struct MxTile {
    int item, tl, row0, kb;
    const float* X1;  // X rows k < kb
    const float* X2;  // X rows k >= kb (indexed with the same k)
};

template <int KIND>
__device__ __forceinline__ MxTile mx_tile(const MixItem* __restrict__ items, int s, int B, int rt, int tpi,
                                          int tile) {
    MxTile t;
    t.item = tile / tpi;
    t.tl = tile - t.item * tpi;
    t.row0 = t.tl * rt;
    const MixItem& it = items[t.item];
    if (KIND == MX_W) { t.X1 = it.hd; t.X2 = t.X1; t.kb = 4 * s; }
    else if (KIND == MX_DOWN) { t.X1 = it.gf; t.X2 = t.X1; t.kb = 8 * s; }
    else {
        int c, q, Ia, Ib;
        mx_ext_map(t.row0, s, c, q);
        mx_child_ifaces(c, Ia, Ib);
        t.X1 = it.w + (long long)Ia * s * B;
        t.X2 = it.w + (long long)(Ib - 1) * s * B;  // row k >= s of [w_Ia; w_Ib] is w_Ib[k - s]
        t.kb = s;
    }
    return t;
}

// Work list of a CTA: a split launch (ksplit > 1, one cluster per tile) gives each CTA one K range of
// one tile; otherwise the CTA strides over tiles (persistent), so the TMA pipeline runs on across
// tile boundaries and each epilogue overlaps the next tile's loads.
template <int BN, int KIND>
__global__ void __launch_bounds__(128, KIND == MX_W ? 5 : 4) k_mx_gemm(const __grid_constant__ CUtensorMap tmA,
                                                 const MixItem* __restrict__ items, int s, int B, int rt,
                                                 int ksplit, int ntiles, int* __restrict__ err) {
    constexpr int TXN = BN / 4;
    // dynamic shared memory: kStages A stages of rt x 32 floats (1024-byte aligned for the 128-byte
    // swizzle), kStages X stages of 32 x BN floats, kStages mbarriers
    extern __shared__ unsigned char mx_smem[];
    const int astage = mx_astage_floats(rt);
    float* As0 = reinterpret_cast<float*>(mx_smem + ((1024u - (smem_u32(mx_smem) & 1023u)) & 1023u));
    float* Xs0 = As0 + kStages * astage;
    unsigned long long* full = reinterpret_cast<unsigned long long*>(Xs0 + kStages * kKC * BN);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int tx = tid % TXN, ty = tid / TXN;
    const int rq = rt / 4;  // thread rows: ty + i*rq, i < 4
    int rows_item, K;
    mx_shape<KIND>(s, rows_item, K);
    const int tpi = rows_item / rt;
    const int nkc = (K + kKC - 1) / kKC;
    const bool vecx = (B & 3) == 0;
    int first_tile, tile_step, nunits, cpu, cbase;
    if (ksplit > 1) {
        const int kp = blockIdx.x % ksplit;
        const int cpp = (nkc + ksplit - 1) / ksplit;
        first_tile = blockIdx.x / ksplit;
        tile_step = 0;
        nunits = 1;
        cbase = min(nkc, kp * cpp);
        cpu = min(nkc, cbase + cpp) - cbase;
    } else {
        first_tile = blockIdx.x;
        tile_step = gridDim.x;
        nunits = first_tile < ntiles ? (ntiles - 1 - first_tile) / tile_step + 1 : 0;
        cbase = 0;
        cpu = nkc;
    }
    const int total = cpu > 0 ? nunits * cpu : 0;
    const int b0 = blockIdx.y * BN;
    const unsigned tile_bytes = unsigned(rt) * kKC * sizeof(float);

    unsigned long long* never = full + kStages;  // nothing arrives on it (failure-path test)
    if (tid == 0) {
        for (int st = 0; st < kStages; ++st) mbar_init(&full[st], 1);
        mbar_init(never, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    __syncthreads();

    // the issuing side walks the work list in order: its tile is looked up once per unit and its
    // chunk advances by a counter (no divisions, no item reads on the way to each copy)
    int iss_unit = 0, iss_ch = 0;
    MxTile iss_t = {};
    if (total > 0) iss_t = mx_tile<KIND>(items, s, B, rt, tpi, first_tile);
    auto issue = [&](int st) {
        if (iss_ch == cpu) {
            iss_ch = 0;
            ++iss_unit;
            iss_t = mx_tile<KIND>(items, s, B, rt, tpi, first_tile + iss_unit * tile_step);
        }
        const MxTile& t = iss_t;
        const int c = cbase + iss_ch;
        ++iss_ch;
        if (tid == 0)
            tma_load_tile(&tmA, &full[st], As0 + st * astage, c * kKC, t.item * rows_item + t.row0, tile_bytes,
                          l2_evict_first());
        const int k0 = c * kKC;
        if (vecx) {
            for (int e = tid; e < kKC * TXN; e += nt) {
                const int k = e / TXN, col = (e - (e / TXN) * TXN) * 4;
                const int gk = k0 + k, gb = b0 + col;
                const bool ok = gk < K && gb < B;
                const float* src = ok ? ((gk < t.kb ? t.X1 : t.X2) + (long long)gk * B + gb) : t.X1;
                cp_async16(Xs0 + st * (kKC * BN) + k * BN + col, src, ok ? 16 : 0);
            }
        } else {
            for (int e = tid; e < kKC * BN; e += nt) {
                const int k = e / BN, col = e - (e / BN) * BN;
                const int gk = k0 + k, gb = b0 + col;
                const bool ok = gk < K && gb < B;
                const float* src = ok ? ((gk < t.kb ? t.X1 : t.X2) + (long long)gk * B + gb) : t.X1;
                cp_async4(Xs0 + st * (kKC * BN) + e, src, ok ? 4 : 0);
            }
        }
    };

    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;

    auto epilogue = [&](int tile) {
        const MxTile t = mx_tile<KIND>(items, s, B, rt, tpi, tile);
        const MixItem& it = items[t.item];
        const int bq = b0 + 4 * tx;
        // the rows' epilogue operands (h_ext for H; w and u_Gamma for DOWN) are all loaded before
        // any store: the compiler cannot move a load above a store to another array of the item
        float4 pre4[4];
        double2 preu0[4], preu1[4];
        if (vecx && bq < B && KIND != MX_W) {
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = t.row0 + ty + i * rq;
                const long long rb = (long long)r * B + bq;
                if (KIND == MX_H) {
                    int c, q;
                    mx_ext_map(r, s, c, q);
                    pre4[i] = *reinterpret_cast<const float4*>(it.hc[c] + (long long)q * B + bq);
                } else {
                    pre4[i] = *reinterpret_cast<const float4*>(it.w + rb);
                    if (it.uG) {
                        preu0[i] = reinterpret_cast<const double2*>(it.uG + rb)[0];
                        preu1[i] = reinterpret_cast<const double2*>(it.uG + rb)[1];
                    }
                }
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = t.row0 + ty + i * rq;
            const long long rb = (long long)r * B + bq;
            float v[4] = {acc[i][0], acc[i][1], acc[i][2], acc[i][3]};
            float* dst0;
            float* dst1 = nullptr;
            if (KIND == MX_W) {
                dst0 = it.w + rb;
            } else if (KIND == MX_H) {
                int c, q;
                mx_ext_map(r, s, c, q);
                const float* hp = it.hc[c] + (long long)q * B + bq;
                if (vecx && bq < B) {
                    const float4 hv = pre4[i];
                    v[0] += hv.x; v[1] += hv.y; v[2] += hv.z; v[3] += hv.w;
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (bq + j < B) v[j] += hp[j];
                }
                dst0 = it.h + rb;
            } else {
                const int I = r / s, o = r - (r / s) * s;
                const float* wp = it.w + rb;
                if (vecx && bq < B) {
                    const float4 wv = pre4[i];
                    v[0] += wv.x; v[1] += wv.y; v[2] += wv.z; v[3] += wv.w;
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (bq + j < B) v[j] += wp[j];
                }
                dst0 = it.gc[mx_lower_child(I)] + (long long)mx_q_lower(I, o, s) * B + bq;
                dst1 = it.gc[mx_upper_child(I)] + (long long)mx_q_upper(I, o, s) * B + bq;
                // the FP64 state (none: one launch adds the whole pass's values at its end)
                double* ug = it.uG ? it.uG + rb : nullptr;
                if (!ug) {
                } else if (vecx && bq < B) {
                    double2 u0 = preu0[i], u1 = preu1[i];
                    u0.x += f2d_bits(v[0]); u0.y += f2d_bits(v[1]);
                    u1.x += f2d_bits(v[2]); u1.y += f2d_bits(v[3]);
                    reinterpret_cast<double2*>(ug)[0] = u0;
                    reinterpret_cast<double2*>(ug)[1] = u1;
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        if (bq + j < B) ug[j] += f2d_bits(v[j]);
                }
            }
            if (vecx) {
                if (bq < B) {
                    const float4 o4 = make_float4(v[0], v[1], v[2], v[3]);
                    *reinterpret_cast<float4*>(dst0) = o4;
                    if (KIND == MX_DOWN) *reinterpret_cast<float4*>(dst1) = o4;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (bq + j < B) {
                        dst0[j] = v[j];
                        if (KIND == MX_DOWN) dst1[j] = v[j];
                    }
            }
        }
    };

    int issued = 0;
    for (int p = 0; p < kStages - 1; ++p) {
        if (p < total) { issue(p); ++issued; }
        cp_async_commit();
    }
    int fail_v = -1;
    // consumer position: stage st of phase parity ph; the unit's chunk counter cch triggers the epilogue
    int st = 0, cch = 0, cunit = 0;
    unsigned ph = 0;
    for (int v = 0; v < total; ++v) {
        cp_async_wait<kStages - 2>();
        const bool ok = (v == 0 && g_mx_inject_timeout) ? mbar_wait_ns(never, 0u, 1000000LL) : mbar_wait(&full[st], ph);
        if (__syncthreads_or(!ok)) { fail_v = v; break; }
        if (v + kStages - 1 < total) {
            issue(st == 0 ? kStages - 1 : st - 1);
            ++issued;
        }
        cp_async_commit();
        const float* as = As0 + st * astage;
        const float* xs = Xs0 + st * (kKC * BN);
#pragma unroll
        for (int k4 = 0; k4 < kKC / 4; ++k4) {
            float4 a[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = ty + i * rq;
                a[i] = *reinterpret_cast<const float4*>(as + r * kKC + 4 * (k4 ^ (r & 7)));
            }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const float4 x = *reinterpret_cast<const float4*>(xs + (4 * k4 + kk) * BN + 4 * tx);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const float av = kk == 0 ? a[i].x : kk == 1 ? a[i].y : kk == 2 ? a[i].z : a[i].w;
                    acc[i][0] = fmaf(av, x.x, acc[i][0]);
                    acc[i][1] = fmaf(av, x.y, acc[i][1]);
                    acc[i][2] = fmaf(av, x.z, acc[i][2]);
                    acc[i][3] = fmaf(av, x.w, acc[i][3]);
                }
            }
        }
        if (ksplit == 1 && ++cch == cpu) {
            epilogue(first_tile + cunit * tile_step);
            cch = 0;
            ++cunit;
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
        }
        if (++st == kStages) {
            st = 0;
            ph ^= 1u;
        }
    }
    cp_async_wait<0>();
    if (fail_v >= 0) {
        // let the tiles still in flight land before this CTA's shared memory goes away
        for (int v = fail_v; v < issued; ++v) (void)mbar_wait(&full[v % kStages], unsigned(v / kStages) & 1u);
        if (tid == 0) atomicExch(err, 1);
    }
    __syncthreads();
    if (ksplit == 1) return;

    // partial tiles -> rank 0 of the cluster through distributed shared memory
    cg::cluster_group cluster = cg::this_cluster();
    float* red = As0;
#pragma unroll
    for (int i = 0; i < 4; ++i)
        *reinterpret_cast<float4*>(red + (ty + i * rq) * BN + 4 * tx) =
            make_float4(acc[i][0], acc[i][1], acc[i][2], acc[i][3]);
    cluster.sync();
    const bool lead = cluster.block_rank() == 0;
    if (lead) {
        for (int rk = 1; rk < ksplit; ++rk) {
            const float* rr = cluster.map_shared_rank(red, rk);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const float4 v = *reinterpret_cast<const float4*>(rr + (ty + i * rq) * BN + 4 * tx);
                acc[i][0] += v.x; acc[i][1] += v.y; acc[i][2] += v.z; acc[i][3] += v.w;
            }
        }
    }
    cluster.sync();
    if (lead && fail_v < 0) epilogue(first_tile);
}

// ---- residual: interface data of the state -------------------------------------------------------
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

// the same with four requests per thread (B % 4 == 0): 32-byte loads and stores, every load of a
// thread issued before its stores
__global__ void k_mx_scatter64_4(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int m4 = 4 * s, m8 = 8 * s, B4 = B >> 2;
    for (int e4 = blockIdx.x * blockDim.x + threadIdx.x; e4 < (m8 + m4) * B4; e4 += gridDim.x * blockDim.x) {
        const int row = e4 / B4, b = (e4 - row * B4) * 4;
        if (row < m8) {
            int c, q;
            mx_ext_map(row, s, c, q);
            const double2* src = reinterpret_cast<const double2*>(it.gf64 + (long long)row * B + b);
            const double2 v0 = src[0], v1 = src[1];
            double2* dst = reinterpret_cast<double2*>(it.gc64[c] + (long long)q * B + b);
            dst[0] = v0;
            dst[1] = v1;
        } else {
            const int r = row - m8, I = r / s, o = r - (r / s) * s;
            const double2* src = reinterpret_cast<const double2*>(it.uG + (long long)r * B + b);
            const double2 v0 = src[0], v1 = src[1];
            double2* d0 = reinterpret_cast<double2*>(it.gc64[mx_lower_child(I)] + (long long)mx_q_lower(I, o, s) * B + b);
            double2* d1 = reinterpret_cast<double2*>(it.gc64[mx_upper_child(I)] + (long long)mx_q_upper(I, o, s) * B + b);
            d0[0] = v0;
            d0[1] = v1;
            d1[0] = v0;
            d1[1] = v1;
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
            it.mout[f] = d2f_rn_bits(ml - mu);
        }
    }
}

// the same with four requests per thread (B % 4 == 0)
__global__ void k_mx_flux_up4(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int m4 = 4 * s, m8 = 8 * s, B4 = B >> 2;
    for (int e4 = blockIdx.x * blockDim.x + threadIdx.x; e4 < (m8 + m4) * B4; e4 += gridDim.x * blockDim.x) {
        const int row = e4 / B4, b = (e4 - row * B4) * 4;
        if (row < m8) {
            int c, q;
            mx_ext_map(row, s, c, q);
            const double2* src = reinterpret_cast<const double2*>(it.hc64[c] + (long long)q * B + b);
            const double2 v0 = src[0], v1 = src[1];
            double2* dst = reinterpret_cast<double2*>(it.h64 + (long long)row * B + b);
            dst[0] = v0;
            dst[1] = v1;
        } else {
            const int r = row - m8, I = r / s, o = r - (r / s) * s;
            const double2* pl = reinterpret_cast<const double2*>(it.hc64[mx_lower_child(I)] + (long long)mx_q_lower(I, o, s) * B + b);
            const double2* pu = reinterpret_cast<const double2*>(it.hc64[mx_upper_child(I)] + (long long)mx_q_upper(I, o, s) * B + b);
            const double2 l0 = pl[0], l1 = pl[1], u0 = pu[0], u1 = pu[1];
            *reinterpret_cast<float4*>(it.mout + (long long)r * B + b) =
                make_float4(d2f_rn_bits(l0.x - u0.x), d2f_rn_bits(l0.y - u0.y), d2f_rn_bits(l1.x - u1.x),
                            d2f_rn_bits(l1.y - u1.y));
        }
    }
}

// The same two steps on a tree without coarsening steps, where every row is copied unchanged from
// level to level: the leaves' residual kernels read their Dirichlet rows where they live (the
// root data and the ancestors' interface states, through MixLeaf::gsrc), and every interface row
// of every node takes its flux mismatch straight from the edge fluxes of the two leaves that meet
// there -- one launch instead of a scatter and a flux step per level.
// The index type I of these grid-stride kernels is int whenever the element count fits (the launchers
// choose): a 64-bit integer division runs on GB300's narrow FP64 pipe, a 32-bit one does not.
template <class I>
__global__ void k_mx_mismatch(const char* __restrict__ arena, const MxMis* __restrict__ rows, I nrows, int B) {
    if ((B & 3) == 0) {
        const int B4 = B >> 2;
        for (I e4 = blockIdx.x * (I)blockDim.x + threadIdx.x; e4 < nrows * B4; e4 += (I)gridDim.x * blockDim.x) {
            const I r = e4 / B4;
            const int b = int(e4 - r * B4) * 4;
            const MxMis m = rows[r];
            const double* lo = mx_row<const double>(arena, m.lo, B) + b;
            const double* up = mx_row<const double>(arena, m.up, B) + b;
            const double2 l0 = *reinterpret_cast<const double2*>(lo), l1 = *reinterpret_cast<const double2*>(lo + 2);
            const double2 u0 = *reinterpret_cast<const double2*>(up), u1 = *reinterpret_cast<const double2*>(up + 2);
            *reinterpret_cast<float4*>(mx_row<float>(arena, m.out, B) + b) = make_float4(d2f_rn_bits(l0.x - u0.x), d2f_rn_bits(l0.y - u0.y),
                                                                d2f_rn_bits(l1.x - u1.x), d2f_rn_bits(l1.y - u1.y));
        }
    } else {
        for (I e = blockIdx.x * (I)blockDim.x + threadIdx.x; e < nrows * B; e += (I)gridDim.x * blockDim.x) {
            const I r = e / B;
            const int b = int(e - r * B);
            const MxMis m = rows[r];
            mx_row<float>(arena, m.out, B)[b] = d2f_rn_bits(mx_row<const double>(arena, m.lo, B)[b] -
                                                            mx_row<const double>(arena, m.up, B)[b]);
        }
    }
}

// The FP64 interface state of every node takes the pass's correction in one launch at the end of the
// downward pass (trees without coarsening steps), instead of a read-modify-write in every DOWN
// epilogue, where its latency sat on the epilogue warps.
template <class I>
__global__ void k_mx_state_add(const char* __restrict__ arena, const MxAdd* __restrict__ rows, I nrows, int B) {
    if ((B & 3) == 0) {
        const int B4 = B >> 2;
        for (I e4 = blockIdx.x * (I)blockDim.x + threadIdx.x; e4 < nrows * B4; e4 += (I)gridDim.x * blockDim.x) {
            const I r = e4 / B4;
            const int b = int(e4 - r * B4) * 4;
            const MxAdd a = rows[r];
            double* ug = mx_row<double>(arena, a.ug, B) + b;
            const float4 u = *reinterpret_cast<const float4*>(mx_row<const float>(arena, a.u, B) + b);
            double2 g0 = *reinterpret_cast<const double2*>(ug), g1 = *reinterpret_cast<const double2*>(ug + 2);
            g0.x += f2d_bits(u.x);
            g0.y += f2d_bits(u.y);
            g1.x += f2d_bits(u.z);
            g1.y += f2d_bits(u.w);
            *reinterpret_cast<double2*>(ug) = g0;
            *reinterpret_cast<double2*>(ug + 2) = g1;
        }
    } else {
        for (I e = blockIdx.x * (I)blockDim.x + threadIdx.x; e < nrows * B; e += (I)gridDim.x * blockDim.x) {
            const I r = e / B;
            const int b = int(e - r * B);
            const MxAdd a = rows[r];
            mx_row<double>(arena, a.ug, B)[b] += f2d_bits(mx_row<const float>(arena, a.u, B)[b]);
        }
    }
}

template <class I>
__global__ void k_mx_gather_rows64(const char* __restrict__ arena, const MxRow* __restrict__ src,
                                   double* __restrict__ dst, int nrows, int B) {
    for (I e = blockIdx.x * (I)blockDim.x + threadIdx.x; e < (I)nrows * B; e += (I)gridDim.x * blockDim.x) {
        const int r = int(e / B), b = int(e - (I)r * B);
        dst[e] = mx_row<const double>(arena, src[r], B)[b];
    }
}

// Exterior points of a parent go to its children unchanged (the pass's FP32 Dirichlet data): rows p
// of gf, p < 8s, to row q of child c.  Its own launch per level, ahead of the level's DOWN GEMM,
// whose epilogue writes the children's interface rows.
__global__ void k_mx_ext32(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int m8 = 8 * s;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m8 * B; e += gridDim.x * blockDim.x) {
        const int p = e / B, b = e - (e / B) * B;
        int c, q;
        mx_ext_map(p, s, c, q);
        it.gc[c][(long long)q * B + b] = it.gf[e];
    }
}
// the same with four requests per thread (B % 4 == 0), two rows' loads ahead of their stores
__global__ void k_mx_ext32_4(const MixItem* __restrict__ items, int s, int B) {
    const MixItem& it = items[blockIdx.y];
    const int m8 = 8 * s, B4 = B >> 2, tot = m8 * B4;
    const int stride = gridDim.x * blockDim.x;
    for (int e4 = blockIdx.x * blockDim.x + threadIdx.x; e4 < tot; e4 += 2 * stride) {
        const int e4b = e4 + stride;
        const int r0 = e4 / B4, r1 = e4b / B4;
        const float4 v0 = reinterpret_cast<const float4*>(it.gf)[e4];
        const float4 v1 = e4b < tot ? reinterpret_cast<const float4*>(it.gf)[e4b] : v0;
        int c, q;
        mx_ext_map(r0, s, c, q);
        reinterpret_cast<float4*>(it.gc[c] + (long long)q * B)[e4 - r0 * B4] = v0;
        if (e4b < tot) {
            mx_ext_map(r1, s, c, q);
            reinterpret_cast<float4*>(it.gc[c] + (long long)q * B)[e4b - r1 * B4] = v1;
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
// float offset of the 4-float chunk c4 of row `row` in an item buffer (row-major)
template <int NT>
__device__ __forceinline__ int mx_xoff(int row, int c4, int n) {
    return row * (NT ? NT : n) + 4 * c4;
}

// FP32 eigenbasis leaf pass over the items (leaf, b), b fastest, for leaf sizes other than 16 (16 x 16
// leaves run k_mx_leaf16).  A group of (n/4)^2 threads owns
// two items; each thread owns a 4 x 4 block of every product of both
//   WT = (V^T F)^T,  G = Dinv o (V^T F V),  U1T = (V G)^T,  u = V G V^T
// with float4 operand reads from shared memory.  One operand of every product is V (it depends on
// n only, so one copy serves all leaf types): read once for the two items, it makes 3 shared loads
// per 32 FMA instead of 4 -- the products are bound by shared-memory wavefronts (a 128-bit load
// costs four).  Each stage overwrites its item's single buffer in place between two barriers, so
// an item holds n*n floats of shared memory.  Every sum runs over t = 0 .. n-1 in order.
// NEUMANN writes h32 = DtN(0, q); SOLVE adds the solution of (g32, q) to the FP64 state u64 (or
// stores it there when accumulate is 0).
template <int MODE, int NT>
__global__ void __launch_bounds__(256, 4) k_mx_leaf32(const LeafType32* __restrict__ types,
                                                   const MixLeaf* __restrict__ leaves, int L, int B, int n_arg,
                                                   int ipc, const float* __restrict__ q, double* __restrict__ u64,
                                                   int accumulate) {
    extern __shared__ __align__(16) float smf[];
    const int n = NT ? NT : n_arg;  // NT > 0: leaf size known at compile time (loops unrolled)
    const int nn = n * n, nb = n / 4, tpi = nb * nb;
    const int istride = nn + 16;
    float* VS = smf;
    float* VT = smf + nn;
    const int tid = threadIdx.x;
    const int grp = tid / tpi, lt = tid - grp * tpi;
    const int bi = lt / nb, bj = lt - (lt / nb) * nb;
    // only the indices stay in registers; the leaf and type records are read where they are used
    int leaf[2], b[2];
    bool act[2];
    float* X[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int item = blockIdx.x * ipc + 2 * grp + k;
        act[k] = 2 * grp + k < ipc && (long long)item < (long long)L * B;
        leaf[k] = act[k] ? item / B : 0;
        b[k] = act[k] ? item - leaf[k] * B : 0;
        X[k] = smf + 2 * nn + (2 * grp + k) * istride;
    }
    {
        const float* V0 = types[0].V;
        for (int e = tid; e < nn; e += blockDim.x) {
            const float v = V0[e];
            VS[e] = v;
            VT[(e % n) * n + e / n] = v;
        }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (!act[k]) continue;
        const float* qq = q + ((long long)b[k] * L + leaf[k]) * nn;
        const MixLeaf lfk = leaves[leaf[k]];
        const LeafType32 tyk = types[lfk.type];
        const float cx = 1.0f / (tyk.dx * tyk.dx), cy = 1.0f / (tyk.dy * tyk.dy);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = 4 * bi + i;
            float4 v = *reinterpret_cast<const float4*>(qq + r * n + 4 * bj);
            if (MODE == LEAF_SOLVE) {
                float t[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = 4 * bj + j;
                    float acc = 0.f;
                    if (r == 0) acc += cx * lfk.g32[(long long)(0 * n + c) * B + b[k]];
                    else if (r == n - 1) acc += cx * lfk.g32[(long long)(1 * n + c) * B + b[k]];
                    if (c == 0) acc += cy * lfk.g32[(long long)(2 * n + r) * B + b[k]];
                    else if (c == n - 1) acc += cy * lfk.g32[(long long)(3 * n + r) * B + b[k]];
                    t[j] += -2.0f * acc;
                }
                v = make_float4(t[0], t[1], t[2], t[3]);
            }
            *reinterpret_cast<float4*>(X[k] + mx_xoff<NT>(r, bj, n)) = v;
        }
    }
    __syncthreads();
    float acc[2][4][4];
    auto zero = [&]() {
#pragma unroll
        for (int k = 0; k < 2; ++k)
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[k][i][j] = 0.f;
    };
    auto fma4 = [&](int k, const float4& x, const float4& y) {
        const float xa[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            acc[k][a][0] = fmaf(xa[a], y.x, acc[k][a][0]);
            acc[k][a][1] = fmaf(xa[a], y.y, acc[k][a][1]);
            acc[k][a][2] = fmaf(xa[a], y.z, acc[k][a][2]);
            acc[k][a][3] = fmaf(xa[a], y.w, acc[k][a][3]);
        }
    };
    // acc[k][a][c] += V[t][4 bi + a] * X_k[t][4 bj + c] over t < n
    auto outer_vp = [&](const float* V) {
#pragma unroll
        for (int t = 0; t < (NT ? NT : n); ++t) {
            const float4 x = *reinterpret_cast<const float4*>(V + t * n + 4 * bi);
            const int o = mx_xoff<NT>(t, bj, n);
            const float4 y0 = *reinterpret_cast<const float4*>(X[0] + o);
            const float4 y1 = *reinterpret_cast<const float4*>(X[1] + o);
            fma4(0, x, y0);
            fma4(1, x, y1);
        }
    };
    // acc[k][a][c] += X_k[t][4 bi + a] * V[t][4 bj + c] over t < n
    auto outer_vq = [&](const float* V) {
#pragma unroll
        for (int t = 0; t < (NT ? NT : n); ++t) {
            const float4 y = *reinterpret_cast<const float4*>(V + t * n + 4 * bj);
            const int o = mx_xoff<NT>(t, bi, n);
            const float4 x0 = *reinterpret_cast<const float4*>(X[0] + o);
            const float4 x1 = *reinterpret_cast<const float4*>(X[1] + o);
            fma4(0, x0, y);
            fma4(1, x1, y);
        }
    };
    // X_k[4 bj + c][4 bi + a] = acc[k][a][c] (the transposed block)
    auto store_t = [&]() {
#pragma unroll
        for (int k = 0; k < 2; ++k)
            if (act[k])
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    *reinterpret_cast<float4*>(X[k] + mx_xoff<NT>(4 * bj + c, bi, n)) =
                        make_float4(acc[k][0][c], acc[k][1][c], acc[k][2][c], acc[k][3][c]);
    };
    // (1) WT[j][k] = sum_i V[i][k] F[i][j]
    zero();
    outer_vp(VS);
    __syncthreads();
    store_t();
    __syncthreads();
    // (2) G[k][l] = Dinv[k][l] sum_j WT[j][k] V[j][l]
    zero();
    outer_vq(VS);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 2; ++k)
        if (act[k]) {
            const float* Dinv = types[leaves[leaf[k]].type].Dinv;
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const float4 d = *reinterpret_cast<const float4*>(Dinv + (4 * bi + a) * n + 4 * bj);
                *reinterpret_cast<float4*>(X[k] + mx_xoff<NT>(4 * bi + a, bj, n)) =
                    make_float4(acc[k][a][0] * d.x, acc[k][a][1] * d.y, acc[k][a][2] * d.z, acc[k][a][3] * d.w);
            }
        }
    __syncthreads();
    // (3) U1T[l][i] = sum_k VT[k][i] G[k][l]
    zero();
    outer_vp(VT);
    __syncthreads();
    store_t();
    __syncthreads();
    if (MODE == LEAF_SOLVE) {
        // (4) u[i][j] = sum_l U1T[l][i] VT[l][j]
        zero();
        outer_vq(VT);
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (!act[k]) continue;
            double* uu = u64 + ((long long)b[k] * L + leaf[k]) * nn;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                double2* row = reinterpret_cast<double2*>(uu + (4 * bi + i) * n + 4 * bj);
                double2 v0 = make_double2(f2d_bits(acc[k][i][0]), f2d_bits(acc[k][i][1]));
                double2 v1 = make_double2(f2d_bits(acc[k][i][2]), f2d_bits(acc[k][i][3]));
                if (accumulate) {
                    const double2 o0 = row[0], o1 = row[1];
                    v0.x += o0.x; v0.y += o0.y;
                    v1.x += o1.x; v1.y += o1.y;
                }
                row[0] = v0;
                row[1] = v1;
            }
        }
    } else {
        // edge values u[i][j] = sum_l U1T[l][i] VT[l][j], four consecutive points of one side per
        // step: W/E (i = 0, n-1) take a broadcast U1T[l][i] and a float4 of VT row l, S/N (j = 0,
        // n-1) a float4 of U1T row l and a broadcast VT[l][j]; the same sums in the same order as
        // one point at a time
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (!act[k]) continue;
            const MixLeaf lfk = leaves[leaf[k]];
            const LeafType32 tyk = types[lfk.type];
            const float dtn_x = 2.0f / tyk.dx, dtn_y = 2.0f / tyk.dy;
            const float* W = X[k];
            for (int g4 = lt; g4 < n; g4 += tpi) {
                const int side = (4 * g4) / n, p0 = 4 * g4 - side * n;
                const int fixed = side == 0 || side == 2 ? 0 : n - 1;
                float4 u = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int l = 0; l < (NT ? NT : n); ++l) {
                    // a float4 along the side and a broadcast value per l
                    const float4 v = *reinterpret_cast<const float4*>(
                        side < 2 ? VT + l * n + p0 : W + mx_xoff<NT>(l, p0 >> 2, n));
                    const float a = side < 2 ? W[mx_xoff<NT>(l, fixed >> 2, n) + (fixed & 3)] : VT[l * n + fixed];
                    u.x = fmaf(a, v.x, u.x);
                    u.y = fmaf(a, v.y, u.y);
                    u.z = fmaf(a, v.z, u.z);
                    u.w = fmaf(a, v.w, u.w);
                }
                const float sc = ((side == 0 || side == 2) ? 1.0f : -1.0f) * (side < 2 ? dtn_x : dtn_y);
                float* hp = lfk.h32 + (long long)(side * n + p0) * B + b[k];
                hp[0] = sc * u.x;
                hp[(long long)B] = sc * u.y;
                hp[2LL * B] = sc * u.z;
                hp[3LL * B] = sc * u.w;
            }
        }
    }
}

// ---- 16 x 16 leaves: register-resident sine transforms ---------------------------------------------
// The eigenbasis V[i][k] = c_k sin(pi (k + 1)(i + 1/2) / 16) satisfies V[15 - i][k] = (-1)^k V[i][k],
// so its rows 0..7 (in constant memory: every FMA takes its coefficient as the constant operand,
// with no shared-memory traffic) define the whole basis.  The odd modes fold twice more: V[7 - i][k]
// = +V[i][k] for k = 1, 5, 9, 13 and -V[i][k] for k = 3, 7, 11, 15, and V[3 - i][k] = +V[i][k] for
// k = 3, 11 and -V[i][k] for k = 7, 15 (sin(n pi - a) = -(-1)^n sin a; the FP32 table keeps these
// equalities exactly).  A 16-point transform is then 88 FMAs and 28 additions on the folded
// combinations instead of 256 FMAs (128 after the first fold alone).
__constant__ float c_mxV16[8 * 16];

// Analysis X[k] = sum_j V[j][k] x[j] over the spatial index, out(k, X[k]) as the outputs are made:
// the even modes from P[j] = x[j] + x[15 - j] (8 x 8), the odd ones from M[j] = x[j] - x[15 - j]
// folded again (4 x 4 and two 2 x 2)
template <class Out>
__device__ __forceinline__ void mx_dst16_fwd(const float (&x)[16], Out&& out) {
    float P[8], M[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        P[j] = x[j] + x[15 - j];
        M[j] = x[j] - x[15 - j];
    }
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
        float a = 0.f;
#pragma unroll
        for (int j = 0; j < 8; ++j) a = fmaf(c_mxV16[j * 16 + k], P[j], a);
        out(k, a);
    }
    float MP[4], MM[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        MP[j] = M[j] + M[7 - j];
        MM[j] = M[j] - M[7 - j];
    }
#pragma unroll
    for (int k = 1; k < 16; k += 4) {
        float a = 0.f;
#pragma unroll
        for (int j = 0; j < 4; ++j) a = fmaf(c_mxV16[j * 16 + k], MP[j], a);
        out(k, a);
    }
    const float Q0 = MM[0] + MM[3], Q1 = MM[1] + MM[2], R0 = MM[0] - MM[3], R1 = MM[1] - MM[2];
    out(3, fmaf(c_mxV16[16 + 3], Q1, c_mxV16[3] * Q0));
    out(11, fmaf(c_mxV16[16 + 11], Q1, c_mxV16[11] * Q0));
    out(7, fmaf(c_mxV16[16 + 7], R1, c_mxV16[7] * R0));
    out(15, fmaf(c_mxV16[16 + 15], R1, c_mxV16[15] * R0));
}
// Synthesis x[i] = sum_k V[i][k] X[k], out(i, x[i], x[15 - i]) for i < 8: x[i] = e_i + o_i, x[15 - i]
// = e_i - o_i with e_i, o_i the sums over the even and odd modes, the o_i from the folded odd modes
template <class Out>
__device__ __forceinline__ void mx_dst16_syn(const float (&X)[16], Out&& out) {
    const float c0 = fmaf(c_mxV16[11], X[11], c_mxV16[3] * X[3]);
    const float c1 = fmaf(c_mxV16[16 + 11], X[11], c_mxV16[16 + 3] * X[3]);
    const float d0 = fmaf(c_mxV16[15], X[15], c_mxV16[7] * X[7]);
    const float d1 = fmaf(c_mxV16[16 + 15], X[15], c_mxV16[16 + 7] * X[7]);
    const float b[4] = {c0 + d0, c1 + d1, c1 - d1, c0 - d0};
    float o[8];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float a = 0.f;
#pragma unroll
        for (int k = 1; k < 16; k += 4) a = fmaf(c_mxV16[i * 16 + k], X[k], a);
        o[i] = a + b[i];
        o[7 - i] = a - b[i];
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        float e = 0.f;
#pragma unroll
        for (int k = 0; k < 16; k += 2) e = fmaf(c_mxV16[i * 16 + k], X[k], e);
        out(i, e + o[i], e - o[i]);
    }
}

// FP32 leaf pass for n = 16: a 16-thread group per item (leaf, b), thread t owning row t (x index).
//   A = F V (rows), G = Dinv o (V^T A) (columns), C = V G (columns), u = C V^T (rows)
// Two transposes per item pass through a 16 x 17 shared buffer (conflict-free both ways) under
// __syncwarp only: an item never leaves its half-warp.  NEUMANN writes h32 = DtN(0, q) from the
// edges of u; SOLVE adds the solution of (g32, q) to the FP64 state u64 (or stores it when
// accumulate is 0).  Steps (2)-(6) on row t of the item's load in x (shared with the fused first
// residual, k_mx_leaf16_first):
template <int MODE>
__device__ __forceinline__ void mx_leaf16_body(float (&x)[16], float* bf, const float* Vs, const LeafType32* __restrict__ types,
                                               int type, const MixLeaf* __restrict__ leaves, int leaf, int b, int L, int B,
                                               int t, bool act, double* __restrict__ u64, int accumulate) {
    float X[16];
    // (2) A[t][l] = sum_j F[t][j] V[j][l]; transpose: this thread takes column l = t
    mx_dst16_fwd(x, [&](int l, float v) { bf[t * 17 + l] = v; });
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = bf[i * 17 + t];
    // (3) G[k][t] = Dinv[k][t] sum_i V[i][k] A[i][t]
    {
        const float* Dinv = types[type].Dinv + t;
        mx_dst16_fwd(x, [&](int k, float v) { X[k] = v * __ldg(Dinv + k * 16); });
    }
    // (4) C[i][t] = sum_k V[i][k] G[k][t]; transpose back: buffer row t holds column t of C
    __syncwarp();
    mx_dst16_syn(X, [&](int i, float lo, float hi) {
        bf[t * 17 + i] = lo;
        bf[t * 17 + 15 - i] = hi;
    });
    __syncwarp();
    if (MODE == LEAF_SOLVE) {
        // (5) u[t][j] = sum_l C[t][l] V[j][l], staged in the buffer (row t)
#pragma unroll
        for (int l = 0; l < 16; ++l) X[l] = bf[l * 17 + t];
        __syncwarp();
        mx_dst16_syn(X, [&](int i, float lo, float hi) {
            bf[t * 17 + i] = lo;
            bf[t * 17 + 15 - i] = hi;
        });
        __syncwarp();
        // (6) the FP64 state, coalesced: thread t takes the value pairs 2 (t + 16 m), m < 8; a first
        // pass stores the doubles' words as they are assembled
        if (act && accumulate) {
            double2* st = reinterpret_cast<double2*>(u64 + ((long long)b * L + leaf) * 256);
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                const int e2 = t + 16 * m, i = e2 >> 3, j = (e2 & 7) * 2;
                double2 v = make_double2(f2d_bits(bf[i * 17 + j]), f2d_bits(bf[i * 17 + j + 1]));
                const double2 o = st[e2];
                v.x += o.x;
                v.y += o.y;
                st[e2] = v;
            }
        } else if (act) {
            uint4* st = reinterpret_cast<uint4*>(u64 + ((long long)b * L + leaf) * 256);
#pragma unroll
            for (int m = 0; m < 8; ++m) {
                const int e2 = t + 16 * m, i = e2 >> 3, j = (e2 & 7) * 2;
                uint4 w;
                f2d_words(bf[i * 17 + j], w.y, w.x);
                f2d_words(bf[i * 17 + j + 1], w.w, w.z);
                st[e2] = w;
            }
        }
    } else {
        // (5) edge values u[i][j] = sum_l C[i][l] V[j][l]: S/N (j = 0, 15) at i = t from row t of C;
        // W (i = 0) on lanes t < 8 and E (i = 15) on lanes t >= 8, each lane the pair j = t & 7 and
        // 15 - (t & 7) from one row of C (V[15 - j][l] = (-1)^l V[j][l])
        float e = 0.f, o = 0.f, ew = 0.f, ow = 0.f;
        const int jw = t & 7, rc = t < 8 ? 0 : 15;
        __syncthreads();  // the block's basis copy Vs (written at kernel start by every thread) is complete
#pragma unroll
        for (int l = 0; l < 16; l += 2) {
            e = fmaf(c_mxV16[l], bf[l * 17 + t], e);
            o = fmaf(c_mxV16[l + 1], bf[(l + 1) * 17 + t], o);
            ew = fmaf(bf[l * 17 + rc], Vs[jw * 17 + l], ew);
            ow = fmaf(bf[(l + 1) * 17 + rc], Vs[jw * 17 + l + 1], ow);
        }
        if (act) {
            const float dtn_x = 2.0f / types[type].dx, dtn_y = 2.0f / types[type].dy;
            float* h = leaves[leaf].h32 + b;
            const float sw = t < 8 ? dtn_x : -dtn_x;
            const int side = t < 8 ? 0 : 1;
            h[(long long)(side * 16 + jw) * B] = sw * (ew + ow);
            h[(long long)(side * 16 + 15 - jw) * B] = sw * (ew - ow);
            h[(long long)(2 * 16 + t) * B] = dtn_y * (e + o);
            h[(long long)(3 * 16 + t) * B] = -dtn_y * (e - o);
        }
    }
}

template <int MODE>
__global__ void __launch_bounds__(256, MODE == LEAF_SOLVE ? 4 : 3) k_mx_leaf16(const LeafType32* __restrict__ types,
                                                   const MixLeaf* __restrict__ leaves, int L, int B,
                                                   const float* __restrict__ q, double* __restrict__ u64,
                                                   int accumulate) {
    __shared__ float buf[16 * 272];
    __shared__ float Vs[16 * 17];
    const int tid = threadIdx.x, slot = tid >> 4, t = tid & 15;
    const int item = blockIdx.x * 16 + slot;  // L * B < 2^31 (the launchers check)
    const bool act = item < L * B;
    const int leaf = act ? item / B : 0;
    const int b = act ? item - leaf * B : 0;
    float* bf = buf + slot * 272;
    if (MODE == LEAF_NEUMANN) {
        // the full basis, for the edge sums whose basis row depends on the thread
        const int i = tid >> 4, k = tid & 15;
        const float v = c_mxV16[(i < 8 ? i : 15 - i) * 16 + k];
        Vs[i * 17 + k] = (i >= 8 && (k & 1)) ? -v : v;  // read after the body's block barrier
    }
    const int type = leaves[leaf].type;
    if (MODE == LEAF_SOLVE && accumulate && act) {
        // the item's FP64 state (2 KB, read back at the end) on its way to L2 while the pass runs:
        // 128 bytes a thread
        const double* sp = u64 + ((long long)b * L + leaf) * 256 + t * 16;
        asm volatile("prefetch.global.L2 [%0];" ::"l"(sp));
    }
    float x[16];
    // (1) row t of the load; the solve adds the Dirichlet terms -2 (cx g_x + cy g_y) of the edge cells
    if (act) {
        const float4* qr = reinterpret_cast<const float4*>(q + ((long long)b * L + leaf) * 256 + t * 16);
#pragma unroll
        for (int c4 = 0; c4 < 4; ++c4) {
            const float4 v = qr[c4];
            x[4 * c4] = v.x; x[4 * c4 + 1] = v.y; x[4 * c4 + 2] = v.z; x[4 * c4 + 3] = v.w;
        }
        if (MODE == LEAF_SOLVE) {
            const float* g = leaves[leaf].g32 + b;
            const float dx = types[type].dx, dy = types[type].dy;
            const float cx = 1.0f / (dx * dx), cy = 1.0f / (dy * dy);
            const float gs = g[(long long)(2 * 16 + t) * B], gn = g[(long long)(3 * 16 + t) * B];
            if (t == 0 || t == 15) {
                const long long side = t == 0 ? 0 : 16;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float acc = cx * g[(side + j) * B];
                    if (j == 0) acc += cy * gs;
                    else if (j == 15) acc += cy * gn;
                    x[j] += -2.0f * acc;
                }
            } else {
                x[0] += -2.0f * (cy * gs);
                x[15] += -2.0f * (cy * gn);
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) x[j] = 0.f;
    }
    mx_leaf16_body<MODE>(x, bf, Vs, types, type, leaves, leaf, b, L, B, t, act, u64, accumulate);
}

// The first residual of a block for 16 x 16 leaves fused with the first pass's Neumann step.  The
// residual of the zero state (r = f - 2 cx g_x - 2 cy g_y at the edge cells, the arithmetic of
// k_mx_leaf_residual0_16 bit for bit: f read as coalesced 16-byte pairs, FP64 -> FP32 by integer
// bit operations, the ghost terms through shared memory) is stored as the pass's load q for its
// solve step and handed to the leaf pass body through the transpose buffer instead of memory; the
// edge fluxes of the zero state (FP64) and the items' largest |r| are written as by the residual
// kernel.
__global__ void __launch_bounds__(256, 4) k_mx_leaf16_first(const LeafType32* __restrict__ types,
                                                            const MixCoef* __restrict__ coefs,
                                                            const MixLeaf* __restrict__ leaves, int L, int B,
                                                            const double* __restrict__ f, float* __restrict__ q,
                                                            float* __restrict__ rleaf, const MxRow* __restrict__ gsrc,
                                                            const char* __restrict__ arena) {
    __shared__ float buf[16 * 272];
    __shared__ float Vs[16 * 17];
    __shared__ float gts[16 * 80];  // 80 floats per item: the two items of a warp use other banks
    const int tid = threadIdx.x, slot = tid >> 4, t = tid & 15;
    const int item = blockIdx.x * 16 + slot;  // L * B < 2^31 (the launchers check)
    const bool act = item < L * B;
    const int leaf = act ? item / B : 0;
    const int b = act ? item - leaf * B : 0;
    float* bf = buf + slot * 272;
    {
        // the full basis, for the edge sums whose basis row depends on the thread
        const int i = tid >> 4, k = tid & 15;
        const float v = c_mxV16[(i < 8 ? i : 15 - i) * 16 + k];
        Vs[i * 17 + k] = (i >= 8 && (k & 1)) ? -v : v;  // read after the body's block barrier
    }
    // the item's Dirichlet rows (MixLeaf::gsrc of every leaf is gsrc + 64 leaf in one arena): their
    // table entries are loaded first, independent of the leaf record
    MxRow gr[4];
#pragma unroll
    for (int side = 0; side < 4; ++side) gr[side] = act ? gsrc[leaf * 64 + side * 16 + t] : MxRow{0u, 0u};
    const MixLeaf lf = leaves[leaf];
    const MixCoef cf = coefs[lf.type];
    const long long base = ((long long)b * L + leaf) * 256;
    const double2* f2 = reinterpret_cast<const double2*>(f + base);
    double2 fv[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) fv[m] = act ? f2[t + 16 * m] : make_double2(0.0, 0.0);
    double gv[4];
#pragma unroll
    for (int side = 0; side < 4; ++side) gv[side] = act ? mx_row<const double>(arena, gr[side], B)[b] : 0.0;
    float* gt = gts + slot * 80;
#pragma unroll
    for (int side = 0; side < 4; ++side)
        gt[side * 16 + t] = -2.0f * (side < 2 ? cf.cx32 : cf.cy32) * d2f_rn_bits(gv[side]);
    if (act) {
        // edge fluxes of the zero state, h = -+(2/d) g
        double* h = lf.h64 + b;
        h[(long long)(0 * 16 + t) * B] = -cf.dtn_x * gv[0];
        h[(long long)(1 * 16 + t) * B] = cf.dtn_x * gv[1];
        h[(long long)(2 * 16 + t) * B] = -cf.dtn_y * gv[2];
        h[(long long)(3 * 16 + t) * B] = cf.dtn_y * gv[3];
    }
    __syncwarp();
    float mx = 0.f;
    float2* q2 = reinterpret_cast<float2*>(q + base);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int e2 = t + 16 * m, i = e2 >> 3, j = (e2 & 7) * 2;
        float r0 = d2f_rn_bits(fv[m].x), r1 = d2f_rn_bits(fv[m].y);
        if (i == 0) {
            r0 += gt[j];
            r1 += gt[j + 1];
        } else if (i == 15) {
            r0 += gt[16 + j];
            r1 += gt[16 + j + 1];
        }
        if (j == 0) r0 += gt[32 + i];
        if (j == 14) r1 += gt[48 + i];
        mx = fmaxf(mx, fmaxf(fabsf(r0), fabsf(r1)));
        if (act) q2[e2] = make_float2(r0, r1);
        bf[i * 17 + j] = act ? r0 : 0.f;
        bf[i * 17 + j + 1] = act ? r1 : 0.f;
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (rleaf && act && t == 0) rleaf[(long long)b * L + leaf] = mx;
    __syncwarp();
    float x[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = bf[t * 17 + j];
    mx_leaf16_body<LEAF_NEUMANN>(x, bf, Vs, types, lf.type, leaves, leaf, b, L, B, t, act, nullptr, 0);
}

// Leaf residual r = f - (cx (u_W + u_E) + cy (u_S + u_N) + cc u_C) (stored as the next pass's FP32
// load), where a neighbour across the patch edge is the ghost value 2g - u_C of the Dirichlet face
// data (the discrete operator of FiniteVolumeSolver.cpp:27-223), and the leaf's edge fluxes
// h = +-(2/d)(u_edge - g) (FP64).
//
// GB300's FP64 pipe is narrow (about 2 FMA per clock per SM, and it also carries the 64-bit
// integer <-> floating-point conversions), so the residual runs in 64-bit integer arithmetic on the
// integer pipes instead, and more accurately than an FP64 evaluation:
//  - the item's u and ghost values become fixed point on one scale 2^(Eu - 1081), Eu the largest
//    biased exponent among them, so |M| < 2^59 and every value within 2^6 of the largest is exact
//    (smaller ones keep all bits above 2^-59 of the largest);
//  - the second differences Sx = M_W + M_E - 2 M_C and Sy = M_S + M_N - 2 M_C (ghosts 2 M_g - M_C)
//    are exact integer sums below 2^62: the cancellation that costs an FP64 stencil its digits
//    happens without rounding;
//  - the products cx Sx, cy Sy, lambda M_C are exact 128-bit products with the coefficients'
//    64-bit significands, shifted to one fixed scale 2^sc per item on which the item's largest |f|
//    and largest product are just below 2^61 (a first sweep over the tile measures the largest
//    second difference); r = F - P is one exact subtraction, rounded to FP32 at the end.  The
//    error is a few units of 2^sc, about 2^-59 of the item's largest term (an FP64 stencil errs
//    by 2^-53 of |u|/h^2 per cell).
// Items (leaf, b) with b fastest; each thread owns 4 consecutive cells of one row; the fixed-point
// tile of an item lives in shared memory, and the ghost data and edge fluxes ([4n][B] in HBM) pass
// through shared memory so that a block's consecutive requests read and write them together.
// The largest |r| (as FP32) of every item goes to rleaf[b][leaf] (reduced per request by k_mx_rmax).
// Values below 2^-1022 (FP64 subnormals) of f count as zero; a non-finite u, g or f makes the
// item's residual NaN.
__device__ __forceinline__ int fx_bexp(double v) {
    return int((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ff;
}
// v · 2^(1075 - E - 6) = v · 2^(1081 - E) for E >= 1 the largest exponent of its group: |M| < 2^59
// (truncated toward zero); with a general shift, v · 2^-sc has shift e - 1075 - sc
__device__ __forceinline__ long long fx_shift(double v, int E_off) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    int e = int(bits >> 52) & 0x7ff;
    unsigned long long m = bits & 0xfffffffffffffull;
    if (e) m |= 1ull << 52;
    else e = 1;
    const int sh = e - E_off;
    const unsigned long long a = sh >= 0 ? (m << sh) : (sh > -64 ? (m >> -sh) : 0ull);
    return (bits >> 63) ? -(long long)a : (long long)a;
}
__device__ __forceinline__ long long fx_from(double v, int E) { return fx_shift(v, E - 6); }
// v · 2^-sc for FP64 data (subnormals count as zero); the caller keeps e - 1075 - sc <= 8
__device__ __forceinline__ long long fx_scaled(double v, int sc) {
    return fx_bexp(v) ? fx_shift(v, 1075 + sc) : 0ll;
}
// S · m / 2^d with the exact signed 128-bit product S · m (m a signed 63-bit significand), rounded
// toward minus infinity; d >= 1 and the caller keeps the result below 2^61 in magnitude
__device__ __forceinline__ long long fx_term(long long S, long long m, int d) {
    const long long hi = __mul64hi(S, m);
    const unsigned long long lo = (unsigned long long)S * (unsigned long long)m;
    return d >= 128 ? (hi < 0 ? -1ll : 0ll)
           : d >= 64 ? hi >> (d - 64)
                     : (long long)(((unsigned long long)hi << (64 - d)) | (lo >> d));
}
// FP64 of D · 2^sc rounded to nearest (ties to even); |D| < 2^63, result inside the normal range
__device__ __forceinline__ double fx_to_double(long long D, int sc) {
    const unsigned long long sgn = D < 0 ? 1ull << 63 : 0ull;
    const unsigned long long a = D < 0 ? 0ull - (unsigned long long)D : (unsigned long long)D;
    if (a == 0ull) return 0.0;
    const int lz = __clzll((long long)a);
    const unsigned long long nrm = a << lz;
    unsigned long long m = nrm >> 11;
    const unsigned long long rest = nrm & 0x7ffull;
    if (rest > 0x400ull || (rest == 0x400ull && (m & 1ull))) ++m;
    int be = 1023 + 63 - lz + sc;
    if (m >> 53) { m >>= 1; ++be; }
    if (be <= 0) return __longlong_as_double((long long)sgn);
    if (be >= 2047) return __longlong_as_double((long long)(sgn | 0x7ff0000000000000ull));
    return __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) | (m & 0xfffffffffffffull)));
}

// The same three conversions for the 16 x 16 kernel, written with one variable shift each (the
// general kernel keeps the forms above, so the test comparing the two kernels checks these against
// them): for a shift sh = e - E_off <= s_max, m << sh = (m << s_max) >> (s_max - sh) exactly and
// m >> -sh = (m << s_max) >> (s_max - sh) with truncation, and (m << s_max) < 2^61, so a shift of
// 63 or more gives 0 as a shift of 64 or more does in fx_shift.
__device__ __forceinline__ long long fx_from_1(double v, int E) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int e0 = int(bits >> 52) & 0x7ff;
    const unsigned long long m = (bits & 0xfffffffffffffull) | (e0 ? (1ull << 52) : 0ull);
    const int k = min(E - max(e0, 1), 63);  // 6 - sh
    const unsigned long long a = (m << 6) >> k;
    return (bits >> 63) ? -(long long)a : (long long)a;
}
__device__ __forceinline__ long long fx_scaled_1(double v, int sc) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
    const int e0 = int(bits >> 52) & 0x7ff;
    const unsigned long long m = (bits & 0xfffffffffffffull) | (1ull << 52);
    const int k = min(1083 + sc - e0, 63);  // 8 - sh, sh = e - 1075 - sc <= 8
    const unsigned long long a = e0 ? (m << 8) >> k : 0ull;
    return (bits >> 63) ? -(long long)a : (long long)a;
}
// fx_term with the branch on d taken once per item (d is uniform over an item's lanes)
__device__ __forceinline__ long long fx_term_1(long long S, long long m, int d) {
    const long long hi = __mul64hi(S, m);
    if (d >= 64) return d >= 128 ? (hi < 0 ? -1ll : 0ll) : hi >> (d - 64);
    const unsigned long long lo = (unsigned long long)S * (unsigned long long)m;
    return (long long)(((unsigned long long)hi << (64 - d)) | (lo >> d));
}

// FORM 0: every leaf type has cx = cy and lambda = 0 (one product per cell); FORM 1: general
template <int NT, int FORM>
__global__ void __launch_bounds__(256, FORM == 0 ? 4 : 2) k_mx_leaf_residual(const MixCoef* __restrict__ coefs,
                                                          const MixLeaf* __restrict__ leaves, int L, int B,
                                                          int n_arg, int ipc, const double* __restrict__ f,
                                                          const double* __restrict__ u64, float* __restrict__ q,
                                                          float* __restrict__ rleaf) {
    // per item: n*n fixed-point cells, 4n fixed-point ghosts, 4n FP64 ghosts (later the fluxes)
    extern __shared__ long long fx_tile[];
    __shared__ unsigned smax[64];
    __shared__ int seu[64], sef[64], sbx[64], sby[64];
    __shared__ const MxRow* sg[64];  // the item's Dirichlet data rows
    __shared__ int sgb[64];                   // and its request
    __shared__ double* sh[64];
    const int n = NT ? NT : n_arg;
    const int nn = n * n, tpi = nn / 4, n4 = 4 * n;
    const int tpe = tpi < 256 ? tpi : 256;
    const int slot = threadIdx.x / tpe, lt = threadIdx.x - slot * tpe;
    const long long items = (long long)L * B;
    const int item0 = blockIdx.x * ipc, item = item0 + slot;
    const bool act = slot < ipc && (long long)item < items;
    if (threadIdx.x < ipc) {
        smax[threadIdx.x] = 0u;
        seu[threadIdx.x] = 1;
        sef[threadIdx.x] = 1;
        sbx[threadIdx.x] = 0;
        sby[threadIdx.x] = 0;
        const int it = item0 + int(threadIdx.x);
        if ((long long)it < items) {
            const int lf = it / B, bb = it - lf * B;
            sg[threadIdx.x] = leaves[lf].gsrc;
            sgb[threadIdx.x] = bb;
            sh[threadIdx.x] = leaves[lf].h64 + bb;
        }
    }
    __syncthreads();
    const int leaf = act ? item / B : 0;
    const int b = act ? item - leaf * B : 0;
    const MixCoef cf = coefs[leaves[leaf].type];
    const long long base = ((long long)b * L + leaf) * nn;
    const double* uu = u64 + base;
    const double* ff = f + base;
    long long* tile = fx_tile + (long long)slot * (nn + 2 * n4);
    long long* gfx = tile + nn;
    double* gd = reinterpret_cast<double*>(gfx + n4);
    const int nact = (long long)item0 + ipc <= items ? ipc : int(items - item0);
    // items per block, a compile-time constant for the fixed leaf sizes
    const int IPC = NT ? 256 / (NT * NT / 4 < 256 ? NT * NT / 4 : 256) : ipc;
    // the first loads of f and u are issued before the ghost phase so that the latencies overlap
    double2 pf01 = make_double2(0.0, 0.0), pf23 = pf01, pu01 = pf01, pu23 = pf01;
    if (act) {
        pf01 = *reinterpret_cast<const double2*>(ff + 4 * lt);
        pf23 = *reinterpret_cast<const double2*>(ff + 4 * lt + 2);
        pu01 = *reinterpret_cast<const double2*>(uu + 4 * lt);
        pu23 = *reinterpret_cast<const double2*>(uu + 4 * lt + 2);
    }
    // (0) ghost data of the block's items, requests fastest: the items of a block are consecutive
    // requests of one leaf whenever B is a multiple of ipc, so these reads coalesce
    for (int idx = threadIdx.x; idx < n4 * IPC; idx += blockDim.x) {
        const int k = idx / IPC, s = idx - k * IPC;
        if (s < nact)
            reinterpret_cast<double*>(fx_tile + (long long)s * (nn + 2 * n4) + nn + n4)[k] =
                mx_row<const double>(leaves[0].arena, sg[s][k], B)[sgb[s]];
    }
    __syncthreads();
    // (1) scales: largest biased exponents of u and the ghosts (Eu), and of f (Ef)
    int eu = 1, ef = 1;
    if (act) {
        for (int e4 = lt; e4 < tpi; e4 += tpe) {
            const double2 f01 = e4 == lt ? pf01 : *reinterpret_cast<const double2*>(ff + 4 * e4);
            const double2 f23 = e4 == lt ? pf23 : *reinterpret_cast<const double2*>(ff + 4 * e4 + 2);
            ef = max(max(ef, max(fx_bexp(f01.x), fx_bexp(f01.y))), max(fx_bexp(f23.x), fx_bexp(f23.y)));
            const double2 c01 = e4 == lt ? pu01 : *reinterpret_cast<const double2*>(uu + 4 * e4);
            const double2 c23 = e4 == lt ? pu23 : *reinterpret_cast<const double2*>(uu + 4 * e4 + 2);
            eu = max(max(eu, max(fx_bexp(c01.x), fx_bexp(c01.y))), max(fx_bexp(c23.x), fx_bexp(c23.y)));
        }
        for (int k = lt; k < n4; k += tpe) eu = max(eu, fx_bexp(gd[k]));
    }
    // items of a power-of-two width own whole warps or aligned parts of one: reduce by shuffles first
    const bool seg = (tpe & (tpe - 1)) == 0;
    if (seg)
        for (int o = 1; o < tpe && o < 32; o <<= 1) {
            eu = max(eu, __shfl_xor_sync(0xffffffffu, eu, o));
            ef = max(ef, __shfl_xor_sync(0xffffffffu, ef, o));
        }
    if (act && (!seg || (lt & 31) == 0)) {
        atomicMax(&seu[slot], eu);
        atomicMax(&sef[slot], ef);
    }
    __syncthreads();
    const int Eu = seu[slot], Ef = sef[slot];
    const int T = max(Eu, Ef);
    // (2) fixed-point u and ghosts
    if (act) {
        for (int e4 = lt; e4 < tpi; e4 += tpe) {
            const double2 c01 = e4 == lt ? pu01 : *reinterpret_cast<const double2*>(uu + 4 * e4);
            const double2 c23 = e4 == lt ? pu23 : *reinterpret_cast<const double2*>(uu + 4 * e4 + 2);
            reinterpret_cast<longlong2*>(tile + 4 * e4)[0] = make_longlong2(fx_from(c01.x, Eu), fx_from(c01.y, Eu));
            reinterpret_cast<longlong2*>(tile + 4 * e4)[1] = make_longlong2(fx_from(c23.x, Eu), fx_from(c23.y, Eu));
        }
        for (int k = lt; k < n4; k += tpe) gfx[k] = fx_from(gd[k], Eu);
    }
    __syncthreads();
    // (3) exact second differences and products, one subtraction
    const bool lam = FORM != 0 && cf.lmm != 0, iso = FORM == 0 || cf.iso != 0;
    // the cell's fixed-point centre and second differences (iso: sx = Sx + Sy, the y term unused)
    auto diffs = [&](int e, long long (&c)[4], long long (&sx)[4], long long (&sy)[4]) {
        const int i = e / n, j0 = e - i * n;
        long long xm[4], xp[4];
        {
            const longlong2 a = reinterpret_cast<const longlong2*>(tile + e)[0];
            const longlong2 d = reinterpret_cast<const longlong2*>(tile + e)[1];
            c[0] = a.x; c[1] = a.y; c[2] = d.x; c[3] = d.y;
        }
        if (i > 0) {
            const longlong2 a = reinterpret_cast<const longlong2*>(tile + e - n)[0];
            const longlong2 d = reinterpret_cast<const longlong2*>(tile + e - n)[1];
            xm[0] = a.x; xm[1] = a.y; xm[2] = d.x; xm[3] = d.y;
        } else {
#pragma unroll
            for (int t = 0; t < 4; ++t) xm[t] = 2 * gfx[j0 + t] - c[t];
        }
        if (i < n - 1) {
            const longlong2 a = reinterpret_cast<const longlong2*>(tile + e + n)[0];
            const longlong2 d = reinterpret_cast<const longlong2*>(tile + e + n)[1];
            xp[0] = a.x; xp[1] = a.y; xp[2] = d.x; xp[3] = d.y;
        } else {
#pragma unroll
            for (int t = 0; t < 4; ++t) xp[t] = 2 * gfx[n + j0 + t] - c[t];
        }
        const long long left = j0 > 0 ? tile[e - 1] : 2 * gfx[2 * n + i] - c[0];
        const long long right = j0 + 4 < n ? tile[e + 4] : 2 * gfx[3 * n + i] - c[3];
        const long long ym[4] = {left, c[0], c[1], c[2]};
        const long long yp[4] = {c[1], c[2], c[3], right};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            sx[t] = xm[t] + xp[t] - 2 * c[t];
            sy[t] = ym[t] + yp[t] - 2 * c[t];
            if (iso) sx[t] += sy[t];  // |Sx + Sy| < 1.5 * 2^62
        }
    };
    // (3a) bit length of the item's largest second difference (per direction).  With the leaf size
    // fixed at compile time every thread owns one group of 4 cells (n*n/4 <= 256): its differences
    // stay in registers for (3b)
    constexpr bool ONE = NT != 0 && NT * NT / 4 <= 256;
    int bx = 0, by = 0;
    long long c1[4], sx1[4], sy1[4];
    if (act)
        for (int e4 = lt; e4 < tpi; e4 += tpe) {
            diffs(4 * e4, c1, sx1, sy1);
            // OR of the one's-complement magnitudes has the bit length of the largest (to one bit)
            unsigned long long ox = 0ull, oy = 0ull;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                ox |= (unsigned long long)(sx1[t] ^ (sx1[t] >> 63));
                if (!iso) oy |= (unsigned long long)(sy1[t] ^ (sy1[t] >> 63));
            }
            bx = max(bx, ox ? 65 - __clzll((long long)ox) : 1);
            if (!iso) by = max(by, oy ? 65 - __clzll((long long)oy) : 1);
        }
    if (seg)
        for (int o = 1; o < tpe && o < 32; o <<= 1) {
            bx = max(bx, __shfl_xor_sync(0xffffffffu, bx, o));
            by = max(by, __shfl_xor_sync(0xffffffffu, by, o));
        }
    if (act && (!seg || (lt & 31) == 0)) {
        atomicMax(&sbx[slot], bx);
        atomicMax(&sby[slot], by);
    }
    __syncthreads();
    // (3b) common fixed scale 2^sc: |F| < 2^61 and every product < 2^61 (a term carries
    // 2^(Eu - 1081) times a coefficient below 2^e_coef), so F and up to three terms sum without
    // overflow and the error is a few units of 2^sc, 2^-59 of the item's largest term
    float mx = 0.f;
    if (act) {
        const bool bad = Eu == 0x7ff || Ef == 0x7ff;
        int top = sbx[slot] + Eu - 1081 + cf.ecx;
        if (!iso) top = max(top, sby[slot] + Eu - 1081 + cf.ecy);
        if (lam) top = max(top, 59 + Eu - 1081 + cf.elm);
        const int sc = max(Ef - 1083, top - 61);
        // the 128-bit products carry 2^(Eu - 1144 + e_coef) (63-bit significands): right shifts d >= 2
        // to the common scale; the result leaves through one int64 -> FP32 conversion and two exact
        // power-of-two scalings
        const int dx = sc - (Eu - 1144 + cf.ecx), dy = sc - (Eu - 1144 + cf.ecy), dl = sc - (Eu - 1144 + cf.elm);
        const int sa = max(-126, min(127, sc)), sb = max(-126, min(127, sc - sa));
        const float pa = __uint_as_float(unsigned(127 + sa) << 23), pb = __uint_as_float(unsigned(127 + sb) << 23);
        for (int e4 = lt; e4 < tpi; e4 += tpe) {
            const int e = 4 * e4;
            long long c[4], sx[4], sy[4];
            if (ONE) {
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    c[t] = c1[t];
                    sx[t] = sx1[t];
                    sy[t] = sy1[t];
                }
            } else {
                diffs(e, c, sx, sy);
            }
            const double2 f01 = e4 == lt ? pf01 : *reinterpret_cast<const double2*>(ff + e);
            const double2 f23 = e4 == lt ? pf23 : *reinterpret_cast<const double2*>(ff + e + 2);
            const double fv[4] = {f01.x, f01.y, f23.x, f23.y};
            float rr[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                long long R = fx_scaled(fv[t], sc) - fx_term(sx[t], cf.cxm, dx);
                if (!iso) R -= fx_term(sy[t], cf.cym, dy);
                if (lam) R -= fx_term(c[t], cf.lmm, dl);
                rr[t] = bad ? __int_as_float(0x7fffffff) : __fmul_rn(__fmul_rn(__ll2float_rn(R), pa), pb);
                mx = fmaxf(mx, fabsf(rr[t]));
            }
            *reinterpret_cast<float4*>(q + base + e) = make_float4(rr[0], rr[1], rr[2], rr[3]);
        }
        // (4) edge fluxes of the state, h = +-(2/d)(u_edge - g): the difference of the fixed-point
        // values is exact, then one rounding to FP64
        for (int r = lt; r < n4; r += tpe) {
            const int side = r / n, pos = r - side * n;
            const int cell = side == 0 ? pos : side == 1 ? (n - 1) * n + pos : side == 2 ? pos * n : pos * n + n - 1;
            const double d = side < 2 ? cf.dtn_x : cf.dtn_y;
            const double dv = fx_to_double(tile[cell] - gfx[r], Eu - 1081);
            gd[r] = (side == 0 || side == 2) ? d * dv : -d * dv;
        }
    }
    if (seg)
        for (int o = 1; o < tpe && o < 32; o <<= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (act && (!seg || (lt & 31) == 0)) atomicMax(&smax[slot], __float_as_uint(mx));
    __syncthreads();
    for (int idx = threadIdx.x; idx < n4 * IPC; idx += blockDim.x) {
        const int k = idx / IPC, s = idx - k * IPC;
        if (s < nact)
            sh[s][(long long)k * B] = reinterpret_cast<const double*>(fx_tile + (long long)s * (nn + 2 * n4) + nn + n4)[k];
    }
    if (rleaf && act && lt == 0) rleaf[(long long)b * L + leaf] = __uint_as_float(smax[slot]);
}

// First residual (u identically zero): r = f - 2 cx g_x - 2 cy g_y on the edge cells, r = f inside,
// and the edge fluxes h = -+(2/d) g.  This right-hand side only feeds the first FP32 pass, so it is
// formed in FP32 (the FP64 data converted by bit operations, rounding to nearest); the fluxes stay
// FP64.  Same item layout and ghost/flux staging as k_mx_leaf_residual.
template <int NT>
__global__ void __launch_bounds__(256) k_mx_leaf_residual0(const MixCoef* __restrict__ coefs,
                                                           const MixLeaf* __restrict__ leaves, int L, int B,
                                                           int n_arg, int ipc, const double* __restrict__ f,
                                                           float* __restrict__ q, float* __restrict__ rleaf) {
    extern __shared__ double r0_gd[];  // per item: 4n ghost values, later the fluxes; then 4n floats
    __shared__ unsigned smax[64];
    __shared__ const MxRow* sg[64];  // the item's Dirichlet data rows
    __shared__ int sgb[64];                   // and its request
    __shared__ double* sh[64];
    const int n = NT ? NT : n_arg;
    const int nn = n * n, tpi = nn / 4, n4 = 4 * n;
    const int tpe = tpi < 256 ? tpi : 256;
    const int slot = threadIdx.x / tpe, lt = threadIdx.x - slot * tpe;
    const long long items = (long long)L * B;
    const int item0 = blockIdx.x * ipc, item = item0 + slot;
    const bool act = slot < ipc && (long long)item < items;
    if (threadIdx.x < ipc) {
        smax[threadIdx.x] = 0u;
        const int it = item0 + int(threadIdx.x);
        if ((long long)it < items) {
            const int lf = it / B, bb = it - lf * B;
            sg[threadIdx.x] = leaves[lf].gsrc;
            sgb[threadIdx.x] = bb;
            sh[threadIdx.x] = leaves[lf].h64 + bb;
        }
    }
    const int leaf = act ? item / B : 0;
    const int b = act ? item - leaf * B : 0;
    const long long base = ((long long)b * L + leaf) * nn;
    const double* ff = f + base;
    // the first four loads are issued before the ghost phase so that both latencies overlap
    double2 p01 = make_double2(0.0, 0.0), p23 = p01;
    if (act) {
        p01 = *reinterpret_cast<const double2*>(ff + 4 * lt);
        p23 = *reinterpret_cast<const double2*>(ff + 4 * lt + 2);
    }
    __syncthreads();
    const int nact = (long long)item0 + ipc <= items ? ipc : int(items - item0);
    const int IPC = NT ? 256 / (NT * NT / 4 < 256 ? NT * NT / 4 : 256) : ipc;
    float* gt = reinterpret_cast<float*>(r0_gd + IPC * n4);  // per item: the ghost terms -2 c g (FP32)
    for (int idx = threadIdx.x; idx < n4 * IPC; idx += blockDim.x) {
        const int k = idx / IPC, s = idx - k * IPC;
        if (s < nact) {
            const double g = mx_row<const double>(leaves[0].arena, sg[s][k], B)[sgb[s]];
            r0_gd[s * n4 + k] = g;
            const MixCoef& c = coefs[leaves[(item0 + s) / B].type];
            gt[s * n4 + k] = -2.0f * (k < 2 * n ? c.cx32 : c.cy32) * d2f_rn_bits(g);
        }
    }
    __syncthreads();
    const MixCoef cf = coefs[leaves[leaf].type];
    double* gd = r0_gd + slot * n4;
    const float* gts = gt + slot * n4;
    float mx = 0.f;
    if (act) {
        for (int e4 = lt; e4 < tpi; e4 += tpe) {
            const int e = 4 * e4, i = e / n, j0 = e - i * n;
            const double2 f01 = e4 == lt ? p01 : *reinterpret_cast<const double2*>(ff + e);
            const double2 f23 = e4 == lt ? p23 : *reinterpret_cast<const double2*>(ff + e + 2);
            float rr[4] = {d2f_rn_bits(f01.x), d2f_rn_bits(f01.y), d2f_rn_bits(f23.x), d2f_rn_bits(f23.y)};
            if (i == 0)
#pragma unroll
                for (int t = 0; t < 4; ++t) rr[t] += gts[j0 + t];
            if (i == n - 1)
#pragma unroll
                for (int t = 0; t < 4; ++t) rr[t] += gts[n + j0 + t];
            if (j0 == 0) rr[0] += gts[2 * n + i];
            if (j0 + 4 == n) rr[3] += gts[3 * n + i];
#pragma unroll
            for (int t = 0; t < 4; ++t) mx = fmaxf(mx, fabsf(rr[t]));
            *reinterpret_cast<float4*>(q + base + e) = make_float4(rr[0], rr[1], rr[2], rr[3]);
        }
    }
    __syncthreads();  // the ghost values are read above before the fluxes replace them
    if (act)
        for (int r = lt; r < n4; r += tpe) {
            const int side = r / n;
            const double d = side < 2 ? cf.dtn_x : cf.dtn_y;
            gd[r] = (side == 0 || side == 2) ? -d * gd[r] : d * gd[r];
        }
    const bool seg = (tpe & (tpe - 1)) == 0;
    if (seg)
        for (int o = 1; o < tpe && o < 32; o <<= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (act && (!seg || (lt & 31) == 0)) atomicMax(&smax[slot], __float_as_uint(mx));
    __syncthreads();
    for (int idx = threadIdx.x; idx < n4 * IPC; idx += blockDim.x) {
        const int k = idx / IPC, s = idx - k * IPC;
        if (s < nact) sh[s][(long long)k * B] = r0_gd[s * n4 + k];
    }
    if (rleaf && act && lt == 0) rleaf[(long long)b * L + leaf] = __uint_as_float(smax[slot]);
}

// rmax[b] = max over leaves of rleaf[b][leaf]
__global__ void __launch_bounds__(1024) k_mx_rmax(const float* __restrict__ rleaf, int L, double* __restrict__ rmax) {
    __shared__ float red[1024];
    const float* p = rleaf + (long long)blockIdx.x * L;
    float m = 0.f;
    for (int l = threadIdx.x; l < L; l += blockDim.x) m = fmaxf(m, p[l]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) rmax[blockIdx.x] = double(red[0]);
}

// FP32 copies of S (RHS columns [0,8s)), X^{-1} (RHS columns [8s,12s)) and the compact H
__global__ void k_mx_convert(const MixConv* __restrict__ items, int s) {
    const MixConv& it = items[blockIdx.y];
    const long long m4 = 4LL * s, m12 = 12LL * s;
    const long long nS = m4 * 8 * s, nX = m4 * m4, nH = 16LL * s * s;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nS + nX + nH;
         e += (long long)gridDim.x * blockDim.x) {
        const bool f32 = it.RHS32 != nullptr;
        if (e < nS) {
            const long long r = e / (8 * s), c = e - r * (8 * s);
            it.S[e] = f32 ? it.RHS32[r * m12 + c] : float(it.RHS[r * m12 + c]);
        } else if (e < nS + nX) {
            const long long f = e - nS, r = f / m4, c = f - r * m4;
            it.Xi[f] = f32 ? it.RHS32[r * m12 + 8 * s + c] : float(it.RHS[r * m12 + 8 * s + c]);
        } else {
            const long long f = e - nS - nX;
            it.H32[f] = f32 ? it.Hsrc32[f] : float(it.H[f]);
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

// Robin root data a u + b du/dn = r (HPSAlgorithm.hpp:402-420) in the mixed form.  The root's
// Dirichlet data g are part of the FP64 state; the residual of the root condition is
// rho = r - a g - b h with h the state's exact boundary flux (the root's FP64 edge flux), and a pass
// solves for the correction's root data dg = Z (rho - b h_p) with Z = (diag a + diag b T_root)^{-1}
// (FP32) and h_p the correction's particular flux at the root (the FP32 upward pass).
__global__ void k_mx_root_residual(int m, int B, const double* __restrict__ a, const double* __restrict__ b,
                                   const double* __restrict__ r, const double* __restrict__ g64,
                                   const double* __restrict__ h64, float* __restrict__ rho) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * B; e += gridDim.x * blockDim.x) {
        const int i = e / B, q = e - (e / B) * B;
        rho[e] = d2f_rn_bits(r[(long long)q * m + i] - a[i] * g64[e] - b[i] * h64[e]);
    }
}
__global__ void k_mx_root_rhs(int m, int B, const float* __restrict__ b32, const float* __restrict__ rho,
                              const float* __restrict__ h32, float* __restrict__ rhs) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * B; e += gridDim.x * blockDim.x) {
        const int i = e / B;
        rhs[e] = rho[e] - b32[i] * h32[e];
    }
}
// Z = P I: row r of the permuted identity has its one in column perm[r]
__global__ void k_mx_perm_identity(int m, const int* __restrict__ perm, double* __restrict__ Z) {
    const long long tot = (long long)m * m;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const int r = int(e / m), c = int(e - (e / m) * m);
        Z[e] = perm[r] == c ? 1.0 : 0.0;
    }
}
__global__ void k_mx_root_update(int m, int B, const float* __restrict__ dg, double* __restrict__ g64) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * B; e += gridDim.x * blockDim.x) g64[e] += f2d_bits(dg[e]);
}

inline unsigned mx_grid(long long tot) {
    long long b = (tot + 255) / 256;
    if (b > 8192) b = 8192;
    return unsigned(b < 1 ? 1 : b);
}

template <int BN, int KIND>
int mx_gemm_slots(int rt) {
    static std::atomic<int> slots[65];
    if (!slots[rt].load()) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int threads = (rt / 4) * (BN / 4);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mx_gemm<BN, KIND>, threads, mx_gemm_smem(rt, BN));
        slots[rt].store((sms > 0 ? sms : 1) * (per > 0 ? per : 1));
    }
    return slots[rt].load();
}

template <int BN, int KIND>
void mx_gemm_launch(cudaStream_t st, const CUtensorMap& tm, const MixItem* items, int ntiles, int s, int B, int rt,
                    int ksplit, int* err) {
    const int chunks = (B + BN - 1) / BN;
    unsigned gx;
    if (ksplit > 1) {
        gx = unsigned(ntiles * ksplit);
    } else {
        const int slots = mx_gemm_slots<BN, KIND>(rt) / chunks;
        gx = unsigned(std::max(1, std::min(ntiles, slots)));
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(gx, unsigned(chunks));
    cfg.blockDim = dim3(unsigned((rt / 4) * (BN / 4)));
    cfg.dynamicSmemBytes = mx_gemm_smem(rt, BN);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(ksplit);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = ksplit > 1 ? 1 : 0;
    cudaLaunchKernelEx(&cfg, k_mx_gemm<BN, KIND>, tm, items, s, B, rt, ksplit, ntiles, err);
}

template <int KIND>
void mx_gemm(cudaStream_t st, const CUtensorMap& tm, const MixItem* items, int nitems, int s, int B, int* err,
             int ksplit_req) {
    int rows_item, K;
    mx_shape<KIND>(s, rows_item, K);
    const int rt = mx_tile_rows(KIND == MX_H ? 1 : 0, s);
    const int tiles = nitems * (rows_item / rt);
    const int BN = B <= 8 ? 8 : (B <= 16 ? 16 : 32);
    const int nkc = (K + kKC - 1) / kKC;
    // Split K (one cluster of ksplit CTAs per tile) only while fewer than ~4 CTAs per SM would be in
    // flight and every CTA keeps at least 8 chunks.  Chosen from the tile count alone so that every
    // request's sums are grouped the same way whatever the batch size.
    int ksplit = 1;
    if (ksplit_req > 0) {
        ksplit = std::min(ksplit_req, 8);
        while (ksplit > 1 && nkc < 2 * ksplit) ksplit /= 2;
    } else {
        while (ksplit < 8 && (long long)tiles * ksplit < 608 && nkc >= 16 * ksplit) ksplit *= 2;
    }
    if (BN == 8) mx_gemm_launch<8, KIND>(st, tm, items, tiles, s, B, rt, ksplit, err);
    else if (BN == 16) mx_gemm_launch<16, KIND>(st, tm, items, tiles, s, B, rt, ksplit, err);
    else mx_gemm_launch<32, KIND>(st, tm, items, tiles, s, B, rt, ksplit, err);
    ++g_kernel_launches;
}

}  // namespace

void mx_hdiff(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    if (B % 4 == 0) {
        dim3 g4(mx_grid((long long)s * B), nitems);
        k_mx_hdiff4<<<g4, 256, 0, st>>>(items, s, B);
    } else {
        dim3 g1(mx_grid(4LL * s * B), nitems);
        k_mx_hdiff<<<g1, 256, 0, st>>>(items, s, B);
    }
    ++g_kernel_launches;
}

void mx_gemm(cudaStream_t st, int kind, const CUtensorMap& tm, const MixItem* items, int nitems, int s, int B,
             int* err, int ksplit) {
    if (kind == 0) mx_gemm<MX_W>(st, tm, items, nitems, s, B, err, ksplit);
    else if (kind == 1) mx_gemm<MX_H>(st, tm, items, nitems, s, B, err, ksplit);
    else mx_gemm<MX_DOWN>(st, tm, items, nitems, s, B, err, ksplit);
}

void mx_set_inject_timeout(int on) {
    if (cudaMemcpyToSymbol(g_mx_inject_timeout, &on, sizeof(int)) != cudaSuccess)
        throw std::runtime_error("node GEMM: setting the failure-path test switch failed");
    mx_tc_set_inject_timeout(on);
}

int mx_gemm_max_split(int kind, int s) {
    const int K = kind == 0 ? 4 * s : (kind == 1 ? 2 * s : 8 * s);
    const int nkc = (K + kKC - 1) / kKC;
    int k = 1;
    while (k < 8 && nkc >= 4 * k) k *= 2;
    return k;
}

void mx_scatter64(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    if (B % 4 == 0) {
        dim3 g(mx_grid(3LL * s * B), nitems);
        k_mx_scatter64_4<<<g, 256, 0, st>>>(items, s, B);
    } else {
        dim3 g(mx_grid(12LL * s * B), nitems);
        k_mx_scatter64<<<g, 256, 0, st>>>(items, s, B);
    }
    ++g_kernel_launches;
}

void mx_ext32(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    if (B % 4 == 0) {
        dim3 g(mx_grid(2LL * s * B), nitems);
        k_mx_ext32_4<<<g, 256, 0, st>>>(items, s, B);
    } else {
        dim3 g(mx_grid(8LL * s * B), nitems);
        k_mx_ext32<<<g, 256, 0, st>>>(items, s, B);
    }
    ++g_kernel_launches;
}

void mx_flux_up(cudaStream_t st, const MixItem* items, int nitems, int s, int B) {
    if (B % 4 == 0) {
        dim3 g(mx_grid(3LL * s * B), nitems);
        k_mx_flux_up4<<<g, 256, 0, st>>>(items, s, B);
    } else {
        dim3 g(mx_grid(12LL * s * B), nitems);
        k_mx_flux_up<<<g, 256, 0, st>>>(items, s, B);
    }
    ++g_kernel_launches;
}

void mx_mismatch(cudaStream_t st, const char* arena, const MxMis* rows, long long nrows, int B) {
    if (nrows <= 0) return;
    const long long work = (B % 4 == 0) ? nrows * (B / 4) : nrows * B;
    if (nrows * B <= INT_MAX / 2) k_mx_mismatch<int><<<mx_grid(work), 256, 0, st>>>(arena, rows, int(nrows), B);
    else k_mx_mismatch<long long><<<mx_grid(work), 256, 0, st>>>(arena, rows, nrows, B);
    ++g_kernel_launches;
}

void mx_state_add(cudaStream_t st, const char* arena, const MxAdd* rows, long long nrows, int B) {
    if (nrows <= 0) return;
    const long long work = (B % 4 == 0) ? nrows * (B / 4) : nrows * B;
    if (nrows * B <= INT_MAX / 2) k_mx_state_add<int><<<mx_grid(work), 256, 0, st>>>(arena, rows, int(nrows), B);
    else k_mx_state_add<long long><<<mx_grid(work), 256, 0, st>>>(arena, rows, nrows, B);
    ++g_kernel_launches;
}

void mx_gather_rows64(cudaStream_t st, const char* arena, const MxRow* src, double* dst, int nrows, int B) {
    if (nrows <= 0) return;
    if ((long long)nrows * B <= INT_MAX / 2) k_mx_gather_rows64<int><<<mx_grid((long long)nrows * B), 256, 0, st>>>(arena, src, dst, nrows, B);
    else k_mx_gather_rows64<long long><<<mx_grid((long long)nrows * B), 256, 0, st>>>(arena, src, dst, nrows, B);
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

template <int MODE, int NT>
void mx_leaf32_launch(cudaStream_t st, unsigned grid, unsigned threads, size_t smem, const LeafType32* types,
                      const MixLeaf* leaves, int L, int B, int n, int ipc, const float* q, double* u64,
                      int accumulate) {
    static size_t configured = 48 * 1024;
    if (smem > configured) {
        cudaFuncSetAttribute(k_mx_leaf32<MODE, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        configured = smem;
    }
    k_mx_leaf32<MODE, NT><<<grid, threads, smem, st>>>(types, leaves, L, B, n, ipc, q, u64, accumulate);
}

template <int MODE>
void mx_leaf32_mode(cudaStream_t st, unsigned grid, unsigned threads, size_t smem, const LeafType32* types,
                    const MixLeaf* leaves, int L, int B, int n, int ipc, const float* q, double* u64,
                    int accumulate) {
    // 16 x 16 leaves never come here (k_mx_leaf16)
    if (n == 8) mx_leaf32_launch<MODE, 8>(st, grid, threads, smem, types, leaves, L, B, n, ipc, q, u64, accumulate);
    else if (n == 32) mx_leaf32_launch<MODE, 32>(st, grid, threads, smem, types, leaves, L, B, n, ipc, q, u64, accumulate);
    else mx_leaf32_launch<MODE, 0>(st, grid, threads, smem, types, leaves, L, B, n, ipc, q, u64, accumulate);
}

void mx_set_basis16(cudaStream_t st, const float* V) {
    // rows 0..7 of the 16 x 16 basis (row-major); the copy is ordered on st
    if (cudaMemcpyToSymbolAsync(c_mxV16, V, sizeof(float) * 8 * 16, 0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        throw std::runtime_error("mixed solver: leaf basis upload failed");
}

// Grid of the 16 x 16 leaf kernels (16 items (leaf, request) per block), whose item index is an int
inline unsigned mx_grid16(int L, int B) {
    const long long items = (long long)L * B;
    if (items > INT_MAX - 16) throw std::invalid_argument("mixed solver: leaves x requests must stay below 2^31");
    return unsigned((items + 15) / 16);
}

void mx_leaf32(cudaStream_t st, int mode, const LeafType32* types, const MixLeaf* leaves, int L, int B, int n,
               const float* q, double* u64, int accumulate) {
    if (n == 16) {
        const unsigned grid16 = mx_grid16(L, B);
        if (mode == LEAF_NEUMANN) k_mx_leaf16<LEAF_NEUMANN><<<grid16, 256, 0, st>>>(types, leaves, L, B, q, u64, 0);
        else k_mx_leaf16<LEAF_SOLVE><<<grid16, 256, 0, st>>>(types, leaves, L, B, q, u64, accumulate);
        ++g_kernel_launches;
        return;
    }
    // groups of (n/4)^2 threads, two items per group, up to 256 threads per block
    const int nb = n / 4, tpi = nb * nb, groups = tpi >= 256 ? 1 : 256 / tpi, ipc = 2 * groups;
    const size_t smem = (size_t(2) * n * n + size_t(ipc) * (n * n + 16)) * sizeof(float);
    const long long items = (long long)L * B;
    const unsigned grid = unsigned((items + ipc - 1) / ipc);
    const unsigned threads = unsigned(groups * tpi);
    if (mode == LEAF_NEUMANN)
        mx_leaf32_mode<LEAF_NEUMANN>(st, grid, threads, smem, types, leaves, L, B, n, ipc, q, u64, 0);
    else
        mx_leaf32_mode<LEAF_SOLVE>(st, grid, threads, smem, types, leaves, L, B, n, ipc, q, u64, accumulate);
    ++g_kernel_launches;
}

// First residual for 16 x 16 leaves: 16 threads per item (16 items per block), each converting 16
// cells read as coalesced 16-byte pairs; the item's ghost terms pass through shared memory under
// __syncwarp.  The same arithmetic in the same order as k_mx_leaf_residual0.
__global__ void __launch_bounds__(256) k_mx_leaf_residual0_16(const MixCoef* __restrict__ coefs,
                                                           const MixLeaf* __restrict__ leaves, int L, int B,
                                                           const double* __restrict__ f, float* __restrict__ q,
                                                           float* __restrict__ rleaf) {
    __shared__ float gts[16 * 80];  // 80 floats per item: the two items of a warp use other banks
    const int tid = threadIdx.x, slot = tid >> 4, t = tid & 15;
    const int item = blockIdx.x * 16 + slot;  // L * B < 2^31 (the launchers check)
    const bool act = item < L * B;
    const int leaf = act ? item / B : 0;
    const int b = act ? item - leaf * B : 0;
    const MixLeaf lf = leaves[leaf];
    const MixCoef cf = coefs[lf.type];
    const long long base = ((long long)b * L + leaf) * 256;
    const double2* f2 = reinterpret_cast<const double2*>(f + base);
    // the cells' loads first, then the ghost data at position t of every side
    double2 fv[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) fv[m] = act ? f2[t + 16 * m] : make_double2(0.0, 0.0);
    double gv[4];
#pragma unroll
    for (int side = 0; side < 4; ++side) gv[side] = act ? mx_row<const double>(lf.arena, lf.gsrc[side * 16 + t], B)[b] : 0.0;
    float* gt = gts + slot * 80;
#pragma unroll
    for (int side = 0; side < 4; ++side)
        gt[side * 16 + t] = -2.0f * (side < 2 ? cf.cx32 : cf.cy32) * d2f_rn_bits(gv[side]);
    if (act) {
        // edge fluxes of the zero state, h = -+(2/d) g
        double* h = lf.h64 + b;
        h[(long long)(0 * 16 + t) * B] = -cf.dtn_x * gv[0];
        h[(long long)(1 * 16 + t) * B] = cf.dtn_x * gv[1];
        h[(long long)(2 * 16 + t) * B] = -cf.dtn_y * gv[2];
        h[(long long)(3 * 16 + t) * B] = cf.dtn_y * gv[3];
    }
    __syncwarp();
    float mx = 0.f;
    float2* q2 = reinterpret_cast<float2*>(q + base);
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        const int e2 = t + 16 * m, i = e2 >> 3, j = (e2 & 7) * 2;
        float r0 = d2f_rn_bits(fv[m].x), r1 = d2f_rn_bits(fv[m].y);
        if (i == 0) {
            r0 += gt[j];
            r1 += gt[j + 1];
        } else if (i == 15) {
            r0 += gt[16 + j];
            r1 += gt[16 + j + 1];
        }
        if (j == 0) r0 += gt[32 + i];
        if (j == 14) r1 += gt[48 + i];
        mx = fmaxf(mx, fmaxf(fabsf(r0), fabsf(r1)));
        if (act) q2[e2] = make_float2(r0, r1);
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (rleaf && act && t == 0) rleaf[(long long)b * L + leaf] = mx;
}

// Exact residual for 16 x 16 leaves: the arithmetic of k_mx_leaf_residual (same scales, exact
// second differences, 128-bit products, one rounding; bit-identical results) with 16 threads per
// item and 16 items per block, and no block barrier:
//  - lane t first owns column t of its item: the 16 lanes load the item's rows as 128-byte
//    segments, convert their cells to fixed point and write them into the item's tile in shared
//    memory, whose rows -1 and 16 receive the W and E ghost cells 2 M_g - M_C;
//  - after __syncwarp lane t owns row t: its cells, the rows above and below (ghost rows at the
//    W and E faces) and its own S and N ghost cells give both second differences in registers,
//    and the rest of the cell's work (products, subtraction, rounding, the store of q) follows in
//    that layout;
//  - the item's largest exponents and bit lengths reduce over its 16 lanes by shuffles.
// The tile's rows are 18 words apart (144 B), so the row reads (16-byte vectors) and the column
// writes (8-byte) are both free of bank conflicts; a row's neighbour cells across its 16-byte pairs
// come from the pairs already read.  The items' tiles are 328 words apart (= 16 banks mod 32), so the
// two items of a warp also meet no conflict when the Neumann step reuses the tiles as 17-float-row
// transpose buffers.  FORM 0 keeps the cells' second differences in
// registers between the bit-length sweep and the products and loads f by columns (coalesced),
// handing it to the row owners through the tile; FORM 1 (two differences and the lambda term)
// recomputes them from the tile and loads f by rows (16-byte vectors).
// NEU (FORM 0): the residual then feeds the next pass's Neumann step from registers (the leaf pass
// body on row t of r, the tile reused as its transpose buffer) -- q is still stored for the pass's
// solve step.
template <int FORM, bool NEU>
__global__ void __launch_bounds__(256, 2) k_mx_resid16(const MixCoef* __restrict__ coefs,
                                                       const MixLeaf* __restrict__ leaves, int L, int B,
                                                       const double* __restrict__ f, const double* __restrict__ u64,
                                                       float* __restrict__ q, float* __restrict__ rleaf,
                                                       const LeafType32* __restrict__ types,
                                                       const MxRow* __restrict__ gsrc, const char* __restrict__ arena) {
    static_assert(!NEU || FORM == 0, "the Neumann step is fused with the FORM 0 residual only");
    constexpr int RS = 18, TS = 18 * RS + 4;
    __shared__ __align__(16) long long tiles[16 * TS];
    __shared__ float Vs[NEU ? 16 * 17 : 1];
    if constexpr (NEU) {
        // the full basis, for the Neumann step's edge sums
        const int i = threadIdx.x >> 4, k = threadIdx.x & 15;
        const float v = c_mxV16[(i < 8 ? i : 15 - i) * 16 + k];
        Vs[i * 17 + k] = (i >= 8 && (k & 1)) ? -v : v;  // read after the body's block barrier
    }
    const int tid = threadIdx.x, slot = tid >> 4, t = tid & 15;
    const int item = blockIdx.x * 16 + slot;  // L * B < 2^31 (the launchers check)
    const bool act = item < L * B;
    const int leaf = act ? item / B : 0;
    const int b = act ? item - leaf * B : 0;
    // the item's Dirichlet rows (MixLeaf::gsrc of every leaf is gsrc + 64 leaf in one arena): their
    // table entries are loaded first, independent of the leaf record
    MxRow gr[4];
#pragma unroll
    for (int side = 0; side < 4; ++side) gr[side] = act ? gsrc[leaf * 64 + side * 16 + t] : MxRow{0u, 0u};
    const MixLeaf lf = leaves[leaf];
    const MixCoef cf = coefs[lf.type];
    const long long base = ((long long)b * L + leaf) * 256;
    long long* tl = tiles + slot * TS;  // row r (-1..16) at tl + (r + 1) * RS
    // (0) loads: column t of u and this lane's ghost value on every side
    double uc[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) uc[i] = act ? u64[base + i * 16 + t] : 0.0;
    double gv[4];
#pragma unroll
    for (int side = 0; side < 4; ++side) gv[side] = act ? mx_row<const double>(arena, gr[side], B)[b] : 0.0;
    // (1) largest biased exponent of u and the ghosts (Eu), at least 1
    int eu = 1;
#pragma unroll
    for (int i = 0; i < 16; ++i) eu = max(eu, fx_bexp(uc[i]));
#pragma unroll
    for (int side = 0; side < 4; ++side) eu = max(eu, fx_bexp(gv[side]));
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) eu = max(eu, __shfl_xor_sync(0xffffffffu, eu, o));
    const int Eu = eu;
    // (2) fixed point: the column into the tile, the W/E ghost rows, this lane's S/N ghosts
    long long gx[4];
#pragma unroll
    for (int side = 0; side < 4; ++side) gx[side] = fx_from_1(gv[side], Eu);
    long long top_c, bot_c;  // the column's first and last cells (W and E edge fluxes)
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const long long m = fx_from_1(uc[i], Eu);
        tl[(i + 1) * RS + t] = m;
        if (i == 0) top_c = m;
        if (i == 15) bot_c = m;
    }
    tl[t] = 2 * gx[0] - top_c;
    tl[17 * RS + t] = 2 * gx[1] - bot_c;
    // f, in flight while the second differences are formed: FORM 0 loads column t (coalesced) and
    // moves it to the row owners through the tile once the second differences are formed; FORM 1,
    // which reads the tile again for its products, loads row t (16-byte vectors)
    constexpr bool KEEP = FORM == 0;
    double fc[KEEP ? 16 : 1];
    double2 fr[KEEP ? 1 : 8];
    if constexpr (KEEP) {
#pragma unroll
        for (int i = 0; i < 16; ++i) fc[i] = act ? f[base + i * 16 + t] : 0.0;
    } else {
        const double2* f2 = reinterpret_cast<const double2*>(f + base + t * 16);
#pragma unroll
        for (int m = 0; m < 8; ++m) fr[m] = act ? f2[m] : make_double2(0.0, 0.0);
    }
    __syncwarp();
    // (3) row t: second differences (iso: sx = Sx + Sy) from the rows above and below and the
    // row's own cells, the S/N ghost cells at its ends
    const bool lam = FORM != 0 && cf.lmm != 0, iso = FORM == 0 || cf.iso != 0;
    const long long* rw = tl + (t + 1) * RS;
    if (act) {
        // edge fluxes of the state, h = +-(2/d)(u_edge - g): W/E at column t, S/N at row t; the
        // difference of the fixed-point values is exact, then one rounding to FP64
        double* h = lf.h64 + b;
        h[(long long)(0 * 16 + t) * B] = cf.dtn_x * fx_to_double(top_c - gx[0], Eu - 1081);
        h[(long long)(1 * 16 + t) * B] = -cf.dtn_x * fx_to_double(bot_c - gx[1], Eu - 1081);
        h[(long long)(2 * 16 + t) * B] = cf.dtn_y * fx_to_double(rw[0] - gx[2], Eu - 1081);
        h[(long long)(3 * 16 + t) * B] = -cf.dtn_y * fx_to_double(rw[15] - gx[3], Eu - 1081);
    }
    auto row_diffs = [&](int m, long long (&c)[2], long long (&sx)[2], long long (&sy)[2]) {
        const longlong2 cc = reinterpret_cast<const longlong2*>(rw)[m];
        const longlong2 up = reinterpret_cast<const longlong2*>(rw - RS)[m];
        const longlong2 dn = reinterpret_cast<const longlong2*>(rw + RS)[m];
        const long long left = m > 0 ? rw[2 * m - 1] : 2 * gx[2] - cc.x;
        const long long right = m < 7 ? rw[2 * m + 2] : 2 * gx[3] - cc.y;
        c[0] = cc.x;
        c[1] = cc.y;
        sx[0] = up.x + dn.x - 2 * cc.x;
        sx[1] = up.y + dn.y - 2 * cc.y;
        sy[0] = left + cc.y - 2 * cc.x;
        sy[1] = cc.x + right - 2 * cc.y;
        if (iso) {
            sx[0] += sy[0];
            sx[1] += sy[1];
        }
    };
    // FORM 0: the same differences, the row's pairs read once (a pair's outer neighbours are the
    // adjacent pairs' inner cells)
    auto row_diffs_w = [&](int m, longlong2 cc, long long left, long long right, long long (&sx)[2]) {
        const longlong2 up = reinterpret_cast<const longlong2*>(rw - RS)[m];
        const longlong2 dn = reinterpret_cast<const longlong2*>(rw + RS)[m];
        sx[0] = up.x + dn.x - 2 * cc.x + (left + cc.y - 2 * cc.x);
        sx[1] = up.y + dn.y - 2 * cc.y + (cc.x + right - 2 * cc.y);
    };
    long long ks[KEEP ? 16 : 1];
    unsigned long long ox = 0ull, oy = 0ull;
    longlong2 cur = reinterpret_cast<const longlong2*>(rw)[0];
    long long left = 2 * gx[2] - cur.x;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        long long c[2], sx[2], sy[2];
        if constexpr (KEEP) {
            const longlong2 nxt = reinterpret_cast<const longlong2*>(rw)[m < 7 ? m + 1 : 7];
            const long long right = m < 7 ? nxt.x : 2 * gx[3] - cur.y;
            row_diffs_w(m, cur, left, right, sx);
            left = cur.y;
            cur = nxt;
        } else {
            row_diffs(m, c, sx, sy);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (KEEP) ks[(2 * m + k) % (KEEP ? 16 : 1)] = sx[k];
            ox |= (unsigned long long)(sx[k] ^ (sx[k] >> 63));
            if (!iso) oy |= (unsigned long long)(sy[k] ^ (sy[k] >> 63));
        }
    }
    int bx = ox ? 65 - __clzll((long long)ox) : 1, by = oy ? 65 - __clzll((long long)oy) : 1;
    // largest biased exponent of f (Ef), at least 1
    int ef = 1;
    if constexpr (KEEP) {
#pragma unroll
        for (int i = 0; i < 16; ++i) ef = max(ef, fx_bexp(fc[i]));
    } else {
#pragma unroll
        for (int m = 0; m < 8; ++m) ef = max(ef, max(fx_bexp(fr[m].x), fx_bexp(fr[m].y)));
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) {
        bx = max(bx, __shfl_xor_sync(0xffffffffu, bx, o));
        if (!iso) by = max(by, __shfl_xor_sync(0xffffffffu, by, o));
        ef = max(ef, __shfl_xor_sync(0xffffffffu, ef, o));
    }
    const int Ef = ef;
    // (4) the common scale and the products, as in k_mx_leaf_residual
    const bool bad = Eu == 0x7ff || Ef == 0x7ff;
    int top = bx + Eu - 1081 + cf.ecx;
    if (!iso) top = max(top, by + Eu - 1081 + cf.ecy);
    if (lam) top = max(top, 59 + Eu - 1081 + cf.elm);
    const int sc = max(Ef - 1083, top - 61);
    const int dx = sc - (Eu - 1144 + cf.ecx), dy = sc - (Eu - 1144 + cf.ecy), dl = sc - (Eu - 1144 + cf.elm);
    const int sa = max(-126, min(127, sc)), sb = max(-126, min(127, sc - sa));
    const float pa = __uint_as_float(unsigned(127 + sa) << 23), pb = __uint_as_float(unsigned(127 + sb) << 23);
    float mx = 0.f;
    float4* q4 = reinterpret_cast<float4*>(q + base + t * 16);
    float xr[NEU ? 16 : 1];  // NEU: row t of r
    // r of cells 2m, 2m+1 of the row
    auto finish = [&](const long long (&c)[2], const long long (&sx)[2], const long long (&sy)[2], double2 fv,
                      float& r0, float& r1) {
        float rr[2];
        const double fk[2] = {fv.x, fv.y};
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            long long R = fx_scaled_1(fk[k], sc) - fx_term_1(sx[k], cf.cxm, dx);
            if (!iso) R -= fx_term_1(sy[k], cf.cym, dy);
            if (lam) R -= fx_term_1(c[k], cf.lmm, dl);
            rr[k] = bad ? __int_as_float(0x7fffffff) : __fmul_rn(__fmul_rn(__ll2float_rn(R), pa), pb);
            mx = fmaxf(mx, fabsf(rr[k]));
        }
        r0 = rr[0];
        r1 = rr[1];
    };
    if constexpr (KEEP) {
        // f column t into the tile (every lane has read its rows of u), row t back out
        __syncwarp();
#pragma unroll
        for (int i = 0; i < 16; ++i) tl[(i + 1) * RS + t] = __double_as_longlong(fc[i]);
        __syncwarp();
        const double2* frow = reinterpret_cast<const double2*>(rw);
#pragma unroll
        for (int m2 = 0; m2 < 4; ++m2) {
            float4 r4;
            const long long c0[2] = {0, 0}, sx0[2] = {ks[4 * m2], ks[4 * m2 + 1]};
            const long long sx1[2] = {ks[4 * m2 + 2], ks[4 * m2 + 3]};
            finish(c0, sx0, c0, frow[2 * m2], r4.x, r4.y);
            finish(c0, sx1, c0, frow[2 * m2 + 1], r4.z, r4.w);
            if (act) q4[m2] = r4;
            if (NEU) {
                xr[4 * m2] = r4.x;
                xr[4 * m2 + 1] = r4.y;
                xr[4 * m2 + 2] = r4.z;
                xr[4 * m2 + 3] = r4.w;
            }
        }
    } else {
        // the second differences again from the tile, f again from memory (cached): the fully
        // unrolled sweep would hold too many registers with three products per cell
        const double2* f2 = reinterpret_cast<const double2*>(f + base + t * 16);
#pragma unroll 1
        for (int m2 = 0; m2 < 4; ++m2) {
            float4 r4;
            long long c[2], sx[2], sy[2];
            const double2 fa = act ? f2[2 * m2] : make_double2(0.0, 0.0);
            const double2 fb = act ? f2[2 * m2 + 1] : make_double2(0.0, 0.0);
            row_diffs(2 * m2, c, sx, sy);
            finish(c, sx, sy, fa, r4.x, r4.y);
            row_diffs(2 * m2 + 1, c, sx, sy);
            finish(c, sx, sy, fb, r4.z, r4.w);
            if (act) q4[m2] = r4;
        }
    }
#pragma unroll
    for (int o = 8; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (rleaf && act && t == 0) rleaf[(long long)b * L + leaf] = mx;
    if constexpr (NEU) {
        __syncwarp();  // every lane has read its row of f from the tile
        mx_leaf16_body<LEAF_NEUMANN>(xr, reinterpret_cast<float*>(tl), Vs, types, lf.type, leaves, leaf, b, L, B, t,
                                     act, nullptr, 0);
    }
}

template <int FORM>
void mx_residual_launch(cudaStream_t st, unsigned grid, unsigned threads, size_t smem, const MixCoef* coefs,
                        const MixLeaf* leaves, int L, int B, int n, int ipc, const double* f, const double* u64,
                        float* q, float* rl) {
    if (n == 16)
        k_mx_leaf_residual<16, FORM><<<grid, threads, smem, st>>>(coefs, leaves, L, B, n, ipc, f, u64, q, rl);
    else if (n == 8)
        k_mx_leaf_residual<8, FORM><<<grid, threads, smem, st>>>(coefs, leaves, L, B, n, ipc, f, u64, q, rl);
    else if (n == 32)
        k_mx_leaf_residual<32, FORM><<<grid, threads, smem, st>>>(coefs, leaves, L, B, n, ipc, f, u64, q, rl);
    else
        k_mx_leaf_residual<0, FORM><<<grid, threads, smem, st>>>(coefs, leaves, L, B, n, ipc, f, u64, q, rl);
}

void mx_leaf_residual(cudaStream_t st, const MixCoef* coefs, int form, const MixLeaf* leaves, int L, int B, int n,
                      int zero_state, const double* f, const double* u64, float* q, float* rleaf, double* rmax,
                      const MxRow* gsrc, const char* arena) {
    const int tpi = n * n / 4, tpe = tpi < 256 ? tpi : 256, ipc = 256 / tpe;
    const long long items = (long long)L * B;
    const unsigned grid = unsigned((items + ipc - 1) / ipc);
    // fixed-point tiles: n <= 64 keeps them within the default 48 KB of shared memory
    const size_t smem = size_t(ipc) * (size_t(n) * n + 8 * size_t(n)) * sizeof(long long);
    if (n % 4 != 0 || smem > 48 * 1024) throw std::invalid_argument("leaf residual: leaf size out of range");
    float* rl = rmax ? rleaf : nullptr;
    if (zero_state) {
        const size_t smem0 = size_t(ipc) * 4 * size_t(n) * (sizeof(double) + sizeof(float));
        if (n == 16)
            k_mx_leaf_residual0_16<<<mx_grid16(L, B), 256, 0, st>>>(coefs, leaves, L, B, f, q, rl);
        else if (n == 8)
            k_mx_leaf_residual0<8><<<grid, unsigned(ipc * tpe), smem0, st>>>(coefs, leaves, L, B, n, ipc, f, q, rl);
        else
            k_mx_leaf_residual0<0><<<grid, unsigned(ipc * tpe), smem0, st>>>(coefs, leaves, L, B, n, ipc, f, q, rl);
        ++g_kernel_launches;
        if (rmax) mx_rmax(st, rleaf, L, B, rmax);
        return;
    }
    if (n == 16 && !g_general_residual.load()) {
        const unsigned grid16 = mx_grid16(L, B);
        if (form == 0) k_mx_resid16<0, false><<<grid16, 256, 0, st>>>(coefs, leaves, L, B, f, u64, q, rl, nullptr, gsrc, arena);
        else k_mx_resid16<1, false><<<grid16, 256, 0, st>>>(coefs, leaves, L, B, f, u64, q, rl, nullptr, gsrc, arena);
    } else if (form == 0) {
        mx_residual_launch<0>(st, grid, unsigned(ipc * tpe), smem, coefs, leaves, L, B, n, ipc, f, u64, q, rl);
    } else {
        mx_residual_launch<1>(st, grid, unsigned(ipc * tpe), smem, coefs, leaves, L, B, n, ipc, f, u64, q, rl);
    }
    ++g_kernel_launches;
    if (rmax) mx_rmax(st, rleaf, L, B, rmax);
}

void mx_leaf16_first(cudaStream_t st, const LeafType32* types, const MixCoef* coefs, const MixLeaf* leaves, int L,
                     int B, const double* f, float* q, float* rleaf, double* rmax, const MxRow* gsrc,
                     const char* arena) {
    k_mx_leaf16_first<<<mx_grid16(L, B), 256, 0, st>>>(types, coefs, leaves, L, B, f, q, rmax ? rleaf : nullptr, gsrc,
                                                       arena);
    ++g_kernel_launches;
    if (rmax) mx_rmax(st, rleaf, L, B, rmax);
}

void mx_leaf16_residual_neumann(cudaStream_t st, const LeafType32* types, const MixCoef* coefs, const MixLeaf* leaves,
                                int L, int B, const double* f, const double* u64, float* q, float* rleaf, double* rmax,
                                const MxRow* gsrc, const char* arena) {
    k_mx_resid16<0, true><<<mx_grid16(L, B), 256, 0, st>>>(coefs, leaves, L, B, f, u64, q, rmax ? rleaf : nullptr,
                                                           types, gsrc, arena);
    ++g_kernel_launches;
    if (rmax) mx_rmax(st, rleaf, L, B, rmax);
}

void mx_rmax(cudaStream_t st, const float* rleaf, int L, int B, double* rmax) {
    k_mx_rmax<<<B, 1024, 0, st>>>(rleaf, L, rmax);
    ++g_kernel_launches;
}

void mx_root_residual(cudaStream_t st, int m, int B, const double* a, const double* b, const double* r,
                      const double* g64, const double* h64, float* rho) {
    k_mx_root_residual<<<mx_grid((long long)m * B), 256, 0, st>>>(m, B, a, b, r, g64, h64, rho);
    ++g_kernel_launches;
}
void mx_root_rhs(cudaStream_t st, int m, int B, const float* b32, const float* rho, const float* h32, float* rhs) {
    k_mx_root_rhs<<<mx_grid((long long)m * B), 256, 0, st>>>(m, B, b32, rho, h32, rhs);
    ++g_kernel_launches;
}
void mx_perm_identity(cudaStream_t st, int m, const int* perm, double* Z) {
    k_mx_perm_identity<<<mx_grid((long long)m * m), 256, 0, st>>>(m, perm, Z);
    ++g_kernel_launches;
}
void mx_root_update(cudaStream_t st, int m, int B, const float* dg, double* g64) {
    k_mx_root_update<<<mx_grid((long long)m * B), 256, 0, st>>>(m, B, dg, g64);
    ++g_kernel_launches;
}

void mx_root(cudaStream_t st, int m, int B, const double* a, const double* r, double* g) {
    k_mx_root<<<mx_grid((long long)m * B), 256, 0, st>>>(m, B, a, r, g);
    ++g_kernel_launches;
}

}  // namespace efgb
