// Tensor-core (tcgen05) form of the mixed solver's node GEMMs Y[rows][B] = A[rows][K] X[K][B]
// (the FP32 passes' mergeW / mergeH / applyS products, HPSAlgorithm.hpp:1059-1117, :1194-1230).
//
// Precision.  The operators are FP32; each entry a is split once, at set-up, into three bf16 parts
// a = a1 + a2 + a3 (round to nearest at every step: a1 = bf16(a), a2 = bf16(a - a1),
// a3 = bf16(a - a1 - a2); the three 8-bit significands cover FP32's 24 bits, so the sum is exact),
// and the request block X the same way as it is staged.  Every product is formed from the six
// partial products that reach 2^-24 of |a x|:
//     D_hi   += a1 x1                   (TMEM accumulator 1)
//     D_lo_a += a1 x2 + a2 x1 + a3 x1    (TMEM accumulator 2)
//     D_lo_b += a1 x3 + a2 x2            (TMEM accumulator 3)
// with tcgen05.mma kind::f16 (bf16 inputs, exact products, FP32 accumulation); y = D_hi + D_lo_a +
// D_lo_b.  The three X planes lie in shared memory as consecutive rows of one K-major operand
// [x1 | x2 | x3], and the three accumulators as consecutive TMEM columns, so one k-step is three
// MMAs: a1 [x1 x2 x3] (N = 96), a2 [x1 x2] (N = 64, into the two low accumulators) and a3 x1
// (N = 32), each A plane read from shared memory once per k-step (six MMAs of N = 32 read a1 three
// times and a2 twice).  Keeping the small terms in their own accumulators stops them from being
// rounded against the large running sum.  The dropped terms a2 x3, a3 x2, a3 x3 are below
// 2^-24 |a x|.  The tensor core's own FP32 accumulation is not round-to-nearest (a first version
// that accumulated all of K in TMEM made an FP32 pass 2.1x less accurate than CUDA-core FMA
// chains), so every 64-wide K chunk goes to a fresh set of TMEM accumulators and the epilogue warps
// add the chunk's sums to FP32 registers with round-to-nearest: the pass is then at least as
// accurate as the FMA chains, which the one FP64 refinement sweep is sized for (a 3-pass split-TF32
// would round each product to ~2^-21).  The CTA holds all 512 TMEM columns (its shared memory keeps
// it alone on the SM): five sets of 96 columns for one request block per tile, two of 192 for two,
// so the MMAs run that many chunks ahead of the epilogue warps while they store a tile's rows.
//
// Layout.  The three planes of a group's operators (the rows of one kind's operators back to back,
// H with each child's two runs of s rows made adjacent) are stored tiled: each 128-row x 64-column
// block (one 128-byte swizzle row of bf16 per row) is 16 KB of sequential memory already in the
// canonical K-major SWIZZLE_128B order of the MMA operand, so a stage loads each plane with one
// bulk copy (cp.async.bulk) of sequential bytes rather than a tensor-map box of 128 rows K apart.  X is read as FP32 from the pass buffers ([K][B], requests fastest), split, and written
// to shared memory in the same swizzled K-major form by the producer warps.  A tile is 128 rows; a
// tile whose rows use several right-hand-side blocks (nodes of 4s < 128 rows, or the compact H's
// four children) puts the blocks side by side in N (32 requests each) and keeps each row's own
// block in the epilogue.
//
// Roles (256 threads, eight warps: two per SM sub-partition, so up to 255 registers a thread):
// warps 0-3 add each chunk's accumulators to registers and run the epilogue (warp w reads TMEM lanes
// 32w..32w+31; the operands a row's epilogue reads are prefetched when its tile starts; the
// exterior rows of DOWN's children are copied by their own launch, k_mx_ext32), warps 4-6
// stage X (the next chunk's loads in flight while the current one is split and written), warp 7
// allocates TMEM, its lane 0 issues the bulk copies and its lane 1 the MMAs.  Stages
// are handed over through mbarriers; the MMA issuer frees a stage with tcgen05.commit.  Every wait
// gives up after about one second: the kernel then sets the error word, lets its copies and MMAs in
// flight finish (bounded waits), frees its TMEM and returns.
#include <cooperative_groups.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "ef_kernels.cuh"
#include "ef_mixed_common.cuh"

namespace cg = cooperative_groups;

namespace efgb {

namespace {

constexpr int kTM = 128;                  // rows per tile (MMA M)
constexpr int kTK = 64;                   // K per stage: 64 bf16 = one 128-byte swizzle row
constexpr int kTB = 32;                   // requests per right-hand-side block (MMA N per block)
constexpr int kPlaneA = kTM * kTK * 2;    // bytes of one A plane per stage (16 KB)
constexpr int kPlaneX = kTB * kTK * 2;    // bytes of one X plane per block per stage (4 KB)
constexpr int kTcThreads = 256;
constexpr int kStageThreads = 96;  // warps 4-6
constexpr int kMaxSeg = 2;
constexpr int kXRing = 3;  // FP32 request-block chunks in the staging ring

struct TcShape {
    int rows_item, K, seg_rows, nseg;
};

__host__ __device__ inline TcShape tc_shape(int kind, int s) {
    TcShape t;
    if (kind == MX_W) { t.rows_item = 4 * s; t.K = 4 * s; t.seg_rows = 4 * s; }
    else if (kind == MX_H) { t.rows_item = 8 * s; t.K = 2 * s; t.seg_rows = 2 * s; }
    else { t.rows_item = 4 * s; t.K = 8 * s; t.seg_rows = 4 * s; }
    t.nseg = t.seg_rows >= kTM ? 1 : kTM / t.seg_rows;
    return t;
}

__host__ __device__ constexpr int tc_stages(int nseg) { return nseg <= 1 ? 3 : 2; }
__host__ __device__ constexpr int tc_stage_bytes(int nseg) { return 3 * kPlaneA + 3 * nseg * kPlaneX; }
// stages, barriers (256 bytes), then the FP32 staging ring of the request blocks
__host__ __device__ constexpr size_t tc_smem_bytes(int nseg) {
    return 1024 + size_t(tc_stages(nseg)) * tc_stage_bytes(nseg) + 256 + size_t(kXRing) * nseg * kTK * kTB * 4;
}
// two chunk buffers x (D_hi, D_lo) x 32 nseg columns
// accumulator sets of a chunk: D_hi, D_lo_a, D_lo_b of 32 nseg columns each, as many as fit in 512
__host__ __device__ constexpr int tc_acc_sets(int nseg) { return 512 / (3 * kTB * nseg); }
__host__ __device__ constexpr int tc_tmem_cols(int) { return 512; }
// all of TMEM per CTA needs one CTA per SM: the shared memory of two would exceed the SM's 228 KB
static_assert(2 * tc_smem_bytes(1) > 228 * 1024 && 2 * tc_smem_bytes(2) > 228 * 1024, "one CTA per SM");
// the barrier block (256 bytes): 3 per stage, 2 per accumulator set, drain, never, TMEM slot, abort
static_assert((3 * tc_stages(1) + 2 * tc_acc_sets(1) + 2) * 8 + 8 <= 256, "barrier block");
static_assert((3 * tc_stages(2) + 2 * tc_acc_sets(2) + 2) * 8 + 8 <= 256, "barrier block");

// compact H row order of the planes: child c's rows [2s c, 2s c + 2s) are its W/E run and then its
// S/N run; returns the row p of the WESN compact H (the exterior index) of permuted row pr
__host__ __device__ inline int tc_h_unpermute(int pr, int s) {
    const int c = pr / (2 * s), k = pr - c * 2 * s;
    const int run = k >= s ? 1 : 0, o = k - run * s;
    // alpha: W[0,s) S[4s,5s); beta: E[2s,3s) S[5s,6s); gamma: W[s,2s) N[6s,7s); omega: E[3s,4s) N[7s,8s)
    const int base0[4] = {0, 2, 1, 3}, base1[4] = {4, 5, 6, 7};
    return (run ? base1[c] : base0[c]) * s + o;
}

// ---- tcgen05 / TMEM wrappers ---------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(unsigned* dst, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// shared-memory matrix descriptor of a K-major SWIZZLE_128B operand: rows of 128 bytes, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1, swizzle mode 2 (128 bytes)
__device__ __forceinline__ uint64_t tc_desc(unsigned saddr) {
    uint64_t d = uint64_t((saddr & 0x3FFFFu) >> 4);
    d |= uint64_t(1) << 16;            // leading byte offset (unused by swizzled K-major layouts)
    d |= uint64_t(1024 >> 4) << 32;    // stride byte offset
    d |= uint64_t(1) << 46;            // fixed constant 0b001
    d |= uint64_t(2) << 61;            // 128-byte swizzle
    return d;
}
// instruction descriptor of kind::f16: D FP32, A and B bf16, both K-major, M x N
__host__ __device__ constexpr unsigned tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (unsigned(N >> 3) << 17) | (unsigned(M >> 4) << 24);
}
__device__ __forceinline__ void tc_mma(unsigned dtmem, uint64_t a, uint64_t b, unsigned idesc, unsigned acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
// arrive on `bar` once every MMA this thread issued so far has completed
__device__ __forceinline__ void tc_commit(unsigned long long* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(smem_u32(bar))
                 : "memory");
}
// 16 consecutive FP32 columns of the calling warp's 32 TMEM lanes (one lane per thread)
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}
// AND of v over the n threads of named barrier `id` (all of them must call it)
__device__ __forceinline__ bool bar_and(int id, int n, bool v) {
    unsigned r;
    asm volatile(
        "{\n .reg .pred p, q;\n setp.ne.u32 q, %1, 0;\n bar.red.and.pred p, %2, %3, q;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(r)
        : "r"(unsigned(v)), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false after limit_ns (about a second by default, raising the CTA's abort flag) or
// when another role of the CTA has already given up
__device__ __forceinline__ bool tc_wait(unsigned long long* bar, unsigned parity, volatile int* abort,
                                        long long limit_ns = 1000000000LL) {
    long long t0 = 0;
    for (unsigned it = 0;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 31) == 0) {
            if (*abort) return false;
            if (it == 0) t0 = global_ns();
            else if (global_ns() - t0 > limit_ns) {
                *abort = 1;
                return false;
            }
        }
    }
}
// one contiguous block of global memory into shared memory (bulk copy engine), completing on `bar`;
// both addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* bar,
                                          unsigned long long policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
        : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// bf16 parts of x (round to nearest at each step): x = p0 + p1 + p2 for every finite FP32 x
__device__ __forceinline__ void split3(float x, __nv_bfloat16& p0, __nv_bfloat16& p1, __nv_bfloat16& p2) {
    p0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(p0);
    p1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(p1);
    p2 = __float2bfloat16_rn(r2);
}
// the same for a pair (a, b) with packed conversions: planes p0, p1, p2 as (a, b) bf16x2 words
__device__ __forceinline__ void split3x2(float a, float b, unsigned& p0, unsigned& p1, unsigned& p2) {
    const __nv_bfloat162 q0 = __floats2bfloat162_rn(a, b);
    const float ra = a - __low2float(q0), rb = b - __high2float(q0);
    const __nv_bfloat162 q1 = __floats2bfloat162_rn(ra, rb);
    const __nv_bfloat162 q2 = __floats2bfloat162_rn(ra - __low2float(q1), rb - __high2float(q1));
    p0 = *reinterpret_cast<const unsigned*>(&q0);
    p1 = *reinterpret_cast<const unsigned*>(&q1);
    p2 = *reinterpret_cast<const unsigned*>(&q2);
}

// right-hand-side block of segment `gseg` of a group (W, DOWN: one per node; H: one per child)
struct TcSeg {
    const float* X1;  // rows k < kb
    const float* X2;  // rows k >= kb (indexed with the same k)
    int kb;
};
template <int KIND>
__device__ __forceinline__ TcSeg tc_seg(const MixItem* __restrict__ items, int s, int B, int gseg) {
    TcSeg t;
    if (KIND == MX_W) { t.X1 = items[gseg].hd; t.X2 = t.X1; t.kb = 4 * s; }
    else if (KIND == MX_DOWN) { t.X1 = items[gseg].gf; t.X2 = t.X1; t.kb = 8 * s; }
    else {
        const MixItem& it = items[gseg >> 2];
        int Ia, Ib;
        mx_child_ifaces(gseg & 3, Ia, Ib);
        t.X1 = it.w + (long long)Ia * s * B;
        t.X2 = it.w + (long long)(Ib - 1) * s * B;  // row k >= s of [w_Ia; w_Ib] is w_Ib[k - s]
        t.kb = s;
    }
    return t;
}

// Prefetch of the operand a row's epilogue reads (issued when the row's tile starts, so that its
// latency hides behind the K loop): w for DOWN, the child's particular flux hc for H.
template <int KIND>
__device__ __forceinline__ void tc_prefetch_row(const MixItem* __restrict__ items, int s, int B, int b0, int rows_item,
                                                int grow, float (&pre)[32], bool vec) {
    if (KIND == MX_W) return;
    const int item = grow / rows_item, r = grow - item * rows_item;
    const MixItem& it = items[item];
    const int nb = min(32, B - b0);
    const float* src;
    if (KIND == MX_H) {
        int c, q2;
        mx_ext_map(tc_h_unpermute(r, s), s, c, q2);
        src = it.hc[c] + (long long)q2 * B + b0;
    } else {
        src = it.w + (long long)r * B + b0;
    }
    if (vec) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const float4 x = 4 * i < nb ? *reinterpret_cast<const float4*>(src + 4 * i) : make_float4(0.f, 0.f, 0.f, 0.f);
            pre[4 * i] = x.x; pre[4 * i + 1] = x.y; pre[4 * i + 2] = x.z; pre[4 * i + 3] = x.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < 32; ++q) pre[q] = q < nb ? src[q] : 0.f;
    }
}

// Epilogue of one tile row: v[q] = (A X)[row][b0 + q] for the 32 requests of this request block,
// pre[q] the prefetched operand (tc_prefetch_row).  The FP64 interface state of DOWN rows is read
// and written in two halves of 16 requests, each with its loads ahead of its stores; 16-byte
// accesses when B % 4 == 0.
template <int KIND>
__device__ __forceinline__ void tc_store_row(const MixItem* __restrict__ items, int s, int B, int b0, int rows_item,
                                             int grow, const float (&v)[32], const float (&pre)[32], bool vec) {
    const int item = grow / rows_item, r = grow - item * rows_item;
    const MixItem& it = items[item];
    const int nb = min(32, B - b0);
    const long long cb = (long long)b0;
    if (KIND == MX_W) {
        float* dst = it.w + (long long)r * B + cb;
        if (vec) {
#pragma unroll
            for (int q = 0; q < 32; q += 4)
                if (q < nb) *reinterpret_cast<float4*>(dst + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
        } else {
#pragma unroll
            for (int q = 0; q < 32; ++q)
                if (q < nb) dst[q] = v[q];
        }
    } else if (KIND == MX_H) {
        float* dst = it.h + (long long)tc_h_unpermute(r, s) * B + cb;
        if (vec) {
#pragma unroll
            for (int q = 0; q < 32; q += 4)
                if (q < nb)
                    *reinterpret_cast<float4*>(dst + q) =
                        make_float4(v[q] + pre[q], v[q + 1] + pre[q + 1], v[q + 2] + pre[q + 2], v[q + 3] + pre[q + 3]);
        } else {
#pragma unroll
            for (int q = 0; q < 32; ++q)
                if (q < nb) dst[q] = v[q] + pre[q];
        }
    } else {
        const int I = r / s, o = r - (r / s) * s;
        float* d0 = it.gc[mx_lower_child(I)] + (long long)mx_q_lower(I, o, s) * B + cb;
        float* d1 = it.gc[mx_upper_child(I)] + (long long)mx_q_upper(I, o, s) * B + cb;
        // the FP64 state (none: one launch adds the whole pass's values at its end)
        double* ug = it.uG ? it.uG + (long long)r * B + cb : nullptr;
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
            const int q0 = 16 * hf;
            float uu[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) uu[i] = v[q0 + i] + pre[q0 + i];
            if (vec && !ug) {
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (q0 + 4 * i < nb) {
                        const float4 o4 = make_float4(uu[4 * i], uu[4 * i + 1], uu[4 * i + 2], uu[4 * i + 3]);
                        *reinterpret_cast<float4*>(d0 + q0 + 4 * i) = o4;
                        *reinterpret_cast<float4*>(d1 + q0 + 4 * i) = o4;
                    }
            } else if (vec) {
                double2 u2[8];
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    u2[i] = q0 + 2 * i < nb ? *reinterpret_cast<const double2*>(ug + q0 + 2 * i) : make_double2(0.0, 0.0);
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (q0 + 4 * i < nb) {
                        const float4 o4 = make_float4(uu[4 * i], uu[4 * i + 1], uu[4 * i + 2], uu[4 * i + 3]);
                        *reinterpret_cast<float4*>(d0 + q0 + 4 * i) = o4;
                        *reinterpret_cast<float4*>(d1 + q0 + 4 * i) = o4;
                    }
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    if (q0 + 2 * i < nb)
                        *reinterpret_cast<double2*>(ug + q0 + 2 * i) =
                            make_double2(u2[i].x + f2d_bits(uu[2 * i]), u2[i].y + f2d_bits(uu[2 * i + 1]));
            } else {
                double uv[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) uv[i] = (ug && q0 + i < nb) ? ug[q0 + i] : 0.0;
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    if (q0 + i < nb) {
                        d0[q0 + i] = uu[i];
                        d1[q0 + i] = uu[i];
                        if (ug) ug[q0 + i] = uv[i] + f2d_bits(uu[i]);
                    }
            }
        }
    }
}

template <int KIND, int NSEG>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_mx_umma(const __nv_bfloat16* __restrict__ A3, const MixItem* __restrict__ items, int s, int B, int cnt,
              int ksplit, int ntiles, int* __restrict__ err) {
    const TcShape sh = tc_shape(KIND, s);  // sh.nseg == NSEG (checked by the launcher)
    const int K = sh.K, R = cnt * sh.rows_item;
    const int nsegs_total = KIND == MX_H ? 4 * cnt : cnt;
    constexpr int NS = tc_stages(NSEG), SB = tc_stage_bytes(NSEG);
    constexpr int ncol = kTB * NSEG, tcols = tc_tmem_cols(NSEG);
    constexpr int NP = tc_acc_sets(NSEG);
    constexpr unsigned idesc1 = tc_idesc(kTM, ncol), idesc2 = tc_idesc(kTM, 2 * ncol), idesc3 = tc_idesc(kTM, 3 * ncol);
    extern __shared__ unsigned char tc_smem[];
    unsigned char* base = tc_smem + ((1024u - (smem_u32(tc_smem) & 1023u)) & 1023u);
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(base + size_t(NS) * SB);
    unsigned long long* a_full = bars;             // [NS] bulk-copy transaction barriers
    unsigned long long* x_full = bars + NS;        // [NS] 128 staging arrivals
    unsigned long long* empty = bars + 2 * NS;     // [NS] MMA commit
    unsigned long long* acc_full = bars + 3 * NS;   // [NP] MMA commit at the end of a chunk
    unsigned long long* acc_empty = acc_full + NP;  // [NP] 128 epilogue arrivals
    unsigned long long* drain = acc_full + 2 * NP;  // MMA commit before TMEM is freed
    unsigned long long* never = drain + 1;          // nothing arrives on it (failure-path test)
    unsigned* tmem_slot = reinterpret_cast<unsigned*>(drain + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nkc = (K + kTK - 1) / kTK;
    int first_tile, tile_step, nunits, cpu, cbase;
    if (ksplit > 1) {
        const int kp = blockIdx.x % ksplit, cpp = (nkc + ksplit - 1) / ksplit;
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
    if (cpu <= 0) nunits = 0;
    const int total = nunits * cpu;
    const int b0 = blockIdx.y * kTB;
    const bool vec = (B & 3) == 0;

    if (tid == 0) {
        for (int i = 0; i < NS; ++i) {
            mbar_init(&a_full[i], 1);
            mbar_init(&x_full[i], kStageThreads);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < NP; ++i) {
            mbar_init(&acc_full[i], 1);
            mbar_init(&acc_empty[i], 128);
        }
        mbar_init(drain, 1);
        mbar_init(never, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    if (warp == 7) {
        tmem_alloc(tmem_slot, unsigned(tcols));
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = *tmem_slot;

    // per unit: the tile's rows [128 t, 128 t + 128) of the group and its first segment
    auto tile_of = [&](int u) { return first_tile + u * tile_step; };
    auto seg0_of = [&](int tl) { return sh.seg_rows >= kTM ? (tl * kTM) / sh.seg_rows : tl * NSEG; };

    // epilogue state that the K-split reduction below still needs: the row's running sums (v holds
    // the row's result at a unit's end) and its prefetched epilogue operand (w for DOWN, hc for H)
    float v[32];
    float pre[32];
    bool ep_ok = true;

    if (warp == 7) {
        // ---- lane 0: producer of the three A planes of every stage (bulk copies) ----
        if (lane == 0) {
            int st = 0;
            unsigned ph = 0;
            int issued = 0;
            bool ok = true;
            const long long pstride = (long long)ntiles * nkc * (kTM * kTK);  // elements per plane
            const unsigned long long pol = l2_evict_first();
            for (int u = 0; u < nunits && ok; ++u) {
                const long long blk0 = (long long)tile_of(u) * nkc + cbase;
                for (int c = 0; c < cpu && ok; ++c) {
                    if (issued >= NS) ok = tc_wait(&empty[st], ph ^ 1u, abort_flag);
                    if (!ok) break;
                    unsigned char* sa = base + size_t(st) * SB;
                    mbar_expect_tx(&a_full[st], 3u * kPlaneA);
                    const __nv_bfloat16* src = A3 + (blk0 + c) * (kTM * kTK);
                    for (int p = 0; p < 3; ++p)
                        bulk_load(sa + p * kPlaneA, src + p * pstride, kPlaneA, &a_full[st], pol);
                    ++issued;
                    if (++st == NS) { st = 0; ph ^= 1u; }
                }
            }
            if (!ok) {
                // let the loads still in flight land before the shared memory goes away
                // (only the last NS loads can be pending: a stage is reloaded after its MMAs completed)
                int s2 = 0;
                unsigned p2 = 0;
                volatile int never_set = 0;
                const int first = issued > NS ? issued - NS : 0;
                for (int q = 0; q < issued; ++q) {
                    if (q >= first) (void)tc_wait(&a_full[s2], p2, &never_set);
                    if (++s2 == NS) { s2 = 0; p2 ^= 1u; }
                }
                atomicExch(err, 1);
            }
        }
        // ---- lane 1: MMA issuer (independent thread scheduling lets the two lanes wait apart) ----
        if (lane == 1) {
            int st = 0;
            unsigned ph = 0;
            bool ok = true;
            const uint32_t a_base = smem_u32(base);
            if (g_mx_inject_timeout && nunits > 0) ok = tc_wait(never, 0u, abort_flag, 1000000LL);
            for (int gch = 0; gch < total && ok; ++gch) {
                const int c = gch % cpu, bf = gch % NP;
                // the chunk's accumulator set was drained NP chunks ago
                if (gch >= NP) ok = tc_wait(&acc_empty[bf], unsigned(gch / NP - 1) & 1u, abort_flag);
                if (ok) ok = tc_wait(&a_full[st], ph, abort_flag) && tc_wait(&x_full[st], ph, abort_flag);
                if (!ok) break;
                tc_fence_after();
                const uint32_t sa = a_base + uint32_t(st) * SB;
                const uint32_t sx = sa + 3u * kPlaneA;
                const unsigned dhi = tmem + unsigned(bf * 3 * ncol), dlo = dhi + unsigned(ncol);
                const int kleft = K - (cbase + c) * kTK;
                const int nk = kleft >= kTK ? kTK / 16 : (kleft + 15) / 16;
                for (int kk = 0; kk < nk; ++kk) {
                    const uint32_t ko = uint32_t(kk) * 32u;
                    const uint64_t a1 = tc_desc(sa + ko), a2 = tc_desc(sa + kPlaneA + ko),
                                   a3 = tc_desc(sa + 2 * kPlaneA + ko);
                    // the three X planes are consecutive rows of one K-major operand: [x1 | x2 | x3]
                    const uint64_t x123 = tc_desc(sx + ko);
                    const unsigned acc = kk > 0 ? 1u : 0u;  // a fresh accumulator set per chunk
                    tc_mma(dhi, a1, x123, idesc3, acc);  // D_hi = a1 x1, D_lo_a = a1 x2, D_lo_b = a1 x3
                    tc_mma(dlo, a2, x123, idesc2, 1u);   // D_lo_a += a2 x1, D_lo_b += a2 x2
                    tc_mma(dlo, a3, x123, idesc1, 1u);   // D_lo_a += a3 x1
                }
                tc_commit(&empty[st]);
                tc_commit(&acc_full[bf]);
                if (++st == NS) { st = 0; ph ^= 1u; }
            }
            // every MMA issued has completed before TMEM is freed
            tc_commit(drain);
            volatile int never_set = 0;
            if (!tc_wait(drain, 0u, &never_set)) atomicExch(err, 1);
            if (!ok) atomicExch(err, 1);
        }
    } else if (warp >= 4) {
        // ---- warps 4-6: stage X.  FP32 request rows travel by cp.async into a ring of kXRing
        //      chunks (kXRing - 1 chunks ahead of the one being split, so no global-load latency sits
        //      on a chunk's path), then are split into bf16 planes in the swizzled K-major layout ----
        const int t = tid - 128;  // 0 .. kStageThreads-1
        float* ring = reinterpret_cast<float*>(base + size_t(NS) * SB + 256);
        constexpr int RC = NSEG * kTK * kTB;  // floats of one ring chunk: [seg][k][request]
        int st = 0;
        unsigned ph = 0;
        int staged = 0;
        bool ok = true;
        TcSeg seg[NSEG];
        bool sval[NSEG];
        int seg_unit = -1;
        auto issue = [&](int g) {
            if (g < total) {
                const int u = g / cpu, c = g - u * cpu;
                if (u != seg_unit) {
                    seg_unit = u;
                    const int gs0 = seg0_of(tile_of(u));
#pragma unroll
                    for (int j = 0; j < NSEG; ++j) {
                        sval[j] = gs0 + j < nsegs_total;
                        seg[j] = sval[j] ? tc_seg<KIND>(items, s, B, gs0 + j) : TcSeg{nullptr, nullptr, 0};
                    }
                }
                const int k0 = (cbase + c) * kTK;
                float* dst = ring + (g % kXRing) * RC;
                if (vec) {
                    // 16-byte pieces: 8 per row of 32 requests (B % 4 == 0: a piece is all in or all out)
#pragma unroll
                    for (int j = 0; j < NSEG; ++j)
                        for (int e = t; e < kTK * 8; e += kStageThreads) {
                            const int k = k0 + (e >> 3), p4 = (e & 7) * 4;
                            const bool in = sval[j] && k < K && b0 + p4 < B;
                            const float* src = in ? (k < seg[j].kb ? seg[j].X1 : seg[j].X2) + (long long)k * B + b0 + p4
                                                  : reinterpret_cast<const float*>(items);
                            cp_async16(dst + (j * kTK + (e >> 3)) * kTB + p4, src, in ? 16 : 0);
                        }
                } else {
#pragma unroll
                    for (int j = 0; j < NSEG; ++j)
                        for (int e = t; e < kTK * kTB; e += kStageThreads) {
                            const int k = k0 + (e >> 5), q = e & 31;
                            const bool in = sval[j] && k < K && b0 + q < B;
                            const float* src = in ? (k < seg[j].kb ? seg[j].X1 : seg[j].X2) + (long long)k * B + b0 + q
                                                  : reinterpret_cast<const float*>(items);
                            cp_async4(dst + (j * kTK + (e >> 5)) * kTB + q, src, in ? 4 : 0);
                        }
                }
            }
            cp_async_commit();  // one group per chunk (empty past the end) keeps the counting simple
        };
        for (int g = 0; g < kXRing - 1; ++g) issue(g);
        for (int g = 0; g < total && ok; ++g) {
            cp_async_wait<kXRing - 2>();                               // this thread's copies of chunk g
            asm volatile("bar.sync 1, %0;\n" ::"n"(kStageThreads) : "memory");  // everyone's
            issue(g + kXRing - 1);  // into the slot of chunk g - 1, which every thread has split
            // the stage must be free; the staging threads leave together if any of them gives up (a
            // thread left alone at the named barrier would wait forever)
            const bool free_stage = staged < NS || tc_wait(&empty[st], ph ^ 1u, abort_flag);
            if (!(ok = bar_and(2, kStageThreads, free_stage))) break;
            const float* src = ring + (g % kXRing) * RC;
            unsigned char* sx = base + size_t(st) * SB + 3 * kPlaneA;
            constexpr unsigned xp = unsigned(NSEG) * kPlaneX;
            // one 16-byte swizzle chunk (8 consecutive k) of one request per item and plane:
            // NSEG x 8 chunks x 32 requests, the ring read by consecutive requests
            for (int e = t; e < NSEG * 8 * kTB; e += kStageThreads) {
                const int n = e & 31, kg = (e >> 5) & 7, j = e >> 8;
                const float* x = src + (j * kTK + 8 * kg) * kTB + n;
                uint4 c0, c1, c2;
                split3x2(x[0], x[kTB], c0.x, c1.x, c2.x);
                split3x2(x[2 * kTB], x[3 * kTB], c0.y, c1.y, c2.y);
                split3x2(x[4 * kTB], x[5 * kTB], c0.z, c1.z, c2.z);
                split3x2(x[6 * kTB], x[7 * kTB], c0.w, c1.w, c2.w);
                const unsigned off = unsigned(j) * kPlaneX + unsigned(n) * 128u + ((unsigned(kg) ^ unsigned(n & 7)) << 4);
                *reinterpret_cast<uint4*>(sx + off) = c0;
                *reinterpret_cast<uint4*>(sx + xp + off) = c1;
                *reinterpret_cast<uint4*>(sx + 2 * xp + off) = c2;
            }
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            mbar_arrive(&x_full[st]);
            ++staged;
            if (++st == NS) { st = 0; ph ^= 1u; }
        }
        cp_async_wait<0>();  // nothing of this thread's may land after the shared memory is gone
        if (!ok) atomicExch(err, 1);
    } else {
        // ---- warps 0-3: add every chunk's accumulators to FP32 running sums (round to nearest),
        //      run the epilogue of each unit with its operands prefetched at the unit's start ----
        const int t = tid;  // 0..127 = TMEM lane of this thread's tile row
        float rlo[32];
#pragma unroll
        for (int q = 0; q < 32; ++q) { v[q] = 0.f; rlo[q] = 0.f; pre[q] = 0.f; }
        const int jrow = sh.seg_rows >= kTM ? 0 : t / sh.seg_rows;
        const unsigned lane_off = unsigned(warp * 32) << 16;
        for (int gch = 0; gch < total; ++gch) {
            const int u = gch / cpu;
            if (gch - u * cpu == 0) {
                const int grow = tile_of(u) * kTM + t;
                if (grow < R) tc_prefetch_row<KIND>(items, s, B, b0, sh.rows_item, grow, pre, vec);
            }
            const int bf = gch % NP;
            if (!(ep_ok = tc_wait(&acc_full[bf], unsigned(gch / NP) & 1u, abort_flag))) break;
            tc_fence_after();
            const unsigned col = unsigned(bf * 3 * ncol + jrow * kTB);
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
                float hi[16], la[16], lb[16];
                tmem_ld16(tmem + lane_off + col + unsigned(16 * hf), hi);
                tmem_ld16(tmem + lane_off + col + unsigned(ncol + 16 * hf), la);
                tmem_ld16(tmem + lane_off + col + unsigned(2 * ncol + 16 * hf), lb);
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    v[16 * hf + q] += hi[q];
                    rlo[16 * hf + q] += la[q];
                    rlo[16 * hf + q] += lb[q];
                }
            }
            tc_fence_before();
            mbar_arrive(&acc_empty[bf]);
            if ((gch + 1) % cpu != 0) continue;
            // ---- epilogue of the unit ----
            const int tile = tile_of(u);
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                v[q] += rlo[q];
                rlo[q] = 0.f;
            }
            if (ksplit > 1) {
                // partial tiles -> rank 0 of the cluster through distributed shared memory, in rank
                // order (deterministic); the stage memory is free once every MMA has completed
                float* red = reinterpret_cast<float*>(base);
#pragma unroll
                for (int q = 0; q < 32; q += 4)
                    *reinterpret_cast<float4*>(red + t * 32 + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                break;  // the cluster reduction and the epilogue follow below
            }
            const int grow = tile * kTM + t;
            if (grow < R) tc_store_row<KIND>(items, s, B, b0, sh.rows_item, grow, v, pre, vec);
#pragma unroll
            for (int q = 0; q < 32; ++q) v[q] = 0.f;
        }
        if (!ep_ok) atomicExch(err, 1);
    }

    // ---- K split: rank 0 of the cluster adds the partial tiles and runs the epilogue ----
    if (ksplit > 1) {
        cg::cluster_group cluster = cg::this_cluster();
        if (nunits == 0 && tid < 128) {
            // a rank without K chunks adds zeros
            float* red = reinterpret_cast<float*>(base);
#pragma unroll
            for (int q = 0; q < 32; q += 4) *reinterpret_cast<float4*>(red + tid * 32 + q) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        cluster.sync();
        if (cluster.block_rank() == 0 && tid < 128 && nunits > 0 && !*abort_flag) {
            const int t = tid;
            float* red = reinterpret_cast<float*>(base);
#pragma unroll
            for (int q = 0; q < 32; ++q) v[q] = red[t * 32 + q];
            for (int rk = 1; rk < ksplit; ++rk) {
                const float* rr = cluster.map_shared_rank(red, rk);
#pragma unroll
                for (int q = 0; q < 32; ++q) v[q] += rr[t * 32 + q];
            }
            const int tile = first_tile;
            const int grow = tile * kTM + t;
            if (grow < R) tc_store_row<KIND>(items, s, B, b0, sh.rows_item, grow, v, pre, vec);
        }
        cluster.sync();
    }

    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 7) tmem_dealloc(tmem, unsigned(tcols));
}

// A planes of one group: three bf16 planes with src[R][K] = plane 0 + plane 1 + plane 2, each stored
// tiled: the block of row tile t (128 rows) and K chunk c (64 columns) is 16 KB of sequential memory
// at element ((p * ntiles + t) * nkc + c) * 8192 of the group's planes, in the order of its shared-
// memory image (row r at 64 r, its 8-element groups g at 8 (g ^ (r & 7)): the 128-byte swizzle that
// the MMA's shared-memory descriptors read), so that a pipeline stage loads each plane's tile with
// one bulk copy of sequential bytes instead of 128 row pieces K columns apart.  Rows past R and
// columns past K of the last tile and chunk stay as the caller zeroed them.  H rows in the
// child-major order of tc_h_unpermute.
__global__ void k_tc_split(const float* __restrict__ src, __nv_bfloat16* __restrict__ dst, long long R, int K,
                           int s, int permute_h) {
    const long long tot = R * K;
    const int nkc = (K + kTK - 1) / kTK;
    const long long pstride = (R + kTM - 1) / kTM * nkc * (kTM * kTK);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot;
         e += (long long)gridDim.x * blockDim.x) {
        const long long row = e / K;
        const int k = int(e - row * K);
        long long srow = row;
        if (permute_h) {
            const long long node = row / (8 * s);
            const int pr = int(row - node * 8 * s);
            srow = node * 8 * s + tc_h_unpermute(pr, s);
        }
        const long long tile = row / kTM;
        const int r = int(row - tile * kTM), c = k / kTK, kk = k - c * kTK;
        const long long off = (tile * nkc + c) * (kTM * kTK) + r * kTK + (((kk >> 3) ^ (r & 7)) << 3) + (kk & 7);
        __nv_bfloat16 p0, p1, p2;
        split3(src[srow * K + k], p0, p1, p2);
        dst[off] = p0;
        dst[pstride + off] = p1;
        dst[2 * pstride + off] = p2;
    }
}

template <int KIND, int NSEG>
void launch_umma_n(cudaStream_t st, const void* A3, const MixItem* items, int cnt, int s, int B, int* err,
                   int ksplit) {
    const TcShape sh = tc_shape(KIND, s);
    const long long R = (long long)cnt * sh.rows_item;
    const int ntiles = int((R + kTM - 1) / kTM);
    const int chunks = (B + kTB - 1) / kTB;
    const size_t smem = tc_smem_bytes(NSEG);
    cudaFuncSetAttribute(k_mx_umma<KIND, NSEG>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned gx;
    if (ksplit > 1) gx = unsigned(ntiles * ksplit);
    else gx = unsigned(std::max(1, std::min(ntiles, std::max(1, sms / chunks))));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(gx, unsigned(chunks));
    cfg.blockDim = dim3(kTcThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = unsigned(ksplit);
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = ksplit > 1 ? 1 : 0;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, k_mx_umma<KIND, NSEG>, reinterpret_cast<const __nv_bfloat16*>(A3),
                                             items, s, B, cnt, ksplit, ntiles, err);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        throw std::runtime_error(std::string("tensor-core node GEMM launch (K split ") + std::to_string(ksplit) +
                                 "): " + cudaGetErrorString(e));
    }
    ++g_kernel_launches;
}

template <int KIND>
void launch_umma(cudaStream_t st, const void* A3, const MixItem* items, int cnt, int s, int B, int* err,
                 int ksplit) {
    const int nseg = tc_shape(KIND, s).nseg;
    if (nseg == 1) launch_umma_n<KIND, 1>(st, A3, items, cnt, s, B, err, ksplit);
    else launch_umma_n<KIND, 2>(st, A3, items, cnt, s, B, err, ksplit);
}

}  // namespace

bool mx_tc_supported(int kind, int s) {
    // s a power of two >= 16: K a multiple of 16, each right-hand-side block a power-of-two number
    // of rows of at least 64, at most two blocks per tile (the compact H of s = 16 stays on the
    // CUDA-core kernel)
    if (s < 16 || (s & (s - 1)) != 0) return false;
    const TcShape sh = tc_shape(kind, s);
    return sh.nseg <= kMaxSeg && sh.K % 16 == 0;
}

int mx_tc_max_split(int kind, int s) {
    const TcShape sh = tc_shape(kind, s);
    const int nkc = (sh.K + kTK - 1) / kTK;
    int k = 1;
    while (k < 8 && nkc / (2 * k) >= 2) k *= 2;
    return k;
}

long long mx_tc_plane_elems(long long R, int K) {
    return 3 * ((R + kTM - 1) / kTM) * ((K + kTK - 1) / kTK) * (kTM * kTK);
}

void mx_tc_split(cudaStream_t st, int kind, const float* src, void* dst, long long R, int K, int s) {
    const long long tot = R * K;
    const int grid = int(std::min<long long>((tot + 255) / 256, 8192));
    k_tc_split<<<grid, 256, 0, st>>>(src, reinterpret_cast<__nv_bfloat16*>(dst), R, K, s, kind == MX_H ? 1 : 0);
    ++g_kernel_launches;
}

void mx_tc_set_inject_timeout(int on) {
    if (cudaMemcpyToSymbol(g_mx_inject_timeout, &on, sizeof(int)) != cudaSuccess)
        throw std::runtime_error("tensor-core GEMM: setting the failure-path test switch failed");
}

void mx_gemm_tc(cudaStream_t st, int kind, const void* planes, const MixItem* items, int nitems, int s, int B,
                int* err, int ksplit) {
    if (!mx_tc_supported(kind, s)) throw std::invalid_argument("tensor-core node GEMM: unsupported interface size");
    if (ksplit < 1) ksplit = 1;
    if (kind == MX_W) launch_umma<MX_W>(st, planes, items, nitems, s, B, err, ksplit);
    else if (kind == MX_H) launch_umma<MX_H>(st, planes, items, nitems, s, B, err, ksplit);
    else launch_umma<MX_DOWN>(st, planes, items, nitems, s, B, err, ksplit);
}

}  // namespace efgb
