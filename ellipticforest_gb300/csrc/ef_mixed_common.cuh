// Device helpers shared by the mixed-precision kernels (ef_mixed.cu, ef_mixed_tc.cu): the merge
// index maps, float <-> double conversions off the FP64 pipe, shared-memory addresses, cp.async,
// bounded mbarrier waits and 2-D TMA tile loads.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace efgb {
namespace {

__device__ __forceinline__ void mx_child_ifaces(int c, int& Ia, int& Ib) {
    Ia = (c == 0 || c == 2) ? 0 : 1;
    Ib = (c < 2) ? 2 : 3;
}

// float <-> double by integer bit manipulation.  GB300's FP64 pipe, which also converts between the
// two widths, runs at a small fraction of its FP32 and integer rates; these stay off it.  Values
// below the smallest normal number of the target type become signed zeros; d2f_rn_bits rounds to
// nearest (ties to even): a one-signed rounding of every residual entry would bias the correction
// it drives.
// the high and low 32-bit words of the double of x, for stores that need no FP64 register
__device__ __forceinline__ void f2d_words(float x, unsigned& hi, unsigned& lo) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    const unsigned sign = b & 0x80000000u;
    const unsigned e11 = e == 0xffu ? 0x7ffu : e + 896u;
    hi = e == 0 ? sign : (sign | (e11 << 20) | ((b & 0x7fffffu) >> 3));
    lo = e == 0 ? 0u : (b << 29);
}
__device__ __forceinline__ double f2d_bits(float x) {
    // assembled as two 32-bit words (a 64-bit assembly of the same bits measured 7 % slower in the
    // 16 x 16 leaf solve, whose FP64 state stores take 16 of these per thread)
    unsigned hi, lo;
    f2d_words(x, hi, lo);
    return __hiloint2double(int(hi), int(lo));
}
__device__ __forceinline__ float d2f_rn_bits(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hi = unsigned(b >> 32), lo = unsigned(b);
    const unsigned sign = hi & 0x80000000u;
    const int e = int(hi >> 20) & 0x7ff;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (m ? 0x400000u : 0u));
    const int e32 = e - 896;
    if (e32 <= 0) return __uint_as_float(sign);
    if (e32 >= 255) return __uint_as_float(sign | 0x7f800000u);
    const unsigned rest = lo & 0x1fffffffu;
    // a carry out of the significand steps the exponent (up to the infinity pattern)
    const unsigned up = (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | ((unsigned(e32) << 23) + m + up));
}

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, int nbytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(nbytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int nbytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(nbytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
__device__ __forceinline__ long long global_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// bounded wait on an mbarrier phase: false after limit_ns without completion
__device__ __forceinline__ bool mbar_wait_ns(unsigned long long* bar, unsigned parity, long long limit_ns) {
    const unsigned a = smem_u32(bar);
    long long t0 = 0;
    for (unsigned it = 0;; ++it) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (it == 0) t0 = global_ns();
        else if ((it & 63) == 0 && global_ns() - t0 > limit_ns) return false;
    }
}
// bounded wait on an mbarrier phase: false after about a second without completion
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
    return mbar_wait_ns(bar, parity, 1000000000LL);
}

// Failure-path test switch of the node GEMMs (set from the host, per translation unit): when set, the
// first consumer wait of every CTA is on an mbarrier that nothing arrives on, limited to 1 ms, and
// the kernel then leaves through the same path as after a real timeout (copies in flight drained,
// error word set).  Off in normal operation.
static __device__ int g_mx_inject_timeout = 0;

// L2 policy for operator streams: each operator byte is read once per pass, so its lines go first
// and the right-hand sides that several tiles of a node share stay in L2
__device__ __forceinline__ unsigned long long l2_evict_first() {
    unsigned long long p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}

// one TMA tile (32 columns x rows) of A into shared memory, completing on `bar`, with L2 policy `pol`
__device__ __forceinline__ void tma_load_tile(const CUtensorMap* tm, unsigned long long* bar, float* dst, int x,
                                              int y, unsigned bytes, unsigned long long pol) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, %3}], "
        "[%4], %5;\n" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(pol)
        : "memory");
}

enum : int { MX_W = 0, MX_H = 1, MX_DOWN = 2 };

template <int KIND>
__host__ __device__ __forceinline__ void mx_shape(int s, int& rows_item, int& K) {
    if (KIND == MX_W) { rows_item = 4 * s; K = 4 * s; }
    else if (KIND == MX_H) { rows_item = 8 * s; K = 2 * s; }
    else { rows_item = 4 * s; K = 8 * s; }
}


}  // namespace
}  // namespace efgb
