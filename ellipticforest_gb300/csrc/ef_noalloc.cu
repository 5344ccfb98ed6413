// Single-patch solve that allocates nothing (ef_fv_solve_noalloc).
//
// Some callers cannot call cudaMalloc: plugins inside a host framework that owns all device memory
// through its own pool and forbids raw allocations, and real-time loops that must not allocate
// after start-up.  For them this entry point keeps its scratch -- the patch's sine basis, its
// inverse eigenvalue table and the one-item launch descriptors -- in a file-scope device array of
// fixed size instead of allocating it per call like ef_fv_solve does.  The caller passes device
// pointers for the inputs and the output.
//
// The array is sized for patches of at most kNoAllocMaxN = 64 cells per side (about 66 KB) and
// every GPU that loads this library holds it until the process exits.  All calls share it: each
// call overwrites every entry it reads before use, so nothing needs clearing between calls, but two
// calls whose work overlaps on the GPU (different streams, or other threads) race on it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/ellipticforest_gb300.h"
#include "ef_kernels.cuh"

namespace efgb {
void set_last_error_message(const std::string& msg);
}

namespace {

constexpr int kNoAllocMaxN = 64;
constexpr int kTableDoubles = 2 * kNoAllocMaxN * kNoAllocMaxN;  // V and Dinv
constexpr int kTypeOffset = kTableDoubles;                       // one LeafType (5 doubles wide)
constexpr int kItemOffset = kTableDoubles + 8;                   // one LeafItem (4 doubles wide)
constexpr int kScratchDoubles = kTableDoubles + 16;

static_assert(sizeof(efgb::LeafType) <= 8 * sizeof(double), "LeafType slot too small");
static_assert(sizeof(efgb::LeafItem) <= 8 * sizeof(double), "LeafItem slot too small");

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// Fills the sine basis, the inverse eigenvalue table and the launch descriptors of one patch
// (the same tables leaf_tables() computes on the host for the allocating entry points).
__global__ void k_noalloc_tables(int n, double dx, double dy, double lambda, const double* g,
                                 const double* f, double* u, double* scratch) {
    double* V = scratch;
    double* D = scratch + n * n;
    const double pi = 3.141592653589793238462643383279502884;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int a = e / n, b = e - (e / n) * n;
        const double c = (b == n - 1) ? sqrt(1.0 / n) : sqrt(2.0 / n);
        V[e] = c * sin(pi * (b + 1) * (a + 0.5) / n);
        const double sx = sin(pi * (a + 1) / (2.0 * n));
        const double sy = sin(pi * (b + 1) / (2.0 * n));
        D[e] = 1.0 / (-(4.0 / (dx * dx)) * sx * sx - (4.0 / (dy * dy)) * sy * sy + lambda);
    }
    if (threadIdx.x == 0) {
        auto* ty = reinterpret_cast<efgb::LeafType*>(scratch + kTypeOffset);
        auto* it = reinterpret_cast<efgb::LeafItem*>(scratch + kItemOffset);
        *ty = efgb::LeafType{n, dx, dy, V, D};
        *it = efgb::LeafItem{0, 0, f, g, u};
    }
}

std::mutex g_symbol_mutex;
double* g_symbol_addr[64] = {nullptr};
unsigned long long g_symbol_ctx[64] = {0};  // context id the cached address belongs to

// Id of the calling thread's current context (cuCtxGetId through the runtime's driver entry point, no
// link against libcuda); 0 when unavailable.  A cudaDeviceReset by the caller makes a new primary
// context whose id differs, so the cached address is looked up again.
unsigned long long current_ctx_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        void* p = nullptr;
        void* q = nullptr;
        cudaDriverEntryPointQueryResult r1{}, r2{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &r1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2) != cudaSuccess ||
            r1 != cudaDriverEntryPointSuccess || r2 != cudaDriverEntryPointSuccess || !p || !q)
            return 0;
        get_current = reinterpret_cast<GetCurrent>(p);
        get_id = reinterpret_cast<GetId>(q);
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

}  // namespace

extern "C" int ef_fv_solve_noalloc(int solver_type, int n, double x_lower, double x_upper,
                                   double y_lower, double y_upper, double lambda,
                                   const double* g_dev, const double* f_dev, double* u_dev,
                                   void* cuda_stream) {
    if (solver_type != EF_SOLVER_FISHPACK90) {
        efgb::set_last_error_message("ef_fv_solve_noalloc implements the FISHPACK90 solver type");
        return EF_ERR_UNSUPPORTED;
    }
    if (n < 2 || n > kNoAllocMaxN) {
        efgb::set_last_error_message("ef_fv_solve_noalloc: n must be in [2, 64] (size of its fixed scratch)");
        return EF_ERR_INVALID;
    }
    if (!(x_upper > x_lower) || !(y_upper > y_lower)) {
        efgb::set_last_error_message("ef_fv_solve_noalloc: bad patch box");
        return EF_ERR_INVALID;
    }
    if (!g_dev || !u_dev) {
        efgb::set_last_error_message("ef_fv_solve_noalloc: null device pointer");
        return EF_ERR_INVALID;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        efgb::set_last_error_message(std::string("ef_fv_solve_noalloc: cudaGetDevice: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    double* scratch;
    {
        // once per device (and again after a context reset), with that device current: host code
        // needs the device address of the array (its host-side name is only a stand-in)
        std::lock_guard<std::mutex> lock(g_symbol_mutex);
        const unsigned long long ctx = current_ctx_id();
        if (!g_symbol_addr[dev] || ctx == 0 || ctx != g_symbol_ctx[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                efgb::set_last_error_message(std::string("ef_fv_solve_noalloc: cudaGetSymbolAddress: ") +
                                             cudaGetErrorString(e));
                return EF_ERR_CUDA;
            }
            g_symbol_addr[dev] = static_cast<double*>(p);
            // the look-up itself creates the primary context if there was none yet
            g_symbol_ctx[dev] = ctx != 0 ? ctx : current_ctx_id();
        }
        scratch = g_symbol_addr[dev];
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(cuda_stream);
    const double dx = (x_upper - x_lower) / n, dy = (y_upper - y_lower) / n;
    k_noalloc_tables<<<1, 256, 0, st>>>(n, dx, dy, lambda, g_dev, f_dev, u_dev, scratch);
    ++efgb::g_kernel_launches;
    // the table-reading kernel for every n: the 16 x 16 fast kernel reads a constant-memory basis
    // that only the allocating entry points upload
    efgb::leaf_eigen_tables(st, efgb::LEAF_SOLVE, reinterpret_cast<const efgb::LeafType*>(scratch + kTypeOffset),
                     reinterpret_cast<const efgb::LeafItem*>(scratch + kItemOffset), 1, n);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        efgb::set_last_error_message(std::string("ef_fv_solve_noalloc: launch: ") + cudaGetErrorString(e));
        return EF_ERR_CUDA;
    }
    return EF_OK;
}
