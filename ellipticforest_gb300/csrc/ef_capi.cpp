// C ABI of the GB300 HPS solver (include/ellipticforest_gb300.h).
//
// Thin layer over efgb::Mesh and efgb::Hps: argument checks, exception-to-status conversion and
// host<->device copies.  No computation happens on the host here; every numerical step runs in
// the CUDA kernels of this library.
#include <cuda_runtime.h>

#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ellipticforest_gb300.h"
#include "ef_hps.hpp"
#include "ef_kernels.cuh"
#include "ef_mesh.hpp"
#include "ef_server.hpp"

struct ef_mesh {
    efgb::Mesh mesh;
};

struct ef_server {
    std::unique_ptr<efgb::Server> srv;
};

struct ef_hps {
    std::unique_ptr<efgb::Hps> hps;
    std::unique_ptr<efgb::MixedSolver> mixed;
    // further lanes 1.. (share mixed's FP32 operators), each with its own stream
    static constexpr int kMaxLanes = 4;
    std::unique_ptr<efgb::MixedSolver> lanes[kMaxLanes];
    cudaStream_t lane_st[kMaxLanes] = {};
    void drop_lanes() {
        for (int k = 1; k < kMaxLanes; ++k) {
            if (lane_st[k]) cudaStreamSynchronize(lane_st[k]);
            lanes[k].reset();
        }
    }
    ~ef_hps() {
        drop_lanes();
        for (int k = 1; k < kMaxLanes; ++k)
            if (lane_st[k]) cudaStreamDestroy(lane_st[k]);
    }
    bool cache_operators = false;
    bool homogeneous_rhs = false;
    bool upward_done = false;
    // root operator of the block solvers (ef_hps_mixed_set_root), applied to lanes created later
    std::vector<double> root_a, root_b;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

template <class F>
int guarded(F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc& e) {
        return fail(EF_ERR_NOMEM, std::string("allocation failed: ") + e.what());
    } catch (const std::invalid_argument& e) {
        return fail(EF_ERR_INVALID, e.what());
    } catch (const std::runtime_error& e) {
        const std::string m = e.what();
        if (m.find("out of memory") != std::string::npos) return fail(EF_ERR_NOMEM, m);
        return fail(EF_ERR_CUDA, m);
    } catch (...) {
        return fail(EF_ERR_INVALID, "unknown exception");
    }
}

int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return EF_OK;
    if (e == cudaErrorMemoryAllocation)
        return fail(EF_ERR_NOMEM, std::string(what) + ": " + cudaGetErrorString(e));
    return fail(EF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

bool finite_box(double a, double b) { return a == a && b == b && b > a; }

// One-patch run of a leaf kernel (FiniteVolumeSolver entry points).
int run_single_patch(int solver_type, int n, double xl, double xu, double yl, double yu,
                     double lambda, int mode, const double* g_host, const double* f_host,
                     double* out_host, size_t out_count) {
    if (solver_type != EF_SOLVER_FISHPACK90)
        return fail(EF_ERR_UNSUPPORTED,
                    "single-patch entry points implement the FISHPACK90 (constant coefficient) solver");
    if (n < 2 || n > 64) return fail(EF_ERR_INVALID, "n must be in [2, 64]");
    if (!finite_box(xl, xu) || !finite_box(yl, yu)) return fail(EF_ERR_INVALID, "bad patch box");
    if (!out_host) return fail(EF_ERR_INVALID, "null output");
    const int nn = n * n;
    const double dx = (xu - xl) / n, dy = (yu - yl) / n;
    std::vector<double> V(nn), Dinv(nn);
    efgb::leaf_tables(n, dx, dy, lambda, V.data(), Dinv.data());
    const int nitems = (mode == efgb::LEAF_DTN_COLUMN) ? 4 * n : 1;
    const size_t bytes = sizeof(double) * (2 * nn + 4 * n + nn + out_count) + sizeof(efgb::LeafType) +
                         sizeof(efgb::LeafItem) * nitems + 1024;
    char* buf = nullptr;
    int st = cuda_status(cudaMalloc(&buf, bytes), "cudaMalloc");
    if (st) return st;
    double* dV = reinterpret_cast<double*>(buf);
    double* dD = dV + nn;
    double* dg = dD + nn;
    double* df = dg + 4 * n;
    double* dout = df + nn;
    auto* dty = reinterpret_cast<efgb::LeafType*>(
        (reinterpret_cast<uintptr_t>(dout + out_count) + 255) & ~uintptr_t(255));
    auto* ditems = reinterpret_cast<efgb::LeafItem*>(
        (reinterpret_cast<uintptr_t>(dty + 1) + 255) & ~uintptr_t(255));
    if (reinterpret_cast<char*>(ditems + nitems) > buf + bytes + 1024) {
        cudaFree(buf);
        return fail(EF_ERR_INVALID, "internal layout error");
    }
    efgb::LeafType ty{n, dx, dy, dV, dD};
    std::vector<efgb::LeafItem> items(nitems);
    for (int k = 0; k < nitems; ++k)
        items[k] = efgb::LeafItem{0, k, f_host ? df : nullptr, g_host ? dg : nullptr, dout};
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = cudaMemcpy(dV, V.data(), nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dD, Dinv.data(), nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && g_host) e = cudaMemcpy(dg, g_host, 4 * n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && f_host) e = cudaMemcpy(df, f_host, nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dty, &ty, sizeof(ty), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(ditems, items.data(), nitems * sizeof(efgb::LeafItem), cudaMemcpyHostToDevice);
    int singular = 0;
    if (e == cudaSuccess) {
        if (mode == efgb::LEAF_DTN_COLUMN) {
            // the DtN map by a pivoted dense LU of the 5-point operator (as in a tree build)
            try {
                singular = efgb::leaf_dtn_lu(0, n, lambda, {dx}, {dy}, {dout});
            } catch (...) {
                cudaFree(buf);
                throw;
            }
        } else {
            if (n == 16) efgb::leaf_set_basis16(0);
            efgb::leaf_eigen(0, mode, dty, ditems, nitems, n);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out_host, dout, out_count * 8, cudaMemcpyDeviceToHost);
    cudaFree(buf);
    if (singular) return fail(EF_ERR_SINGULAR, "the 5-point operator of the patch is singular");
    return cuda_status(e, "single patch");
}

// One-patch run of the variable-coefficient (FivePointStencil) leaf kernels.
int run_single_patch_fp(int n, double xl, double xu, double yl, double yu, const double* alpha,
                        const double* beta, const double* lambda, int mode, const double* g_host,
                        const double* f_host, double* out_host, size_t out_count) {
    if (n < 2 || n > 64) return fail(EF_ERR_INVALID, "n must be in [2, 64]");
    if (!finite_box(xl, xu) || !finite_box(yl, yu)) return fail(EF_ERR_INVALID, "bad patch box");
    if (!alpha || !beta || !lambda || !out_host) return fail(EF_ERR_INVALID, "null argument");
    const size_t nn = size_t(n) * n;
    const int nitems = (mode == efgb::LEAF_DTN_COLUMN) ? 4 * n : 1;
    // doubles: coefficients 6nn, band nn(2n+1), bcoef 4n, g 4n, f nn, out; then structs
    const size_t ndbl = 6 * nn + nn * (2 * n + 1) + 4 * n + 4 * n + nn + out_count;
    const size_t bytes = ndbl * 8 + 256 + sizeof(efgb::FpLeaf) + 256 + sizeof(efgb::LeafItem) * nitems + 256;
    char* buf = nullptr;
    int st = cuda_status(cudaMalloc(&buf, bytes), "cudaMalloc");
    if (st) return st;
    double* coef = reinterpret_cast<double*>(buf);
    double* band = coef + 6 * nn;
    double* bcoef = band + nn * (2 * n + 1);
    double* dg = bcoef + 4 * n;
    double* df = dg + 4 * n;
    double* dout = df + nn;
    auto* dinfo = reinterpret_cast<int*>((reinterpret_cast<uintptr_t>(dout + out_count) + 255) & ~uintptr_t(255));
    auto* dleaf = reinterpret_cast<efgb::FpLeaf*>((reinterpret_cast<uintptr_t>(dinfo + 1) + 255) & ~uintptr_t(255));
    auto* ditems = reinterpret_cast<efgb::LeafItem*>((reinterpret_cast<uintptr_t>(dleaf + 1) + 255) & ~uintptr_t(255));
    const double dx = (xu - xl) / n, dy = (yu - yl) / n;
    efgb::FpLeaf lf{n, dx, dy, coef, coef + nn, coef + 5 * nn, band, bcoef, dinfo};
    std::vector<efgb::LeafItem> items(nitems);
    for (int k = 0; k < nitems; ++k)
        items[k] = efgb::LeafItem{0, k, f_host ? df : nullptr, g_host ? dg : nullptr, dout};
    cudaError_t e = cudaMemcpy(coef, alpha, nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(coef + nn, beta, 4 * nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(coef + 5 * nn, lambda, nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && g_host) e = cudaMemcpy(dg, g_host, 4 * n * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && f_host) e = cudaMemcpy(df, f_host, nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dinfo, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemcpy(dleaf, &lf, sizeof(lf), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ditems, items.data(), nitems * sizeof(efgb::LeafItem), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        efgb::fp_factor(0, dleaf, 1, n);
        efgb::fp_solve(0, mode, dleaf, ditems, nitems, n);
        e = cudaGetLastError();
    }
    int info = 0;
    if (e == cudaSuccess) e = cudaMemcpy(out_host, dout, out_count * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&info, dinfo, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(buf);
    st = cuda_status(e, "single patch (five-point)");
    if (st) return st;
    if (info > 0) return fail(EF_ERR_SINGULAR, "five-point operator has a zero pivot at row " + std::to_string(info - 1));
    if (info < 0)
        return fail(EF_ERR_UNSUPPORTED, "five-point operator is not negative definite (pivot of the wrong sign at row " +
                                            std::to_string(-info - 1) + "): the band LU without pivoting is not safe");
    return EF_OK;
}

}  // namespace

namespace efgb {
// lets the other translation units of the C ABI report a message through ef_last_error()
void set_last_error_message(const std::string& msg) { g_last_error = msg; }
}  // namespace efgb

extern "C" {

const char* ef_last_error(void) { return g_last_error.c_str(); }

int ef_version(void) { return 1; }

int ef_mesh_create_refined(double xl, double xu, double yl, double yu, int nx, int ny, int min_level,
                           int max_level, ef_refine_fn fn, void* ctx, ef_mesh** out) {
    if (!out || !fn) return fail(EF_ERR_INVALID, "null argument");
    if (!finite_box(xl, xu) || !finite_box(yl, yu)) return fail(EF_ERR_INVALID, "bad domain box");
    return guarded([&] {
        auto m = std::make_unique<ef_mesh>();
        m->mesh = efgb::Mesh::refine_by_function(
            xl, xu, yl, yu, nx, ny, min_level, max_level,
            [fn, ctx](double x, double y) { return fn(x, y, ctx) != 0; });
        *out = m.release();
        return EF_OK;
    });
}

int ef_mesh_create_uniform(double xl, double xu, double yl, double yu, int nx, int ny, int level,
                           ef_mesh** out) {
    if (!out) return fail(EF_ERR_INVALID, "null argument");
    if (!finite_box(xl, xu) || !finite_box(yl, yu)) return fail(EF_ERR_INVALID, "bad domain box");
    if (nx <= 0 || ny <= 0) return fail(EF_ERR_INVALID, "bad patch size");
    return guarded([&] {
        auto m = std::make_unique<ef_mesh>();
        m->mesh = efgb::Mesh::uniform(xl, xu, yl, yu, nx, ny, level);
        *out = m.release();
        return EF_OK;
    });
}

int ef_mesh_num_leaves(const ef_mesh* mesh, int* out) {
    if (!mesh || !out) return fail(EF_ERR_INVALID, "null argument");
    *out = int(mesh->mesh.leaves.size());
    return EF_OK;
}

int ef_mesh_num_nodes(const ef_mesh* mesh, int* out) {
    if (!mesh || !out) return fail(EF_ERR_INVALID, "null argument");
    *out = int(mesh->mesh.nodes.size());
    return EF_OK;
}

int ef_mesh_leaf(const ef_mesh* mesh, int k, int* level, long long* ix, long long* iy, double box[4]) {
    if (!mesh) return fail(EF_ERR_INVALID, "null mesh");
    if (k < 0 || k >= int(mesh->mesh.leaves.size())) return fail(EF_ERR_INVALID, "leaf index out of range");
    const efgb::MeshNode& nd = mesh->mesh.nodes[mesh->mesh.leaves[k]];
    if (level) *level = nd.level;
    if (ix) *ix = nd.ix;
    if (iy) *iy = nd.iy;
    if (box) { box[0] = nd.xl; box[1] = nd.xu; box[2] = nd.yl; box[3] = nd.yu; }
    return EF_OK;
}

int ef_mesh_level_count(const ef_mesh* mesh, int level, int* count) {
    if (!mesh || !count) return fail(EF_ERR_INVALID, "null argument");
    if (level < 0) return fail(EF_ERR_INVALID, "negative level");
    *count = int(efgb::level_nodes(mesh->mesh, level).size());
    return EF_OK;
}

int ef_mesh_subtree(const ef_mesh* mesh, int level, int index, ef_mesh** out) {
    if (!mesh || !out) return fail(EF_ERR_INVALID, "null argument");
    if (level < 0) return fail(EF_ERR_INVALID, "negative level");
    return guarded([&] {
        auto m = std::make_unique<ef_mesh>();
        m->mesh = efgb::subtree_mesh(mesh->mesh, level, index);
        *out = m.release();
        return EF_OK;
    });
}

int ef_mesh_destroy(ef_mesh* mesh) {
    delete mesh;
    return EF_OK;
}

int ef_hps_create(const ef_mesh* mesh, int solver_type, double lambda, ef_hps** out) {
    if (!mesh || !out) return fail(EF_ERR_INVALID, "null argument");
    if (solver_type != EF_SOLVER_FISHPACK90 && solver_type != EF_SOLVER_FIVE_POINT)
        return fail(EF_ERR_INVALID, "unknown solver type");
    return guarded([&] {
        auto h = std::make_unique<ef_hps>();
        h->hps = std::make_unique<efgb::Hps>(mesh->mesh, solver_type, lambda, false);
        *out = h.release();
        return EF_OK;
    });
}

int ef_hps_set_coefficients(ef_hps* h, const double* alpha, const double* beta, const double* lambda) {
    if (!h || !alpha || !beta || !lambda) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        h->hps->set_coefficients(alpha, beta, lambda);
        return EF_OK;
    });
}

int ef_hps_set_option(ef_hps* h, const char* key, int value) {
    if (!h || !key) return fail(EF_ERR_INVALID, "null argument");
    const std::string k(key);
    if (k == "cache-operators") {
        h->cache_operators = value != 0;
    } else if (k == "homogeneous-rhs") {
        h->homogeneous_rhs = value != 0;
        h->hps->set_homogeneous_rhs(value != 0);
    } else if (k == "cuda-graphs") {
        h->hps->set_graphs(value != 0);
    } else if (k == "inject-wait-timeout") {
        // failure-path test of the bounded TMA waits (process-wide): the node GEMMs' first wait runs
        // out and the mixed solve returns EF_ERR_CUDA while the context stays usable
        return guarded([&] {
            efgb::mx_set_inject_timeout(value != 0);
            return EF_OK;
        });
    } else if (k == "tensor-cores") {
        if (value < 0 || value > 2) return fail(EF_ERR_INVALID, "tensor-cores: 0 off, 1 tuned, 2 forced");
        h->hps->set_tensor_cores(value);  // block solvers created from now on
    } else if (k == "per-level-interface") {
        efgb::g_level_interface.store(value != 0);  // process-wide, block solvers created from now on
    } else if (k == "general-leaf-residual") {
        efgb::g_general_residual.store(value != 0);  // process-wide
    } else if (k == "cooperative-lu") {
        efgb::g_cooperative_lu.store(value != 0);  // process-wide
    } else {
        return fail(EF_ERR_INVALID, "unknown option key: " + k);
    }
    return EF_OK;
}

int ef_hps_set_stream(ef_hps* h, void* stream) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    h->hps->set_stream(reinterpret_cast<cudaStream_t>(stream));
    return EF_OK;
}

int ef_hps_build_info(const ef_hps* h, long long* merge_launches, long long* graph_replays) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (merge_launches) *merge_launches = h->hps->build_launches();
    if (graph_replays) *graph_replays = h->hps->build_replays();
    return EF_OK;
}

int ef_hps_root_factorizations(const ef_hps* h, long long* count) {
    if (!h || !count) return fail(EF_ERR_INVALID, "null argument");
    *count = h->hps->root_factorizations();
    return EF_OK;
}

int ef_hps_info(const ef_hps* h, int* nleaves, int* n, int* M, long long* bytes) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (nleaves) *nleaves = h->hps->num_leaves();
    if (n) *n = h->hps->leaf_n();
    if (M) *M = h->hps->root_M();
    if (bytes) *bytes = (long long)h->hps->device_bytes();
    return EF_OK;
}

int ef_hps_setup(ef_hps* h) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    return EF_OK;
}

int ef_hps_build(ef_hps* h) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    return guarded([&] {
        h->mixed.reset();  // FP32 operator copies belong to the previous build
        h->hps->build();
        if (h->hps->indefinite_count() > 0)
            return fail(EF_ERR_UNSUPPORTED,
                        std::to_string(h->hps->indefinite_count()) +
                            " FivePointStencil leaf operators are not negative definite (lambda above the smallest "
                            "eigenvalue of the diffusion part, or alpha*beta changing sign): the band LU without "
                            "pivoting is not safe for them");
        if (h->hps->singular_count() > 0)
            return fail(EF_ERR_SINGULAR, std::to_string(h->hps->singular_count()) +
                                             " interface matrices had a zero pivot (dgesv INFO != 0)");
        return EF_OK;
    });
}

int ef_hps_build_mixed(ef_hps* h, int fp64_levels) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    return guarded([&] {
        h->mixed.reset();
        h->hps->build_mixed(fp64_levels);
        if (h->hps->singular_count() > 0)
            return fail(EF_ERR_SINGULAR, std::to_string(h->hps->singular_count()) +
                                             " interface matrices had a zero pivot");
        return EF_OK;
    });
}

int ef_hps_build_from(ef_hps* h, const ef_hps* old, int* reused) {
    if (!h || !old) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        h->mixed.reset();
        h->hps->build_from(*old->hps);
        if (reused) *reused = h->hps->reused_merges();
        if (h->hps->singular_count() > 0)
            return fail(EF_ERR_SINGULAR, std::to_string(h->hps->singular_count()) +
                                             " interface matrices had a zero pivot (dgesv INFO != 0)");
        return EF_OK;
    });
}

int ef_hps_save(const ef_hps* h, const char* path) {
    if (!h || !path) return fail(EF_ERR_INVALID, "null argument");
    if (!h->hps->built()) return fail(EF_ERR_STATE, "save before build stage");
    if (h->hps->top_level() >= 0) return fail(EF_ERR_STATE, "save of a tree built by ef_hps_build_top");
    return guarded([&] {
        h->hps->save(path);
        return EF_OK;
    });
}

int ef_hps_load(const char* path, ef_mesh** mesh_out, ef_hps** hps_out) {
    if (!path || !mesh_out || !hps_out) return fail(EF_ERR_INVALID, "null argument");
    *mesh_out = nullptr;
    *hps_out = nullptr;
    return guarded([&] {
        auto h = std::make_unique<ef_hps>();
        h->hps = efgb::Hps::load(path);
        auto m = std::make_unique<ef_mesh>();
        m->mesh = h->hps->mesh();
        *mesh_out = m.release();
        *hps_out = h.release();
        return EF_OK;
    });
}

int ef_hps_split_sizes(ef_hps* h, int level, int* sizes) {
    if (!h || !sizes) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        const std::vector<int> v = h->hps->split_sizes(level);
        std::memcpy(sizes, v.data(), v.size() * sizeof(int));
        return EF_OK;
    });
}

int ef_hps_build_top(ef_hps* h, int level, const double* const* T) {
    if (!h || !T) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        h->mixed.reset();
        h->drop_lanes();
        h->hps->build_top(level, T);
        if (h->hps->singular_count() > 0)
            return fail(EF_ERR_SINGULAR, std::to_string(h->hps->singular_count()) +
                                             " interface matrices had a zero pivot (dgesv INFO != 0)");
        return EF_OK;
    });
}

int ef_hps_upwards_top(ef_hps* h, int level, const double* const* hv) {
    if (!h || !hv) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        h->hps->upwards_top(level, hv);
        h->upward_done = true;
        return EF_OK;
    });
}

int ef_hps_solve_top(ef_hps* h, int level, const double* a, const double* b, const double* r, double* const* g) {
    if (!h || !a || !b || !r || !g) return fail(EF_ERR_INVALID, "null argument");
    if (h->hps->top_level() != level) return fail(EF_ERR_STATE, "solve_top before build_top at this level");
    return guarded([&] {
        efgb::Hps& H = *h->hps;
        const size_t m = 4 * size_t(H.root_M());
        bool general = false;
        for (size_t i = 0; i < m; ++i)
            if (b[i] != 0.0) { general = true; break; }
        cudaStream_t s = H.stream();
        int st = cuda_status(cudaMemcpyAsync(H.bc_a(), a, m * 8, cudaMemcpyHostToDevice, s), "copy a");
        if (!st) st = cuda_status(cudaMemcpyAsync(H.bc_b(), b, m * 8, cudaMemcpyHostToDevice, s), "copy b");
        if (!st) st = cuda_status(cudaMemcpyAsync(H.bc_r(), r, m * 8, cudaMemcpyHostToDevice, s), "copy r");
        if (st) return st;
        H.set_bc_general(general);
        H.solve_top(level, g);
        return EF_OK;
    });
}

int ef_hps_upwards(ef_hps* h, const double* f_host) {
    if (!h || !f_host) return fail(EF_ERR_INVALID, "null argument");
    if (!h->hps->built()) return fail(EF_ERR_STATE, "upwards stage before build stage");
    if (h->hps->top_level() >= 0) return fail(EF_ERR_STATE, "tree built by ef_hps_build_top: use ef_hps_upwards_top");
    return guarded([&] {
        efgb::Hps& H = *h->hps;
        const size_t cnt = size_t(H.num_leaves()) * H.leaf_n() * H.leaf_n();
        int st = cuda_status(cudaMemcpyAsync(H.leaf_f(), f_host, cnt * 8, cudaMemcpyHostToDevice,
                                             H.stream()), "copy f");
        if (st) return st;
        H.upwards();
        st = cuda_status(cudaGetLastError(), "upwards launch");
        if (st) return st;
        st = cuda_status(cudaStreamSynchronize(H.stream()), "upwards");
        if (st) return st;
        h->upward_done = true;
        return EF_OK;
    });
}

int ef_hps_solve(ef_hps* h, const double* a, const double* b, const double* r) {
    if (!h || !a || !b || !r) return fail(EF_ERR_INVALID, "null argument");
    if (!h->hps->built()) return fail(EF_ERR_STATE, "solve stage before build stage");
    if (h->hps->top_level() >= 0) return fail(EF_ERR_STATE, "tree built by ef_hps_build_top: use ef_hps_solve_top");
    return guarded([&] {
        efgb::Hps& H = *h->hps;
        const size_t m = 4 * size_t(H.root_M());
        bool general = false;
        for (size_t i = 0; i < m; ++i)
            if (b[i] != 0.0) { general = true; break; }
        cudaStream_t s = H.stream();
        int st = cuda_status(cudaMemcpyAsync(H.bc_a(), a, m * 8, cudaMemcpyHostToDevice, s), "copy a");
        if (!st) st = cuda_status(cudaMemcpyAsync(H.bc_b(), b, m * 8, cudaMemcpyHostToDevice, s), "copy b");
        if (!st) st = cuda_status(cudaMemcpyAsync(H.bc_r(), r, m * 8, cudaMemcpyHostToDevice, s), "copy r");
        if (st) return st;
        H.set_bc_general(general);
        H.root_from_bc();
        H.downwards();
        st = cuda_status(cudaGetLastError(), "solve launch");
        if (st) return st;
        return cuda_status(cudaStreamSynchronize(s), "solve");
    });
}

int ef_hps_solve_root_dirichlet(ef_hps* h, const double* g) {
    if (!h || !g) return fail(EF_ERR_INVALID, "null argument");
    if (!h->hps->built()) return fail(EF_ERR_STATE, "solve stage before build stage");
    if (h->hps->top_level() >= 0) return fail(EF_ERR_STATE, "tree built by ef_hps_build_top: use ef_hps_solve_top");
    return guarded([&] {
        efgb::Hps& H = *h->hps;
        const size_t m = 4 * size_t(H.root_M());
        int st = cuda_status(cudaMemcpyAsync(H.root_g(), g, m * 8, cudaMemcpyHostToDevice, H.stream()),
                             "copy root g");
        if (st) return st;
        H.downwards();
        st = cuda_status(cudaGetLastError(), "solve launch");
        if (st) return st;
        return cuda_status(cudaStreamSynchronize(H.stream()), "solve");
    });
}

int ef_hps_get_leaf_u(ef_hps* h, double* u) {
    if (!h || !u) return fail(EF_ERR_INVALID, "null argument");
    efgb::Hps& H = *h->hps;
    const size_t cnt = size_t(H.num_leaves()) * H.leaf_n() * H.leaf_n();
    int st = cuda_status(cudaMemcpyAsync(u, H.leaf_u(), cnt * 8, cudaMemcpyDeviceToHost, H.stream()), "copy u");
    if (st) return st;
    return cuda_status(cudaStreamSynchronize(H.stream()), "copy u");
}

int ef_hps_get_root_T(ef_hps* h, double* T) {
    if (!h || !T) return fail(EF_ERR_INVALID, "null argument");
    if (!h->hps->built()) return fail(EF_ERR_STATE, "root T before build stage");
    efgb::Hps& H = *h->hps;
    const size_t m = 4 * size_t(H.root_M());
    int st = cuda_status(cudaMemcpyAsync(T, H.root_T(), m * m * 8, cudaMemcpyDeviceToHost, H.stream()), "copy T");
    if (st) return st;
    return cuda_status(cudaStreamSynchronize(H.stream()), "copy T");
}

int ef_hps_get_root_h(ef_hps* h, double* out) {
    if (!h || !out) return fail(EF_ERR_INVALID, "null argument");
    efgb::Hps& H = *h->hps;
    const size_t m = 4 * size_t(H.root_M());
    int st = cuda_status(cudaMemcpyAsync(out, H.root_h(), m * 8, cudaMemcpyDeviceToHost, H.stream()), "copy h");
    if (st) return st;
    return cuda_status(cudaStreamSynchronize(H.stream()), "copy h");
}

int ef_hps_destroy(ef_hps* h) {
    delete h;
    return EF_OK;
}

int ef_hps_device_buffers(ef_hps* h, double** f, double** u, double** a, double** b, double** r) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    efgb::Hps& H = *h->hps;
    if (f) *f = H.leaf_f();
    if (u) *u = H.leaf_u();
    if (a) *a = H.bc_a();
    if (b) *b = H.bc_b();
    if (r) *r = H.bc_r();
    return EF_OK;
}

int ef_hps_load_device_async(ef_hps* h, const double* f, const double* a, const double* b,
                             const double* r) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    efgb::Hps& H = *h->hps;
    cudaStream_t s = H.stream();
    const size_t nf = size_t(H.num_leaves()) * H.leaf_n() * H.leaf_n();
    const size_t m = 4 * size_t(H.root_M());
    int st = EF_OK;
    if (f) st = cuda_status(cudaMemcpyAsync(H.leaf_f(), f, nf * 8, cudaMemcpyDeviceToDevice, s), "load f");
    if (!st && a) st = cuda_status(cudaMemcpyAsync(H.bc_a(), a, m * 8, cudaMemcpyDeviceToDevice, s), "load a");
    if (!st && b) st = cuda_status(cudaMemcpyAsync(H.bc_b(), b, m * 8, cudaMemcpyDeviceToDevice, s), "load b");
    if (!st && r) st = cuda_status(cudaMemcpyAsync(H.bc_r(), r, m * 8, cudaMemcpyDeviceToDevice, s), "load r");
    return st;
}

int ef_hps_solve_device_async(ef_hps* h, int b_is_zero) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (!h->hps->built()) return fail(EF_ERR_STATE, "solve before build stage");
    if (h->hps->top_level() >= 0) return fail(EF_ERR_STATE, "tree built by ef_hps_build_top: use ef_hps_solve_top");
    return guarded([&] {
        h->hps->set_bc_general(b_is_zero == 0);
        h->hps->solve_async();
        return cuda_status(cudaGetLastError(), "solve launch");
    });
}

int ef_hps_synchronize(ef_hps* h) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    return cuda_status(cudaStreamSynchronize(h->hps->stream()), "synchronize");
}

int ef_hps_mixed_init(ef_hps* h, int bmax) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (!h->hps->built() && !h->hps->built32()) return fail(EF_ERR_STATE, "mixed solver before build stage");
    if (h->hps->top_level() >= 0) return fail(EF_ERR_STATE, "mixed solver on a tree built by ef_hps_build_top");
    return guarded([&] {
        h->drop_lanes();
        h->mixed.reset();
        h->root_a.clear();
        h->root_b.clear();
        h->mixed = std::make_unique<efgb::MixedSolver>(*h->hps, bmax);
        return EF_OK;
    });
}

int ef_hps_mixed_buffers(ef_hps* h, double** f, double** a, double** r, double** u) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    if (f) *f = h->mixed->f();
    if (a) *a = h->mixed->a();
    if (r) *r = h->mixed->r();
    if (u) *u = h->mixed->u();
    return EF_OK;
}

int ef_hps_mixed_solve_async(ef_hps* h, int batch, int sweeps) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    return guarded([&] {
        h->mixed->solve(batch, sweeps);
        return cuda_status(cudaGetLastError(), "mixed solve launch");
    });
}

int ef_hps_mixed_solve(ef_hps* h, int batch, int sweeps, const double* f, const double* a, const double* r,
                       double* u) {
    if (!h || !f || !a || !r || !u) return fail(EF_ERR_INVALID, "null argument");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    if (batch < 1 || batch > h->mixed->bmax()) return fail(EF_ERR_INVALID, "batch size out of range");
    return guarded([&] {
        efgb::Hps& H = *h->hps;
        efgb::MixedSolver& X = *h->mixed;
        cudaStream_t s = H.stream();
        const size_t cells = size_t(H.num_leaves()) * H.leaf_n() * H.leaf_n() * batch;
        const size_t m = 4 * size_t(H.root_M()) * batch;
        int st = cuda_status(cudaMemcpyAsync(X.f(), f, cells * 8, cudaMemcpyHostToDevice, s), "copy f");
        if (!st) st = cuda_status(cudaMemcpyAsync(X.a(), a, m * 8, cudaMemcpyHostToDevice, s), "copy a");
        if (!st) st = cuda_status(cudaMemcpyAsync(X.r(), r, m * 8, cudaMemcpyHostToDevice, s), "copy r");
        if (st) return st;
        X.solve(batch, sweeps);
        st = cuda_status(cudaGetLastError(), "mixed solve launch");
        if (!st) st = cuda_status(cudaMemcpyAsync(u, X.u(), cells * 8, cudaMemcpyDeviceToHost, s), "copy u");
        if (st) return st;
        st = cuda_status(cudaStreamSynchronize(s), "mixed solve");
        if (!st && X.take_error()) return fail(EF_ERR_CUDA, "mixed solve: an operator tile copy did not complete");
        return st;
    });
}

namespace {
// lane k >= 1 (shares the FP32 operators of h->mixed, own stream), created on first use; it starts
// after the work already queued on the tree's stream
int ensure_lane(ef_hps* h, int k) {
    if (!h->lanes[k]) {
        if (!h->lane_st[k]) {
            const int st = cuda_status(cudaStreamCreateWithFlags(&h->lane_st[k], cudaStreamNonBlocking), "lane stream");
            if (st) return st;
        }
        h->lanes[k] = std::make_unique<efgb::MixedSolver>(*h->hps, h->mixed->bmax(), h->mixed.get());
        h->lanes[k]->set_stream(h->lane_st[k]);
        if (!h->root_b.empty()) h->lanes[k]->set_root_operator(h->root_a.data(), h->root_b.data());
    }
    cudaEvent_t ready;
    int st = cuda_status(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming), "lane event");
    if (!st) st = cuda_status(cudaEventRecord(ready, h->mixed->stream()), "lane event");
    if (!st) st = cuda_status(cudaStreamWaitEvent(h->lane_st[k], ready, 0), "lane event");
    cudaEventDestroy(ready);
    return st;
}

efgb::MixedSolver* lane_solver(ef_hps* h, int lane) { return lane == 0 ? h->mixed.get() : h->lanes[lane].get(); }
}  // namespace

int ef_hps_mixed_gemm_plan(ef_hps* h, int max_groups, int* table, int* ngroups) {
    if (!h || !ngroups) return fail(EF_ERR_INVALID, "null argument");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    const auto plan = h->mixed->gemm_plan();
    *ngroups = int(plan.size());
    if (table)
        for (int i = 0; i < int(plan.size()) && i < max_groups; ++i)
            for (int k = 0; k < 5; ++k) table[5 * i + k] = plan[i][k];
    return EF_OK;
}

int ef_hps_mixed_set_gemm_plan(ef_hps* h, const int* codes, int ngroups) {
    if (!h || !codes || ngroups < 0) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        std::vector<std::array<int, 3>> c(static_cast<size_t>(ngroups));
        for (int i = 0; i < ngroups; ++i) c[i] = {codes[3 * i], codes[3 * i + 1], codes[3 * i + 2]};
        h->hps->set_mx_plan(c);
        return EF_OK;
    });
}

int ef_hps_mixed_set_root(ef_hps* h, const double* a, const double* b) {
    if (!h || !a || !b) return fail(EF_ERR_INVALID, "null argument");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    return guarded([&] {
        h->mixed->set_root_operator(a, b);
        for (int k = 1; k < ef_hps::kMaxLanes; ++k)
            if (h->lanes[k]) {
                cudaStreamSynchronize(h->lane_st[k]);
                h->lanes[k]->set_root_operator(a, b);
            }
        h->root_a.assign(a, a + 4 * size_t(h->hps->root_M()));
        h->root_b.assign(b, b + 4 * size_t(h->hps->root_M()));
        return EF_OK;
    });
}

int ef_hps_mixed_lane(ef_hps* h, int lane, double** f, double** a, double** r, double** u, void** stream) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    if (lane < 0 || lane >= ef_hps::kMaxLanes) return fail(EF_ERR_INVALID, "lane out of range");
    return guarded([&] {
        if (lane > 0) {
            const int st = ensure_lane(h, lane);
            if (st) return st;
        }
        efgb::MixedSolver* X = lane_solver(h, lane);
        if (f) *f = X->f();
        if (a) *a = X->a();
        if (r) *r = X->r();
        if (u) *u = X->u();
        if (stream) *stream = (void*)X->stream();
        return EF_OK;
    });
}

int ef_hps_mixed_lane_solve_async(ef_hps* h, int lane, int batch, int sweeps) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    if (lane < 0 || lane >= ef_hps::kMaxLanes) return fail(EF_ERR_INVALID, "lane out of range");
    if (lane > 0 && !h->lanes[lane]) return fail(EF_ERR_STATE, "lane not set up (ef_hps_mixed_lane)");
    return guarded([&] {
        lane_solver(h, lane)->solve(batch, sweeps);
        return cuda_status(cudaGetLastError(), "mixed solve launch");
    });
}

int ef_hps_mixed_solve_blocks(ef_hps* h, int nblocks, const int* batch, int sweeps, const double* const* f,
                              const double* const* a, const double* const* r, double* const* u) {
    if (!h || !batch || !f || !a || !r || !u || nblocks < 0) return fail(EF_ERR_INVALID, "null argument");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    for (int k = 0; k < nblocks; ++k) {
        if (batch[k] < 1 || batch[k] > h->mixed->bmax()) return fail(EF_ERR_INVALID, "batch size out of range");
        if (!f[k] || !a[k] || !r[k] || !u[k]) return fail(EF_ERR_INVALID, "null block array");
    }
    return guarded([&] {
        efgb::Hps& H = *h->hps;
        // three lanes: while one lane solves, the copy engines serve the other two in both directions
        const int nl = nblocks < 3 ? (nblocks < 1 ? 1 : nblocks) : 3;
        for (int k = 1; k < nl; ++k) {
            const int st = ensure_lane(h, k);
            if (st) return st;
        }
        const size_t cells1 = size_t(H.num_leaves()) * H.leaf_n() * H.leaf_n();
        const size_t m1 = 4 * size_t(H.root_M());
        for (int k = 0; k < nblocks; ++k) {
            efgb::MixedSolver& X = *lane_solver(h, k % nl);
            cudaStream_t s = X.stream();
            const size_t cells = cells1 * batch[k], m = m1 * batch[k];
            int st = cuda_status(cudaMemcpyAsync(X.f(), f[k], cells * 8, cudaMemcpyHostToDevice, s), "copy f");
            if (!st) st = cuda_status(cudaMemcpyAsync(X.a(), a[k], m * 8, cudaMemcpyHostToDevice, s), "copy a");
            if (!st) st = cuda_status(cudaMemcpyAsync(X.r(), r[k], m * 8, cudaMemcpyHostToDevice, s), "copy r");
            if (st) return st;
            X.solve(batch[k], sweeps);
            st = cuda_status(cudaGetLastError(), "mixed solve launch");
            if (!st) st = cuda_status(cudaMemcpyAsync(u[k], X.u(), cells * 8, cudaMemcpyDeviceToHost, s), "copy u");
            if (st) return st;
        }
        int st = EF_OK;
        int err = 0;
        for (int k = 0; k < nl && k < nblocks; ++k) err |= lane_solver(h, k)->take_error();  // synchronises the lane
        if (err) return fail(EF_ERR_CUDA, "mixed solve: an operator tile copy did not complete");
        return st;
    });
}

int ef_hps_mixed_residuals(ef_hps* h, int passes, double* out) {
    if (!h || !out) return fail(EF_ERR_INVALID, "null argument");
    if (!h->mixed) return fail(EF_ERR_STATE, "mixed solver not initialised");
    if (passes < 1 || passes > efgb::MixedSolver::kMaxPasses) return fail(EF_ERR_INVALID, "passes out of range");
    efgb::MixedSolver& X = *h->mixed;
    int st = cuda_status(cudaStreamSynchronize(h->hps->stream()), "mixed residuals");
    if (st) return st;
    if (X.take_error()) return fail(EF_ERR_CUDA, "mixed solve: an operator tile copy did not complete");
    return cuda_status(cudaMemcpy(out, X.residual_max(), size_t(passes) * X.bmax() * 8, cudaMemcpyDeviceToHost),
                       "copy residuals");
}

int ef_kernel_launches(long long* count) {
    if (!count) return fail(EF_ERR_INVALID, "null argument");
    *count = efgb::g_kernel_launches.load();
    return EF_OK;
}

int ef_hps_profile_enable(ef_hps* h, int on) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    h->hps->set_profiling(on != 0);
    return EF_OK;
}

int ef_hps_profile_count(ef_hps* h, int* count) {
    if (!h || !count) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        *count = int(h->hps->profile_read().size());
        return EF_OK;
    });
}

int ef_hps_profile_entry(ef_hps* h, int i, char* name, int name_len, double* ms, long long* launches,
                         long long* calls, double* bytes, double* flops) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    return guarded([&] {
        const auto& st = h->hps->profile_read();
        if (i < 0 || i >= int(st.size())) return fail(EF_ERR_INVALID, "profile index out of range");
        const auto& e = st[i];
        if (name && name_len > 0) {
            std::strncpy(name, e.name.c_str(), size_t(name_len) - 1);
            name[name_len - 1] = 0;
        }
        if (ms) *ms = e.ms;
        if (launches) *launches = e.launches;
        if (calls) *calls = e.calls;
        if (bytes) *bytes = e.bytes;
        if (flops) *flops = e.flops;
        return EF_OK;
    });
}

int ef_hps_profile_reset(ef_hps* h) {
    if (!h) return fail(EF_ERR_INVALID, "null handle");
    return guarded([&] {
        h->hps->profile_reset();
        return EF_OK;
    });
}

int ef_fv_build_d2n(int solver_type, int n, double xl, double xu, double yl, double yu, double lambda,
                    double* T) {
    return guarded([&] {
        return run_single_patch(solver_type, n, xl, xu, yl, yu, lambda, efgb::LEAF_DTN_COLUMN, nullptr,
                                nullptr, T, size_t(16) * n * n);
    });
}

int ef_fv_solve(int solver_type, int n, double xl, double xu, double yl, double yu, double lambda,
                const double* g, const double* f, double* u) {
    if (!g) return fail(EF_ERR_INVALID, "null Dirichlet data");
    return guarded([&] {
        return run_single_patch(solver_type, n, xl, xu, yl, yu, lambda, efgb::LEAF_SOLVE, g, f, u,
                                size_t(n) * n);
    });
}

int ef_fv_map_d2n(int solver_type, int n, double xl, double xu, double yl, double yu, double lambda,
                  const double* g, const double* f, double* h) {
    if (!g) return fail(EF_ERR_INVALID, "null Dirichlet data");
    return guarded([&] {
        return run_single_patch(solver_type, n, xl, xu, yl, yu, lambda, efgb::LEAF_MAPD2N, g, f, h,
                                size_t(4) * n);
    });
}

int ef_fv5_build_d2n(int n, double xl, double xu, double yl, double yu, const double* alpha,
                     const double* beta, const double* lambda, double* T) {
    return guarded([&] {
        return run_single_patch_fp(n, xl, xu, yl, yu, alpha, beta, lambda, efgb::LEAF_DTN_COLUMN, nullptr,
                                   nullptr, T, size_t(16) * n * n);
    });
}

int ef_fv5_solve(int n, double xl, double xu, double yl, double yu, const double* alpha, const double* beta,
                 const double* lambda, const double* g, const double* f, double* u) {
    if (!g) return fail(EF_ERR_INVALID, "null Dirichlet data");
    return guarded([&] {
        return run_single_patch_fp(n, xl, xu, yl, yu, alpha, beta, lambda, efgb::LEAF_SOLVE, g, f, u,
                                   size_t(n) * n);
    });
}

int ef_fv5_map_d2n(int n, double xl, double xu, double yl, double yu, const double* alpha,
                   const double* beta, const double* lambda, const double* g, const double* f, double* h) {
    if (!g) return fail(EF_ERR_INVALID, "null Dirichlet data");
    return guarded([&] {
        return run_single_patch_fp(n, xl, xu, yl, yu, alpha, beta, lambda, efgb::LEAF_MAPD2N, g, f, h,
                                   size_t(4) * n);
    });
}

// ---- serving loop ----------------------------------------------------------------------------

int ef_server_create(ef_hps* const* trees, const int* bmax, int ntrees, int lanes_per_tree,
                     long long hbm_budget_bytes, int sweeps, ef_server** out) {
    if (!trees || !bmax || !out || ntrees < 1) return fail(EF_ERR_INVALID, "null argument");
    *out = nullptr;
    std::vector<efgb::Server::TreeSpec> specs;
    for (int t = 0; t < ntrees; ++t) {
        if (!trees[t]) return fail(EF_ERR_INVALID, "null tree handle");
        if (!trees[t]->hps->built() && !trees[t]->hps->built32())
            return fail(EF_ERR_STATE, "server tree before build stage");
        specs.push_back(efgb::Server::TreeSpec{trees[t]->hps.get(), bmax[t]});
    }
    return guarded([&] {
        auto s = std::make_unique<ef_server>();
        s->srv = std::make_unique<efgb::Server>(specs, lanes_per_tree, hbm_budget_bytes, sweeps);
        *out = s.release();
        return EF_OK;
    });
}

int ef_server_set_root(ef_server* server, int tree, const double* a, const double* b) {
    if (!server || !a || !b) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        server->srv->set_root_operator(tree, a, b);
        return EF_OK;
    });
}

int ef_server_set_sweeps(ef_server* server, int tree, int sweeps) {
    if (!server) return fail(EF_ERR_INVALID, "null server");
    return guarded([&] {
        server->srv->set_sweeps(tree, sweeps);
        return EF_OK;
    });
}

int ef_server_info(ef_server* server, int tree, int* lanes, long long* device_bytes) {
    if (!server) return fail(EF_ERR_INVALID, "null server");
    return guarded([&] {
        if (lanes) *lanes = server->srv->lanes(tree);
        if (device_bytes) *device_bytes = server->srv->device_bytes();
        return EF_OK;
    });
}

int ef_server_submit(ef_server* server, int tree, const double* f, const double* a, const double* r, double* u,
                     long long* id) {
    if (!server || !id) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        *id = server->srv->submit(tree, f, a, r, u);
        return EF_OK;
    });
}

int ef_server_poll(ef_server* server, long long id, int* done, double* latency_s) {
    if (!server || !done) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        *done = server->srv->poll(id, latency_s);
        return EF_OK;
    });
}

int ef_server_wait(ef_server* server, long long id, double timeout_s, int* done, double* latency_s) {
    if (!server || !done) return fail(EF_ERR_INVALID, "null argument");
    return guarded([&] {
        *done = server->srv->wait(id, timeout_s, latency_s);
        return EF_OK;
    });
}

int ef_server_stats(ef_server* server, long long* submitted, long long* completed, long long* blocks,
                    long long* max_block) {
    if (!server) return fail(EF_ERR_INVALID, "null server");
    const efgb::Server::Stats st = server->srv->stats();
    if (submitted) *submitted = st.submitted;
    if (completed) *completed = st.completed;
    if (blocks) *blocks = st.batches;
    if (max_block) *max_block = st.max_batch;
    return EF_OK;
}

int ef_server_destroy(ef_server* server) {
    if (!server) return EF_OK;
    return guarded([&] {
        delete server;
        return EF_OK;
    });
}

}  // extern "C"
