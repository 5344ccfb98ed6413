// GB300 HPS solver: plan + device storage + stage drivers (plain FP64 form).
//
// Replaces HPSAlgorithm<FiniteVolumeGrid, FiniteVolumeSolver, FiniteVolumePatch, double>
// (src/HPSAlgorithm.hpp) on one GPU.  Instead of one callback per node in a p4est traversal, every
// stage runs level by level: all merges (or splits) of one tree level with the same child size are
// one grouped launch sequence.  Operators live in device memory owned by the Hps object.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "ef_kernels.cuh"
#include "ef_mesh.hpp"

namespace efgb {

enum SolverType : int { SOLVER_FIVE_POINT = 0, SOLVER_FISHPACK90 = 1 };

// Set-up upload ordered on the stream that later kernels run on: a plain cudaMemcpy runs on the
// legacy default stream, which a non-blocking stream does not wait for (and a pageable copy may
// return before its DMA is done), so tables uploaded that way could be read stale or overwritten by
// an earlier asynchronous clear of the same stream.  Copies, then synchronises the stream.
inline cudaError_t upload_sync(cudaStream_t st, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return cudaSuccess;
    const cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    return e != cudaSuccess ? e : cudaStreamSynchronize(st);
}

// Orthonormal sine basis V (n x n, V[i][k]) of the 1-D Dirichlet-ghost operator and the inverse
// 2-D eigenvalue table Dinv[k][l] = 1 / (mu_x[k] + mu_y[l] + lambda) of one patch geometry.
void leaf_tables(int n, double dx, double dy, double lambda, double* V, double* Dinv);

struct NodeDev {
    int nx = 0;        // grid cells per side of the node's patch (leaves: n, internal: 2s)
    int size = 0;      // nx >> ncoarsen (PatchBase::size(), Patch.hpp:99-101)
    int ncoarsen = 0;  // n_coarsens set when the parent merges (HPSAlgorithm.hpp:707-741)
    int s = 0;         // internal: coarsened child side
    int leaf_type = -1;
    double *T = nullptr, *Tc = nullptr;
    double *X = nullptr, *RHS = nullptr, *H = nullptr;
    int *piv = nullptr, *perm = nullptr;
    double *h = nullptr, *hc = nullptr, *g = nullptr, *gf = nullptr, *w = nullptr, *hd = nullptr;
    std::vector<double*> Tsteps, hsteps, gsteps;  // intermediate (un)coarsening buffers
};

struct Group {
    int level = 0, s = 0;
    std::vector<int> nodes;
    MergeItem* d_items = nullptr;
    double** d_X = nullptr;
    double** d_RHS = nullptr;
    double** d_H = nullptr;
    double** d_T = nullptr;
    int** d_piv = nullptr;
    int** d_perm = nullptr;
    int* d_info = nullptr;
    // T += H S as 8 row blocks per node: block b (s rows, child c(b)) multiplies its compact H rows
    // with the S rows of the two interfaces adjacent to c(b)
    const double** d_gA = nullptr;
    const double** d_gB = nullptr;
    const double** d_gB2 = nullptr;
    double** d_gC = nullptr;
};

struct ResampleStep {  // one batched (un)coarsening step: `count` items of fine size nf
    int level = 0;     // tree level of the nodes
    int nf = 0;
    int count = 0;
    const double** d_in = nullptr;
    double** d_out = nullptr;
};

struct LeafTypeHost {
    int n;
    double dx, dy;
    double* T = nullptr;
};

class MixedSolver;

// Replays a fixed launch sequence through a CUDA graph.  The first call with a key runs eagerly (so
// one-time kernel attributes and lazy allocations happen outside a capture), the second captures
// the sequence on a private non-blocking stream, later calls launch the instantiated graph on the
// caller's stream.  A sequence that cannot be captured keeps running eagerly.
class GraphCache {
public:
    GraphCache() = default;
    ~GraphCache() { clear(); }
    GraphCache(const GraphCache&) = delete;
    GraphCache& operator=(const GraphCache&) = delete;
    // body() launches on `stream`, which is switched to the capture stream while capturing
    template <class F>
    void run(cudaStream_t& stream, long long key, bool enabled, F&& body);
    void clear();
    long long replays() const { return replays_; }

private:
    struct Entry {
        long long key;
        bool failed;
        cudaGraphExec_t exec;
        long long launches;  // kernels of the captured sequence, added to the counter per replay
    };
    std::vector<Entry> entries_;
    cudaStream_t cap_ = nullptr;
    long long replays_ = 0;
};

template <class F>
void GraphCache::run(cudaStream_t& stream, long long key, bool enabled, F&& body) {
    if (!enabled) { body(); return; }
    Entry* e = nullptr;
    for (auto& x : entries_)
        if (x.key == key) { e = &x; break; }
    if (!e) {
        entries_.push_back(Entry{key, false, nullptr, 0});
        body();
        return;
    }
    if (e->failed) { body(); return; }
    if (!e->exec) {
        if (!cap_ && cudaStreamCreateWithFlags(&cap_, cudaStreamNonBlocking) != cudaSuccess) {
            cap_ = nullptr;
            e->failed = true;
            (void)cudaGetLastError();
            body();
            return;
        }
        cudaStream_t orig = stream;
        // the capture stream starts after the caller's pending work
        cudaEvent_t ev = nullptr;
        bool ok = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess &&
                  cudaEventRecord(ev, orig) == cudaSuccess && cudaStreamWaitEvent(cap_, ev, 0) == cudaSuccess;
        if (ev) cudaEventDestroy(ev);
        cudaGraph_t g = nullptr;
        if (ok) ok = cudaStreamBeginCapture(cap_, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        const long long l0 = g_kernel_launches.load();
        if (ok) {
            stream = cap_;
            try {
                body();
            } catch (...) {
                // a step that cannot be captured: drop the capture and run the sequence eagerly
                // from now on (a real error then surfaces from the eager run)
                stream = orig;
                cudaStreamEndCapture(cap_, &g);
                if (g) cudaGraphDestroy(g);
                (void)cudaGetLastError();
                g_kernel_launches -= g_kernel_launches.load() - l0;
                e->failed = true;
                body();
                return;
            }
            stream = orig;
            ok = cudaStreamEndCapture(cap_, &g) == cudaSuccess && g;
        }
        // launches counted while capturing belong to the replays
        e->launches = g_kernel_launches.load() - l0;
        g_kernel_launches -= e->launches;
        if (ok) ok = cudaGraphInstantiate(&e->exec, g, 0) == cudaSuccess;
        if (ok) ok = cudaGraphUpload(e->exec, stream) == cudaSuccess;  // first launch pays no upload
        if (g) cudaGraphDestroy(g);
        if (!ok) {
            e->failed = true;
            e->exec = nullptr;
            (void)cudaGetLastError();
            body();
            return;
        }
    }
    if (cudaGraphLaunch(e->exec, stream) != cudaSuccess) {
        (void)cudaGetLastError();
        e->failed = true;
        body();
        return;
    }
    g_kernel_launches += e->launches;
    ++replays_;
}

class Hps {
public:
    friend class MixedSolver;
    Hps(const Mesh& mesh, int solver_type, double lambda, bool cache_operators);
    ~Hps();
    Hps(const Hps&) = delete;
    Hps& operator=(const Hps&) = delete;

    void set_stream(cudaStream_t st) { st_ = st; }
    // CUDA-graph replay of the solve sequences (on by default; profiling runs them eagerly)
    void set_graphs(bool on) { graphs_ = on; }
    bool graphs() const { return graphs_; }
    // tcgen05 node GEMMs in the mixed solver for block solvers created afterwards: 0 off, 1 (default)
    // wherever the autotuner times them faster than the CUDA-core GEMMs, 2 wherever supported
    void set_tensor_cores(int mode) { tensor_cores_ = mode; }
    // node-GEMM plan of the mixed block solvers, per node group the W, H, DOWN codes as
    // MixedSolver::gemm_plan reports them (> 0 CUDA-core K split, 0 its heuristic, < 0 tensor-core
    // K split): block solvers created afterwards use it instead of timing the candidates
    void set_mx_plan(const std::vector<std::array<int, 3>>& codes);
    int tensor_cores() const { return tensor_cores_; }
    // FivePointStencil: per-leaf coefficients sampled at the reference's points (host arrays in leaf
    // order: alpha n*n, beta 4*n*n (W, E, S, N face of every cell), lambda n*n per leaf)
    void set_coefficients(const double* alpha, const double* beta, const double* lambda);
    int solver_type() const { return solver_type_; }
    cudaStream_t stream() const { return st_; }
    void set_homogeneous_rhs(bool v) { homogeneous_ = v; }
    // true when the boundary coefficient b of a*u + b*du/dn = r is not identically zero
    void set_bc_general(bool v) { bc_general_ = v; }
    bool homogeneous_rhs() const { return homogeneous_; }

    // Stages (synchronous to the host at their end unless noted).
    void build();                                  // HPSAlgorithm::buildStage
    // Mixed-precision build (no counterpart in the reference): every merge in FP32 except the
    // interface LU of the top `fp64_levels` tree levels, factored in FP64 and rounded to FP32.  Fills
    // the FP32 operator set the mixed block solver reads; the plain FP64 solve needs build().
    void build_mixed(int fp64_levels);
    bool built32() const { return built32_; }
    // Local re-factorisation after a mesh change (ef_incremental.cpp): merge nodes whose subtree is the
    // same in `old` copy its operators, the others merge; equal to build() bit for bit.
    void build_from(const Hps& old);
    int reused_merges() const { return reused_; }
    // A built tree's solve-time operators to a file and back (ef_serial.cpp).
    void save(const char* path) const;
    static std::unique_ptr<Hps> load(const char* path);
    // Subtree split (ef_subtree.cpp): this handle on the full mesh runs only the top `level` tree
    // levels, on the T / h of the level-`level` nodes built and upward-passed elsewhere as subtrees
    // of their own, and returns their g.  Every leaf must lie below `level`.
    std::vector<int> split_nodes(int level) const;   // node ids at `level`, pre-order
    std::vector<int> split_sizes(int level) const;   // 4m (length of h and g; T is 4m x 4m) per node
    void build_top(int level, const double* const* T_host);
    void upwards_top(int level, const double* const* h_host);
    void solve_top(int level, double* const* g_host);  // root data from bc_a/b/r
    int top_level() const { return top_level_; }      // -1 unless built by build_top
    // kernels launched by the merges of the last build(), and builds replayed from a CUDA graph
    long long build_launches() const { return build_launches_; }
    long long build_replays() const { return graph_build_.replays(); }
    void upwards();                                // HPSAlgorithm::upwardsStage on leaf_f()
    void root_from_bc();                           // root g from bc_a/b/r (HPSAlgorithm.hpp:402-420)
    void downwards();                              // split1to4 + leafSolve for every node
    void solve_async();                            // upwards + root + downwards, no host sync

    // Device buffers (resident, owned by this object).
    double* leaf_f() const { return d_f_; }        // nleaves * n * n, leaf order, j + i*n
    double* leaf_u() const { return d_u_; }
    double* bc_a() const { return d_bca_; }        // 4M each, WESN, root face centres
    double* bc_b() const { return d_bcb_; }
    double* bc_r() const { return d_bcr_; }
    double* root_g() const { return nodes_[0].g; }
    double* root_h() const { return nodes_[0].h; }
    double* root_T() const { return nodes_[0].T; }

    int num_leaves() const { return int(mesh_.leaves.size()); }
    int leaf_n() const { return n_; }
    int root_M() const { return nodes_[0].nx; }
    int num_nodes() const { return int(nodes_.size()); }
    const NodeDev& node(int i) const { return nodes_[i]; }
    const Mesh& mesh() const { return mesh_; }
    bool built() const { return built_; }
    int singular_count() const { return singular_; }
    // FivePointStencil leaves whose operator is not (alpha-scaled) negative definite: the band LU
    // without pivoting is not safe for them (last build)
    int indefinite_count() const { return indefinite_; }
    // LU factorisations of the general root matrix diag(a) + diag(b) T so far (cached across solves)
    long long root_factorizations() const { return root_factorizations_; }
    size_t device_bytes() const { return arena_bytes_; }

    // Counters for the roofline: flops of the build by kernel family (FP64).
    double build_flops() const;
    double solve_bytes() const;
    double solve_flops() const;

    // Section profiler: CUDA events on this handle's stream around every kernel family, with the
    // algorithmic bytes and flops each section moves/performs.
    struct ProfStat {
        std::string name;
        double ms = 0;
        long long launches = 0, calls = 0;
        double bytes = 0, flops = 0;
    };
    void set_profiling(bool on) { prof_ = on; }
    const std::vector<ProfStat>& profile_read();  // synchronises the stream
    void profile_reset();

private:
    void merge_levels(int top);       // merges of levels top .. 0
    void upward_levels(int top);      // upward pass of levels top .. 0
    void downward_levels(int bottom, bool uncoarsen_bottom);  // split from the root to level `bottom`
    int count_singular(int below);    // zero pivots among the merges of levels < below
    void plan();
    void allocate();
    void upload_tables();
    void build_leaf_types();
    void leaf_run(int mode, const LeafItem* items, int nitems);
    void check(cudaError_t e, const char* what);

    Mesh mesh_;
    int solver_type_;
    double lambda_;
    bool cache_ops_;
    bool homogeneous_ = false;
    bool bc_general_ = false;
    int n_ = 0;
    cudaStream_t st_ = 0;

    std::vector<NodeDev> nodes_;
    std::vector<Group> groups_;                 // ordered deepest level first
    std::vector<ResampleStep> tsteps_, hsteps_, gsteps_;
    std::vector<std::vector<int>> step_nodes_t_, step_nodes_g_;
    std::vector<int> step_index_t_, step_index_g_;
    double *d_V_ = nullptr, *d_Dinv_ = nullptr;
    // FivePointStencil leaves
    double* d_coef_ = nullptr;
    FpLeaf* d_fp_ = nullptr;
    int* d_fpinfo_ = nullptr;
    std::vector<double*> fp_band_, fp_bcoef_;
    bool coef_set_ = false;
    std::vector<LeafTypeHost> types_;
    LeafType* d_types_ = nullptr;
    LeafItem *d_items_dtn_ = nullptr, *d_items_neu_ = nullptr, *d_items_solve_ = nullptr;
    int nitems_dtn_ = 0;

    double *d_f_ = nullptr, *d_u_ = nullptr;
    double *d_bca_ = nullptr, *d_bcb_ = nullptr, *d_bcr_ = nullptr;
    // general (b != 0) root solve
    double *d_rootA_ = nullptr, *d_rootrhs_ = nullptr;
    int *d_rootpiv_ = nullptr, *d_rootperm_ = nullptr, *d_rootinfo_ = nullptr, *d_rootflag_ = nullptr;
    double *d_roota_ = nullptr, *d_rootb_ = nullptr;  // (a, b) of the cached root LU
    bool root_lu_valid_ = false;
    int root_flag_host_ = 0;
    long long root_factorizations_ = 0;
    double** d_rootA_arr_ = nullptr;
    double** d_rootrhs_arr_ = nullptr;
    int** d_rootpiv_arr_ = nullptr;
    int** d_rootperm_arr_ = nullptr;

    char* arena_ = nullptr;
    size_t arena_bytes_ = 0, arena_used_ = 0;

    bool built_ = false;
    int singular_ = 0;
    int leaf_singular_ = 0;
    int indefinite_ = 0;  // constant-coefficient leaf operators with a zero pivot (last build)
    int top_level_ = -1;

    struct Mark {
        int stat;
        cudaEvent_t a, b;
        long long launches;
        double bytes, flops;
    };
    // FP32 operator set of the mixed build (ef_build32.cpp)
    struct Node32 {
        float *T = nullptr, *Tc = nullptr, *X = nullptr, *RHS = nullptr, *H = nullptr;
        std::vector<float*> Tsteps;
    };
    struct Group32 {
        MergeItem32* d_items = nullptr;
        float** d_X = nullptr;
        float** d_RHS = nullptr;
        const float** d_gA = nullptr;
        const float** d_gB = nullptr;
        const float** d_gB2 = nullptr;
        float** d_gC = nullptr;
    };
    struct Step32 {
        const float** d_in = nullptr;
        float** d_out = nullptr;
    };
    void allocate32();
    std::vector<Node32> n32_;
    std::vector<Group32> g32_;
    std::vector<Step32> t32_;
    const double** d_tT64_ = nullptr;
    float** d_tT32_ = nullptr;
    char* arena32_ = nullptr;
    size_t arena32_bytes_ = 0;
    bool built32_ = false;
    int reused_ = 0;

    bool prof_ = false;
    bool graphs_ = true;
    int tensor_cores_ = 1;
    int mx_split_tc_ = -1;  // tensor-core mode mx_split_ was tuned with
    // K split of the mixed form's node GEMMs per group and kind (W, H, DOWN), chosen once per tree by
    // MixedSolver::tune and shared by every block solver of the tree
    std::vector<std::array<int, 3>> mx_split_;
    GraphCache graph_solve_;
    GraphCache graph_build_;
    long long build_launches_ = 0;
    std::vector<ProfStat> stats_;
    std::vector<Mark> marks_;
    std::vector<cudaEvent_t> ev_free_;
    int open_stat_ = -1;
    cudaEvent_t open_ev_ = nullptr;
    long long open_launch0_ = 0;
    cudaEvent_t ev_get();
    void pb(const char* name) { pb(name, st_); }                 // begin section
    void pe(double bytes, double flops) { pe(bytes, flops, st_); }  // end section
    void pb(const char* name, cudaStream_t st);
    void pe(double bytes, double flops, cudaStream_t st);
};

// Mixed-precision many-RHS solver on a built FP64 Hps (FISHPACK90 leaves, Dirichlet root data):
// FP32 copies of S, X^{-1}, H and the leaf tables; an exact residual (5-point leaf residual in
// fixed-point integer arithmetic + FP64 interface flux mismatches) and FP32 correction passes, see
// ef_mixed.cu.
class MixedSolver {
public:
    // share: another solver of the same tree whose FP32 operators (and TMA descriptors) this one
    // reuses, so that several lanes of one tree hold the operators once
    MixedSolver(Hps& hps, int bmax, const MixedSolver* share = nullptr);
    ~MixedSolver();
    MixedSolver(const MixedSolver&) = delete;
    MixedSolver& operator=(const MixedSolver&) = delete;

    int bmax() const { return bmax_; }
    // stream of this solver's launches (default: the tree's stream at construction)
    void set_stream(cudaStream_t st) { st_ = st; }
    cudaStream_t stream() const { return st_; }
    // Resident inputs: f [B][L][n*n], a and r [B][4M] (b == 0 assumed); output u [B][L][n*n].
    double* f() const { return f_; }
    double* a() const { return a_; }
    double* r() const { return r_; }
    double* u() const { return u64_; }
    // max |leaf residual| per request before each pass: [passes][bmax]
    double* residual_max() const { return rmax_; }
    size_t device_bytes() const { return bytes_; }
    // 1 + sweeps FP32 passes on B <= bmax requests; asynchronous on the Hps stream.
    void solve(int B, int sweeps);
    // Root operator of every later block (HPSAlgorithm.hpp:402-420): a u + b du/dn = r with a, b
    // (4M each, host) fixed and r per request.  b == 0 everywhere returns to Dirichlet data with the
    // per-request a.  Otherwise the root data become part of the state and every pass solves for
    // their correction with Z = (diag a + diag b T_root)^{-1}, factored in FP64 here (synchronous).
    void set_root_operator(const double* a, const double* b);
    // per node group: {level, s, code W, code H, code DOWN} of the tuned node GEMMs (code > 0: CUDA-core
    // kernel with that K split, code < 0: tensor-core kernel with K split -code)
    std::vector<std::array<int, 5>> gemm_plan() const;
    bool robin() const { return robin_; }
    // synchronises the stream; 1 when a kernel gave up waiting on a TMA copy since the last call
    int take_error();
    static constexpr int kMaxPasses = 8;

private:
    struct MNode {
        float *S = nullptr, *Xi = nullptr, *H32 = nullptr;
        float *h32 = nullptr, *hd32 = nullptr, *w32 = nullptr, *m32 = nullptr, *g32 = nullptr;
        double *uG = nullptr, *g64 = nullptr, *h64 = nullptr;
        std::vector<float*> hs32, gs32;
        std::vector<double*> hs64, gs64;
        float *hc32 = nullptr, *gf32 = nullptr;
        double *hc64 = nullptr, *gf64 = nullptr;
    };
    struct MGroup {
        int level = 0, s = 0, cnt = 0;
        MixItem* d_items = nullptr;
        MixConv* d_conv = nullptr;
        float *S32 = nullptr, *Xi32 = nullptr, *H32 = nullptr;
        CUtensorMap tmS{}, tmXi{}, tmH{};
        // tensor-core path: three bf16 planes per operator kind, tiled as the kernel's stage images
        bool tc[3] = {false, false, false};  // per kind (W, H, DOWN)
        void *S3 = nullptr, *Xi3 = nullptr, *H3 = nullptr;
    };
    struct MStep {
        int level = 0, nf = 0, count = 0;
        void** in32 = nullptr;
        void** out32 = nullptr;
        void** in64 = nullptr;
        void** out64 = nullptr;
    };
    // fused: the zero-state residual of 16 x 16 leaves together with the first pass's Neumann step
    // (mx_leaf16_first); the pass then starts at the upward GEMMs
    void residual(int B, double* rmax, bool zero_state, bool fused = false);
    // last: no residual follows, so the interface state need not take the pass's values
    void pass(int B, bool first, bool neumann_done = false, bool last = false);
    // one node GEMM of a group (kind 0 W, 1 H, 2 DOWN): code > 0 the FP32 CUDA-core kernel with K
    // split `code` (0: its heuristic), code < 0 the tensor-core kernel with K split -code
    void node_gemm(cudaStream_t st, const MGroup& g, int kind, int B, int code);
    double gemm_bytes(const MGroup& g, int kind, int B, int code) const;
    // times the K-split candidates of every node GEMM (CUDA events, block of min(bmax, 32)) and keeps
    // the fastest per group and kind in the tree
    void tune();

    Hps& H_;
    int bmax_;
    cudaStream_t st_;
    const MixedSolver* share_;
    char* arena_ = nullptr;
    size_t bytes_ = 0;
    std::vector<MNode> mn_;
    std::vector<MGroup> groups_;
    std::vector<MStep> hsteps_, gsteps_;
    LeafType32* d_types32_ = nullptr;
    MixLeaf* d_leaves_ = nullptr;
    float* q32_ = nullptr;
    double *u64_ = nullptr, *f_ = nullptr, *a_ = nullptr, *r_ = nullptr, *rmax_ = nullptr;
    int* d_err_ = nullptr;
    float* rleaf_ = nullptr;
    MixCoef* d_coef_ = nullptr;
    int res_form_ = 0;  // residual kernel form: 0 when all leaf types have dx = dy and lambda = 0
    // interface rows traced to the leaves (trees without coarsening steps)
    bool direct_ = false;
    MxRow* d_gsrc_ = nullptr;     // [L][4n] Dirichlet rows of the leaves
    MxMis* d_mis_ = nullptr;      // interface mismatch rows of every node
    MxAdd* d_add_ = nullptr;      // FP64 state update rows of every node
    long long nmis_ = 0;
    MxRow* d_rootsrc_ = nullptr;  // the root's boundary-flux rows (Robin root data)
    int nroot_ = 0;
    MixFp* d_fps_ = nullptr;  // FivePointStencil leaves only
    float* fp_band32_ = nullptr;
    float* fp_bcoef32_ = nullptr;
    double* fp_coef64_ = nullptr;
    GraphCache graphs_;
    char* uG_begin_ = nullptr;
    size_t uG_bytes_ = 0;
    float* tables_ = nullptr;
    // Robin root data (set_root_operator)
    bool robin_ = false;
    char* robin_mem_ = nullptr;
    double *ra64_ = nullptr, *rb64_ = nullptr;
    float *rb32_ = nullptr, *Z32_ = nullptr, *rho32_ = nullptr, *rhs32_ = nullptr;
    const float** zA_ = nullptr;
    const float** zB_ = nullptr;
    float** zC_ = nullptr;
};

}  // namespace efgb
