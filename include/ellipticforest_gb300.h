/* C ABI of the GB300-native HPS solver (drop-in for EllipticForest's HPS path).
 *
 * Every entry point returns EF_OK (0) on success or a negative EF_ERR_* code; ef_last_error()
 * gives the message of the last failure on the calling thread.  Plain pointers and sizes only.
 *
 * Data conventions (the reference's, src/HPSAlgorithm.hpp and
 * src/Patches/FiniteVolume/FiniteVolumeSolver.cpp):
 *   - leaves are numbered in pre-order (z-order: child 0 = SW, 1 = SE, 2 = NW, 3 = NE), the order
 *     in which Quadtree::traversePreOrder visits them;
 *   - a leaf's cell (i, j) (x-index i, y-index j) is stored at j + i*n (FiniteVolumeSolver.cpp:17);
 *   - boundary data are WESN-stacked, each side M long (W and E along y, S and N along x).
 *
 * One ef_hps handle may be used by one host thread at a time.  Calls are synchronous to the host
 * unless their name ends in _async.
 */
#ifndef ELLIPTICFOREST_GB300_H_
#define ELLIPTICFOREST_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

#define EF_OK 0
#define EF_ERR_INVALID (-1)     /* bad argument or size mismatch                       */
#define EF_ERR_CUDA (-2)        /* CUDA runtime error (message in ef_last_error)       */
#define EF_ERR_NOMEM (-3)       /* device or host allocation failed                     */
#define EF_ERR_SINGULAR (-4)    /* an LU factorisation met a zero pivot                 */
#define EF_ERR_STATE (-5)       /* call out of order (e.g. solve before build)          */
#define EF_ERR_UNSUPPORTED (-6) /* option or solver type not available in this build    */

#define EF_SOLVER_FIVE_POINT 0  /* FiniteVolumeSolverType::FivePointStencil */
#define EF_SOLVER_FISHPACK90 1  /* FiniteVolumeSolverType::FISHPACK90       */

typedef struct ef_mesh ef_mesh;
typedef struct ef_hps ef_hps;

/* Refinement predicate of Mesh::refineByFunction: non-zero means "refine". */
typedef int (*ef_refine_fn)(double x, double y, void* ctx);

const char* ef_last_error(void);
int ef_version(void);

/* ---- Mesh ----------------------------------------------------------------------------------- */

/* Mesh::refineByFunction (src/Mesh.hpp:111-180): uniform refinement to min_level, recursive
 * refinement of every patch with a cell centre where fn is true (up to max_level), then 2:1
 * corner balance.  nx, ny: cells per leaf patch side. */
int ef_mesh_create_refined(double x_lower, double x_upper, double y_lower, double y_upper, int nx,
                           int ny, int min_level, int max_level, ef_refine_fn fn, void* ctx,
                           ef_mesh** out);
/* Uniform quadtree of the given level (p4est_new_ext with fill_uniform, src/Mesh.hpp:131). */
int ef_mesh_create_uniform(double x_lower, double x_upper, double y_lower, double y_upper, int nx,
                           int ny, int level, ef_mesh** out);
int ef_mesh_num_leaves(const ef_mesh* mesh, int* out);
int ef_mesh_num_nodes(const ef_mesh* mesh, int* out);
/* Leaf k: level, integer coordinates at that level and its box [xl, xu] x [yl, yu]
 * (the node geometry of FiniteVolumeNodeFactory::createChildNode, NodeFactory.cpp:15-66). */
int ef_mesh_leaf(const ef_mesh* mesh, int k, int* level, long long* ix, long long* iy,
                 double box[4]);
int ef_mesh_destroy(ef_mesh* mesh);

/* ---- HPS solver (HPSAlgorithm<FiniteVolumeGrid, FiniteVolumeSolver, FiniteVolumePatch, double>)
 * -------------------------------------------------------------------------------------------- */

/* Creates the solver for `mesh` (copied) and allocates its device storage.
 * solver_type EF_SOLVER_FISHPACK90: u_xx + u_yy + lambda u = f (FiniteVolumeSolver.cpp:224-290,
 * lambda = lambda_function(0,0)). */
int ef_hps_create(const ef_mesh* mesh, int solver_type, double lambda, ef_hps** out);
/* FivePointStencil coefficients (required before ef_hps_build for EF_SOLVER_FIVE_POINT), sampled
 * per leaf cell at the reference's points (FiniteVolumeSolver.cpp:66-79), host arrays in leaf
 * order: alpha(x_i, y_j) (n*n per leaf), beta at the cell's W, E, S, N faces (x_i -/+ dx/2, y_j),
 * (x_i, y_j -/+ dy/2) (4*n*n per leaf: all W values, then E, S, N), lambda(x_i, y_j) (n*n). */
int ef_hps_set_coefficients(ef_hps* hps, const double* alpha, const double* beta,
                            const double* lambda);
/* Option keys of the reference: "cache-operators", "homogeneous-rhs" (HPSAlgorithm.hpp:134,532).
 * Added key "cuda-graphs" (default 1): replay the device-resident solve sequences
 * (ef_hps_solve_device_async, ef_hps_mixed_solve*) as CUDA graphs after their first two calls.
 * Added key "cooperative-lu" (default 1, process-wide): LU panels of interface matrices with >= 512
 * rows left run on many CTAs (one grid barrier per column); 0 keeps one CTA per panel.  Both give
 * the same factors bit for bit.
 * Added key "tensor-cores" (default 1) for the mixed block solvers created afterwards: 0 CUDA-core
 * node GEMMs only, 1 the faster of the CUDA-core and tcgen05 GEMM per node group (timed), 2 the
 * tcgen05 GEMM wherever it supports the shape.
 * Verification keys (process-wide, default 0): "general-leaf-residual" 1 runs the exact residual of
 * 16 x 16 leaves through the general leaf-size kernel; "per-level-interface" 1 makes mixed block
 * solvers created afterwards move the residual's interface rows level by level even on trees
 * without coarsening steps (which otherwise read and difference them in place).  Both give the same
 * results bit for bit; "inject-wait-timeout" 1 makes the tensor-core GEMMs' first wait run out
 * (failure-path test: the solve returns EF_ERR_CUDA). */
int ef_hps_set_option(ef_hps* hps, const char* key, int value);
/* Use an external CUDA stream (cudaStream_t) for all work of this handle; NULL = default stream. */
int ef_hps_set_stream(ef_hps* hps, void* cuda_stream);
int ef_hps_info(const ef_hps* hps, int* num_leaves, int* leaf_n, int* root_M, long long* device_bytes);
/* Number of LU factorisations of the general root matrix diag(a) + diag(b) T_root made so far.  The
 * reference factors it on every solve with b != 0 (HPSAlgorithm.hpp:402-420); here the factors are
 * reused while a and b are bit-identical to the last factored pair and the tree was not rebuilt. */
int ef_hps_root_factorizations(const ef_hps* hps, long long* count);

/* HPSAlgorithm::setupStage (HPSAlgorithm.hpp:91-106): nothing to do; validates the handle. */
int ef_hps_setup(ef_hps* hps);
/* HPSAlgorithm::buildStage (HPSAlgorithm.hpp:120-161): leaf DtN maps and all 4-to-1 merges. */
int ef_hps_build(ef_hps* hps);
/* Kernels launched by the merges of the last ef_hps_build (the leaf DtN maps excluded) and how many
 * builds of this handle were replayed from a CUDA graph: with "cuda-graphs" on (default), the merge
 * sequence of a tree runs eagerly on its first build, is captured on the second and replayed from
 * the third on (a build is the same launch sequence every time; no counterpart in the reference). */
int ef_hps_build_info(const ef_hps* h, long long* merge_launches, long long* graph_replays);
/* Mixed-precision build (no counterpart in the reference): the same merges with FP32 operators,
 * except the interface LU of the top fp64_levels tree levels (FP64, factors rounded to FP32).  It
 * prepares the tree for the mixed block solver and the server only (ef_hps_mixed_*, ef_server_*);
 * the plain FP64 stages need ef_hps_build.  When both builds exist the mixed solver reads the
 * FP32-built operators. */
int ef_hps_build_mixed(ef_hps* hps, int fp64_levels);

/* Local re-factorisation after a mesh change (no counterpart in the reference; it rebuilds every
 * merge): build `hps`, created on a new mesh of the same domain, patch size and lambda, reusing the
 * operators of every merge node whose subtree is unchanged in the built `old` handle; only the
 * changed nodes (the ancestors of changed leaves) merge.  The operators equal those of
 * ef_hps_build bit for bit.  FISHPACK90 leaves.  `reused` (may be NULL) receives the number of
 * merges copied from `old`. */
int ef_hps_build_from(ef_hps* hps, const ef_hps* old, int* reused);

/* Save a built tree's solve-time operators (every merge node's T, [S | X^-1] and compact H; for
 * FivePointStencil leaves also their coefficients and band LU factors) with its mesh to `path`, and
 * load it back into a new mesh and a built handle that solves bit-identically without re-merging.
 * No counterpart in the reference.  A damaged file returns EF_ERR_INVALID (checksummed payload). */
int ef_hps_save(const ef_hps* hps, const char* path);
int ef_hps_load(const char* path, ef_mesh** mesh_out, ef_hps** hps_out);
/* HPSAlgorithm::upwardsStage (HPSAlgorithm.hpp:225-272) with the load f sampled at leaf cell
 * centres, host array of num_leaves * n * n doubles. */
int ef_hps_upwards(ef_hps* hps, const double* f_host);
/* HPSAlgorithm::solveStage (HPSAlgorithm.hpp:343-445): a, b, r are the boundary condition
 * a u + b du/dn = r sampled at the root face centres, host arrays of 4*M doubles (WESN). */
int ef_hps_solve(ef_hps* hps, const double* a_host, const double* b_host, const double* r_host);
/* HPSAlgorithm::solveStage(patch callback) (HPSAlgorithm.hpp:291-324): the root Dirichlet data
 * g (4*M doubles, host) is given directly. */
int ef_hps_solve_root_dirichlet(ef_hps* hps, const double* g_host);
/* Leaf solutions u (num_leaves * n * n doubles) to host memory (patch.vectorU() of every leaf). */
int ef_hps_get_leaf_u(ef_hps* hps, double* u_host);
/* Root Dirichlet-to-Neumann matrix T (4M x 4M, row-major) and particular Neumann data h (4M). */
int ef_hps_get_root_T(ef_hps* hps, double* T_host);
int ef_hps_get_root_h(ef_hps* hps, double* h_host);
int ef_hps_destroy(ef_hps* hps);

/* Device-resident forms (no host copies; pointers stay valid for the handle's lifetime). */
int ef_hps_device_buffers(ef_hps* hps, double** f_dev, double** u_dev, double** a_dev,
                          double** b_dev, double** r_dev);
/* Device-to-device copy of new inputs into the resident buffers on the handle's stream; any
 * pointer may be NULL (that input is kept).  f: num_leaves*n*n, a/b/r: 4*M doubles. */
int ef_hps_load_device_async(ef_hps* hps, const double* f_dev, const double* a_dev,
                             const double* b_dev, const double* r_dev);
/* upwards + root Dirichlet data + downwards + leaf solves on the resident buffers, without a host
 * synchronisation.  b_is_zero != 0 asserts b == 0 everywhere (Dirichlet root data g = r / a). */
int ef_hps_solve_device_async(ef_hps* hps, int b_is_zero);
int ef_hps_synchronize(ef_hps* hps);

/* ---- Mixed precision, many right-hand sides (no counterpart in the reference) ---------------
 * After ef_hps_build: FP32 copies of the merge operators and leaf tables; each solve runs FP32
 * HPS passes on a block of up to bmax requests and refines them against the exact residual (the
 * 5-point residual of every leaf cell, evaluated in fixed-point integer arithmetic, plus the FP64
 * flux mismatch at every merge interface), so the result converges to the FP64 HPS solution.
 * Dirichlet root data (b == 0) only. */
int ef_hps_mixed_init(ef_hps* hps, int bmax);
/* Root operator of the block solvers (HPSAlgorithm.hpp:402-420 and the thermal driver's Neumann
 * sides, examples/thermal/main.cpp:324-350): a u + b du/dn = r with a and b (4M each, WESN root face
 * centres) fixed and r per request.  With b != 0 the root data become part of the refined state:
 * every pass solves the root condition's residual with (diag a + diag b T_root)^{-1}, factored here
 * in FP64 and applied in FP32; the per-request a arrays of the solve calls are then not read.
 * b == 0 everywhere returns to per-request Dirichlet data.  Applies to the handle's block solvers
 * and lanes until the next ef_hps_mixed_init.  EF_ERR_INVALID when the root matrix is singular. */
/* No counterpart in the reference.  The node-GEMM plan the block solver's autotuner chose (timed
 * once per tree): per node group {level, s, W, H, DOWN}, each code > 0 = FP32 CUDA-core kernel with
 * that K split, < 0 = tcgen05 tensor-core kernel with K split -code.  table: 5 * max_groups ints (or
 * NULL to query the count in *ngroups). */
int ef_hps_mixed_gemm_plan(ef_hps* h, int max_groups, int* table, int* ngroups);
/* No counterpart in the reference.  Sets the node-GEMM plan instead of timing it: codes[3 * i + k]
 * for node group i (the row order of ef_hps_mixed_gemm_plan) and kind k (W, H, DOWN), > 0 the
 * CUDA-core kernel with that K split, 0 its own choice, < 0 the tensor-core kernel with K split
 * -code (needs "tensor-cores" 1 or 2 and a shape it supports).  Block solvers created afterwards
 * (ef_hps_mixed_init) use it.  EF_ERR_INVALID for a wrong group count or an unsupported code. */
int ef_hps_mixed_set_gemm_plan(ef_hps* h, const int* codes, int ngroups);

int ef_hps_mixed_set_root(ef_hps* h, const double* a, const double* b);
/* Resident buffers: f [B][num_leaves*n*n], a and r [B][4M] (root data, a u = r), u [B][...]. */
int ef_hps_mixed_buffers(ef_hps* hps, double** f_dev, double** a_dev, double** r_dev, double** u_dev);
/* 1 + sweeps passes on the first `batch` requests of the resident buffers, no host sync. */
int ef_hps_mixed_solve_async(ef_hps* hps, int batch, int sweeps);
/* Host convenience form: copies the inputs in, solves, copies u out (synchronous). */
int ef_hps_mixed_solve(ef_hps* hps, int batch, int sweeps, const double* f_host, const double* a_host,
                       const double* r_host, double* u_host);
/* Pipelined host form for many blocks: block k (batch[k] <= bmax requests, host arrays f[k], a[k],
 * r[k] in and u[k] out, each laid out as for ef_hps_mixed_solve) runs on lane k mod 3 (lanes share
 * the tree's FP32 operators, each has its own stream and block buffers), so the host copies of two
 * blocks overlap the solve of a third (page-locked host memory keeps the copies asynchronous).
 * Returns when every block's u is on the host. */
int ef_hps_mixed_solve_blocks(ef_hps* hps, int nblocks, const int* batch, int sweeps, const double* const* f_host,
                              const double* const* a_host, const double* const* r_host, double* const* u_host);
/* Device-resident lanes 0..3: lane 0 is the solver of ef_hps_mixed_init (the tree's stream), lanes
 * 1..3 (each set up by the first call for it) share its FP32 operators and run on their own streams,
 * so several blocks can be in flight at once.  Returns the lane's resident buffers (as
 * ef_hps_mixed_buffers) and its stream (a cudaStream_t); a lane >= 1 starts after the work queued on
 * the tree's stream at that call. */
int ef_hps_mixed_lane(ef_hps* hps, int lane, double** f_dev, double** a_dev, double** r_dev, double** u_dev,
                      void** stream);
/* 1 + sweeps passes on the first `batch` requests of the lane's resident buffers, on its stream. */
int ef_hps_mixed_lane_solve_async(ef_hps* hps, int lane, int batch, int sweeps);
/* max |leaf residual| per request before each pass: passes x bmax doubles (synchronous). */
int ef_hps_mixed_residuals(ef_hps* hps, int passes, double* out_host);

/* ---- Instrumentation (the reference's stage timers, EllipticForestApp.hpp:39-137) ------------ */

/* Kernels launched by this library so far (all handles). */
int ef_kernel_launches(long long* count);
/* Per-section CUDA-event timing on the handle's stream (off by default).  A section is one kernel
 * family of one stage step, e.g. "downward" or "leaf_solve"; bytes and flops are the section's
 * algorithmic traffic and FP64 operations. */
int ef_hps_profile_enable(ef_hps* hps, int on);
int ef_hps_profile_count(ef_hps* hps, int* count);
int ef_hps_profile_entry(ef_hps* hps, int i, char* name, int name_len, double* ms,
                         long long* launches, long long* calls, double* bytes, double* flops);
int ef_hps_profile_reset(ef_hps* hps);

/* ---- Single patch (FiniteVolumeSolver::buildD2N / solve / mapD2N) --------------------------- */

/* FiniteVolumeSolver::buildD2N (FiniteVolumeSolver.cpp:355-455) for an n x n patch on
 * [xl,xu] x [yl,yu]; T_host receives 4n x 4n doubles (row-major, WESN). */
int ef_fv_build_d2n(int solver_type, int n, double x_lower, double x_upper, double y_lower,
                    double y_upper, double lambda, double* T_host);
/* FiniteVolumeSolver::solve (FiniteVolumeSolver.cpp:27-290): g (4n, WESN), f (n*n), u (n*n). */
int ef_fv_solve(int solver_type, int n, double x_lower, double x_upper, double y_lower,
                double y_upper, double lambda, const double* g_host, const double* f_host,
                double* u_host);
/* FiniteVolumeSolver::mapD2N (FiniteVolumeSolver.cpp:296-353): h (4n). */
int ef_fv_map_d2n(int solver_type, int n, double x_lower, double x_upper, double y_lower,
                  double y_upper, double lambda, const double* g_host, const double* f_host,
                  double* h_host);

/* FiniteVolumeSolver with solver_type FivePointStencil (FiniteVolumeSolver.cpp:27-223): the same
 * three operations for one patch whose coefficients are sampled as for ef_hps_set_coefficients
 * (alpha n*n, beta 4*n*n, lambda n*n). */
int ef_fv5_build_d2n(int n, double x_lower, double x_upper, double y_lower, double y_upper,
                     const double* alpha, const double* beta, const double* lambda, double* T_host);
int ef_fv5_solve(int n, double x_lower, double x_upper, double y_lower, double y_upper,
                 const double* alpha, const double* beta, const double* lambda, const double* g_host,
                 const double* f_host, double* u_host);
int ef_fv5_map_d2n(int n, double x_lower, double x_upper, double y_lower, double y_upper,
                   const double* alpha, const double* beta, const double* lambda,
                   const double* g_host, const double* f_host, double* h_host);

/* ---- Subtree split across processes ---------------------------------------------------------- */

/* The reference builds and solves one tree over MPI ranks: at the process boundary merge4to1 first
 * broadcasts the children a rank does not own (src/Quadtree.hpp:470-496 merge, :146-148 broadcast of
 * the patch) and split1to4 sends them back down.  Here the split is by subtrees: with 4^level
 * processes, process p builds, upward-passes and solves the subtree under node p of `level` (in
 * z-order) as a tree of its own (ef_mesh_subtree + the usual ef_hps_* calls), and one process
 * runs the top `level` levels on a handle of the full mesh from the gathered level-`level`
 * operators.  Results equal a single-handle build and solve bit for bit.  Transport of T, h and g
 * between processes is the caller's (NCCL, peer copies or host memory).
 *
 * ef_mesh_level_count: number of nodes at `level`.  ef_mesh_subtree: the mesh of the subtree under
 * the index-th node of `level`; its root box is that node's box and every patch box is the full
 * mesh's, bit for bit. */
int ef_mesh_level_count(const ef_mesh* mesh, int level, int* count);
int ef_mesh_subtree(const ef_mesh* mesh, int level, int index, ef_mesh** out);

/* On a handle of the full mesh (every leaf below `level`):
 * ef_hps_split_sizes: 4m for every node of `level` in z-order (the length of its h and g; its T is
 *   4m x 4m, row-major, WESN) -- the root side of the matching subtree handle is m.
 * ef_hps_build_top: the merges of levels level-1 .. 0 (HPSAlgorithm.hpp:120-161 above the split)
 *   from T[k] = root T of subtree k (ef_hps_get_root_T of its handle).
 * ef_hps_upwards_top: the upward pass of levels level-1 .. 0 (HPSAlgorithm.hpp:178-272 above the
 *   split) from h[k] = root h of subtree k after its upwards stage (ef_hps_get_root_h).
 * ef_hps_solve_top: root data a u + b du/dn = r (4M each, as ef_hps_solve), then the downward pass
 *   to `level`: g[k] receives the Dirichlet data of subtree k (4m), which its handle solves with
 *   ef_hps_solve_root_dirichlet.
 * A handle built this way accepts only the *_top calls (others return EF_ERR_STATE) until a
 * regular build stage runs on it. */
int ef_hps_split_sizes(ef_hps* h, int level, int* sizes);
int ef_hps_build_top(ef_hps* h, int level, const double* const* T);
int ef_hps_upwards_top(ef_hps* h, int level, const double* const* hv);
int ef_hps_solve_top(ef_hps* h, int level, const double* a, const double* b, const double* r, double* const* g);

/* ---- Single patch without allocation -------------------------------------------------------- */

/* No counterpart in the reference.  The solve of ef_fv_solve for callers that cannot allocate
 * device memory: plugins inside a host framework that owns all device memory through its own pool
 * and forbids raw allocations, and real-time loops that must not allocate after start-up.  It calls
 * no cudaMalloc, cudaFree or allocating library routine: its scratch (sine basis, eigenvalue table,
 * launch descriptors) lives in a fixed device array of about 66 KB that every GPU loading this
 * library holds until exit, which limits n to 64 (larger n returns EF_ERR_INVALID).  g_dev (4n),
 * f_dev (n*n, NULL = zero load) and u_dev (n*n) are device pointers owned by the caller; the work
 * is queued on cuda_stream (NULL = default stream) and the call returns without synchronising.
 * The first call on each device (and the first after a cudaDeviceReset) looks up the array's
 * device address with that device current; make that first call before any stream capture.  All
 * calls share the array, so calls whose work overlaps on the GPU race. */
int ef_fv_solve_noalloc(int solver_type, int n, double x_lower, double x_upper, double y_lower,
                        double y_upper, double lambda, const double* g_dev, const double* f_dev,
                        double* u_dev, void* cuda_stream);

/* ---- Serving loop over several resident trees ------------------------------------------------ */

/* No counterpart in the reference (its drivers solve one right-hand side per call).  A server keeps
 * several built trees resident and answers requests (tree index, load f, root data a u = r) with
 * the batched mixed-precision solver (results refined to the FP64 HPS solution by `sweeps` FP64
 * sweeps).  Every tree gets up to lanes_per_tree lanes -- a block solver of up to bmax[t] requests
 * with its own CUDA stream; lanes beyond the first of each tree are only created while the device
 * memory of all lanes stays within hbm_budget_bytes (<= 0: no limit).  A scheduler thread forms a
 * block from every request of a tree that has arrived whenever one of its lanes is free
 * (continuous batching) and overlaps the blocks of different lanes and trees on the GPU.  A
 * request's result does not depend on the other requests of its block.  The trees must outlive
 * the server and must not be rebuilt while it exists. */
typedef struct ef_server ef_server;
int ef_server_create(ef_hps* const* trees, const int* bmax, int ntrees, int lanes_per_tree,
                     long long hbm_budget_bytes, int sweeps, ef_server** out);
/* refinement sweeps of tree t's blocks from the next block on (creation value: sweeps) */
int ef_server_set_sweeps(ef_server* server, int tree, int sweeps);
/* Root operator a u + b du/dn = r of one tree's lanes, as ef_hps_mixed_set_root, for the requests
 * submitted afterwards (their a is then not read while b != 0).  The tree must have no request in
 * flight (EF_ERR_INVALID otherwise); returns once the scheduler has put it in place. */
int ef_server_set_root(ef_server* server, int tree, const double* a, const double* b);
/* lanes created for tree t (after the budget) and device bytes held by all lanes */
int ef_server_info(ef_server* server, int tree, int* lanes, long long* device_bytes);
/* f (leaves*n*n), a and r (4M, WESN root face centres) and u (leaves*n*n) are host arrays that
 * must stay valid until the request completes; page-locked memory keeps the copies asynchronous. */
int ef_server_submit(ef_server* server, int tree, const double* f, const double* a, const double* r,
                     double* u, long long* id);
/* done = 1 and latency_s = seconds from submit to the result in u, or done = 0 (pending / time-out).
 * A completed id is reported once. */
int ef_server_poll(ef_server* server, long long id, int* done, double* latency_s);
int ef_server_wait(ef_server* server, long long id, double timeout_s, int* done, double* latency_s);
int ef_server_stats(ef_server* server, long long* submitted, long long* completed, long long* blocks,
                    long long* max_block);
/* waits for the requests already submitted, then frees the lanes */
int ef_server_destroy(ef_server* server);

#ifdef __cplusplus
}
#endif

#endif /* ELLIPTICFOREST_GB300_H_ */
