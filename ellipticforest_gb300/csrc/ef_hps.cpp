// GB300 HPS solver: plan, device arena and the level-by-level stage drivers.
//
// Stage order follows src/HPSAlgorithm.hpp: buildStage (:120-161, leaf DtN + post-order merges),
// upwardsStage (:178-272, leaf particular Neumann data + upwards4to1), solveStage (:343-445, root
// Dirichlet data, pre-order split1to4, leafSolve).  Each tree level is processed as a whole; the
// merges of one level are independent, so the result equals the reference's post-order traversal.
#include "ef_hps.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>

namespace efgb {

namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

int ilog2_exact(int v) {
    int k = 0;
    while ((1 << k) < v) ++k;
    if ((1 << k) != v) throw std::invalid_argument("patch size ratio is not a power of two");
    return k;
}

// Carves the device arena.  Run once dry to measure, once to assign.
struct Carver {
    char* base = nullptr;
    size_t off = 0;
    template <class T>
    T* get(size_t count) {
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += align_up(std::max<size_t>(count, 1) * sizeof(T));
        return p;
    }
};

}  // namespace

void leaf_tables(int n, double dx, double dy, double lambda, double* V, double* Dinv) {
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
            const double c = (k == n - 1) ? std::sqrt(1.0 / n) : std::sqrt(2.0 / n);
            V[i * n + k] = c * std::sin(M_PI * (k + 1) * (i + 0.5) / n);
        }
    for (int k = 0; k < n; ++k)
        for (int l = 0; l < n; ++l) {
            const double sx = std::sin(M_PI * (k + 1) / (2.0 * n));
            const double sy = std::sin(M_PI * (l + 1) / (2.0 * n));
            const double mux = -(4.0 / (dx * dx)) * sx * sx;
            const double muy = -(4.0 / (dy * dy)) * sy * sy;
            Dinv[k * n + l] = 1.0 / (mux + muy + lambda);
        }
}

void Hps::check(cudaError_t e, const char* what) {
    if (e != cudaSuccess)
        throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

Hps::Hps(const Mesh& mesh, int solver_type, double lambda, bool cache_operators)
    : mesh_(mesh), solver_type_(solver_type), lambda_(lambda), cache_ops_(cache_operators) {
    if (mesh.nx != mesh.ny) throw std::invalid_argument("patches must be square (nx == ny)");
    if (mesh.nx < 2 || mesh.nx > 64) throw std::invalid_argument("leaf patch size must be in [2, 64]");
    if (solver_type != SOLVER_FISHPACK90 && solver_type != SOLVER_FIVE_POINT)
        throw std::invalid_argument("unknown solver type");
    n_ = mesh.nx;
    plan();
    allocate();
    upload_tables();
}

Hps::~Hps() {
    for (auto& m : marks_) { ev_free_.push_back(m.a); ev_free_.push_back(m.b); }
    for (cudaEvent_t e : ev_free_) cudaEventDestroy(e);
    if (arena_) cudaFree(arena_);
    if (arena32_) cudaFree(arena32_);
    if (d_rootA_) cudaFree(d_rootA_);
}

cudaEvent_t Hps::ev_get() {
    if (!ev_free_.empty()) {
        cudaEvent_t e = ev_free_.back();
        ev_free_.pop_back();
        return e;
    }
    cudaEvent_t e;
    check(cudaEventCreate(&e), "cudaEventCreate");
    return e;
}

void Hps::pb(const char* name, cudaStream_t st) {
    if (!prof_) return;
    int idx = -1;
    for (size_t i = 0; i < stats_.size(); ++i)
        if (stats_[i].name == name) { idx = int(i); break; }
    if (idx < 0) {
        idx = int(stats_.size());
        stats_.push_back(ProfStat{name});
    }
    open_stat_ = idx;
    open_ev_ = ev_get();
    open_launch0_ = g_kernel_launches.load();
    check(cudaEventRecord(open_ev_, st), "cudaEventRecord");
}

void Hps::pe(double bytes, double flops, cudaStream_t st) {
    if (!prof_ || open_stat_ < 0) return;
    cudaEvent_t b = ev_get();
    check(cudaEventRecord(b, st), "cudaEventRecord");
    marks_.push_back(Mark{open_stat_, open_ev_, b, g_kernel_launches.load() - open_launch0_, bytes, flops});
    open_stat_ = -1;
}

const std::vector<Hps::ProfStat>& Hps::profile_read() {
    check(cudaDeviceSynchronize(), "profile sync");  // sections may sit on several streams
    for (auto& m : marks_) {
        float ms = 0;
        check(cudaEventElapsedTime(&ms, m.a, m.b), "cudaEventElapsedTime");
        ProfStat& ps = stats_[m.stat];
        ps.ms += ms;
        ps.launches += m.launches;
        ps.calls += 1;
        ps.bytes += m.bytes;
        ps.flops += m.flops;
        ev_free_.push_back(m.a);
        ev_free_.push_back(m.b);
    }
    marks_.clear();
    return stats_;
}

void Hps::profile_reset() {
    profile_read();
    stats_.clear();
}

void Hps::plan() {
    const int N = int(mesh_.nodes.size());
    nodes_.assign(N, NodeDev());
    for (int id = N - 1; id >= 0; --id) {  // reverse pre-order: children first
        const MeshNode& mn = mesh_.nodes[id];
        NodeDev& nd = nodes_[id];
        if (mn.leaf()) {
            nd.nx = n_;
        } else {
            int mn_side = 1 << 30;
            for (int c = 0; c < 4; ++c) mn_side = std::min(mn_side, nodes_[mn.child[c]].nx);
            for (int c = 0; c < 4; ++c) {
                NodeDev& ch = nodes_[mn.child[c]];
                ch.ncoarsen = ilog2_exact(ch.nx / mn_side);
                if (ch.ncoarsen > 0 && (ch.nx >> (ch.ncoarsen - 1)) < 8)
                    throw std::invalid_argument("coarsening needs patches of at least 4 cells");
            }
            nd.s = mn_side;
            nd.nx = 2 * mn_side;  // mergePatch_ (HPSAlgorithm.hpp:1004-1009)
        }
        nd.size = nd.nx;
    }
    for (int id = 0; id < N; ++id) nodes_[id].size = nodes_[id].nx >> nodes_[id].ncoarsen;

    // leaf types keyed by the exact grid spacing (FISHPACK90: lambda is global)
    std::map<std::pair<uint64_t, uint64_t>, int> key2type;
    for (int l : mesh_.leaves) {
        const MeshNode& mn = mesh_.nodes[l];
        const double dx = (mn.xu - mn.xl) / n_, dy = (mn.yu - mn.yl) / n_;
        uint64_t kx, ky;
        std::memcpy(&kx, &dx, 8);
        std::memcpy(&ky, &dy, 8);
        auto it = key2type.find({kx, ky});
        int t;
        if (solver_type_ == SOLVER_FIVE_POINT) {
            // variable coefficients: every leaf has its own operator
            t = int(types_.size());
            types_.push_back(LeafTypeHost{n_, dx, dy, nullptr});
        } else if (it == key2type.end()) {
            t = int(types_.size());
            types_.push_back(LeafTypeHost{n_, dx, dy, nullptr});
            key2type[{kx, ky}] = t;
        } else {
            t = it->second;
        }
        nodes_[l].leaf_type = t;
    }
    (void)cache_ops_;

    // groups per (level, s), deepest level first
    std::map<std::pair<int, int>, int> gidx;
    for (int id = 0; id < N; ++id) {
        const MeshNode& mn = mesh_.nodes[id];
        if (mn.leaf()) continue;
        auto key = std::make_pair(-mn.level, nodes_[id].s);
        if (!gidx.count(key)) gidx[key] = 0;
    }
    int gi = 0;
    for (auto& kv : gidx) kv.second = gi++;
    groups_.assign(gidx.size(), Group());
    for (auto& kv : gidx) {
        groups_[kv.second].level = -kv.first.first;
        groups_[kv.second].s = kv.first.second;
    }
    for (int id = 0; id < N; ++id) {
        const MeshNode& mn = mesh_.nodes[id];
        if (mn.leaf()) continue;
        groups_[gidx[{-mn.level, nodes_[id].s}]].nodes.push_back(id);
    }
}

void Hps::allocate() {
    const int N = int(nodes_.size());
    const int L = int(mesh_.leaves.size());
    const int nn = n_ * n_;
    const int M = nodes_[0].nx;

    // resample steps: (level, step, nf) -> list of node ids
    std::map<std::tuple<int, int, int>, std::vector<int>> tmap, gmap;
    for (int id = 0; id < N; ++id) {
        const NodeDev& nd = nodes_[id];
        for (int t = 0; t < nd.ncoarsen; ++t) {
            tmap[{mesh_.nodes[id].level, t, nd.nx >> t}].push_back(id);
            const int cf = nd.ncoarsen - (t + 1);
            gmap[{mesh_.nodes[id].level, t, nd.nx >> cf}].push_back(id);
        }
    }

    const bool fp = solver_type_ == SOLVER_FIVE_POINT;
    auto layout = [&](Carver& cv) {
        for (auto& ty : types_) ty.T = cv.get<double>(size_t(16) * nn);
        if (fp) {
            // per leaf: coefficients [alpha | beta W,E,S,N | lambda], band LU, boundary coefficients
            d_coef_ = cv.get<double>(size_t(L) * 6 * nn);
            fp_band_.assign(L, nullptr);
            fp_bcoef_.assign(L, nullptr);
            for (int k = 0; k < L; ++k) {
                fp_band_[k] = cv.get<double>(size_t(nn) * (2 * n_ + 1));
                fp_bcoef_[k] = cv.get<double>(4 * size_t(n_));
            }
            d_fpinfo_ = cv.get<int>(L);
            d_fp_ = cv.get<FpLeaf>(L);
        } else {
            d_V_ = cv.get<double>(size_t(types_.size()) * nn);
            d_Dinv_ = cv.get<double>(size_t(types_.size()) * nn);
        }
        for (int id = 0; id < N; ++id) {
            NodeDev& nd = nodes_[id];
            const MeshNode& mn = mesh_.nodes[id];
            nd.Tsteps.clear(); nd.hsteps.clear(); nd.gsteps.clear();
            if (mn.leaf()) {
                nd.T = types_[nd.leaf_type].T;
                nd.h = cv.get<double>(4 * n_);
                nd.g = cv.get<double>(4 * n_);
            } else {
                const size_t s = nd.s;
                nd.T = cv.get<double>(64 * s * s);
                nd.X = cv.get<double>(16 * s * s);
                nd.RHS = cv.get<double>(48 * s * s);
                nd.H = cv.get<double>(16 * s * s);
                nd.piv = cv.get<int>(4 * s);
                nd.perm = cv.get<int>(4 * s);
                nd.h = cv.get<double>(8 * s);
                nd.w = cv.get<double>(4 * s);
                nd.hd = cv.get<double>(4 * s);
                nd.g = cv.get<double>(4 * size_t(nd.size));
            }
            for (int t = 0; t < nd.ncoarsen; ++t) {
                const size_t nc = size_t(nd.nx >> t) / 2;
                nd.Tsteps.push_back(cv.get<double>(16 * nc * nc));
                nd.hsteps.push_back(cv.get<double>(4 * nc));
                const int cf = nd.ncoarsen - (t + 1);
                nd.gsteps.push_back(cv.get<double>(4 * size_t(nd.nx >> cf)));
            }
            nd.Tc = nd.ncoarsen ? nd.Tsteps.back() : nd.T;
            nd.hc = nd.ncoarsen ? nd.hsteps.back() : nd.h;
            nd.gf = nd.ncoarsen ? nd.gsteps.back() : nd.g;
        }
        d_f_ = cv.get<double>(size_t(L) * nn);
        d_u_ = cv.get<double>(size_t(L) * nn);
        d_bca_ = cv.get<double>(4 * size_t(M));
        d_bcb_ = cv.get<double>(4 * size_t(M));
        d_bcr_ = cv.get<double>(4 * size_t(M));
        d_types_ = cv.get<LeafType>(types_.size());
        nitems_dtn_ = int(types_.size()) * 4 * n_;
        d_items_dtn_ = cv.get<LeafItem>(nitems_dtn_);
        d_items_neu_ = cv.get<LeafItem>(L);
        d_items_solve_ = cv.get<LeafItem>(L);
        for (auto& g : groups_) {
            const int cnt = int(g.nodes.size());
            g.d_items = cv.get<MergeItem>(cnt);
            g.d_X = cv.get<double*>(cnt);
            g.d_RHS = cv.get<double*>(cnt);
            g.d_H = cv.get<double*>(cnt);
            g.d_T = cv.get<double*>(cnt);
            g.d_piv = cv.get<int*>(cnt);
            g.d_perm = cv.get<int*>(cnt);
            g.d_info = cv.get<int>(cnt);
            g.d_gA = cv.get<const double*>(8 * cnt);
            g.d_gB = cv.get<const double*>(8 * cnt);
            g.d_gB2 = cv.get<const double*>(8 * cnt);
            g.d_gC = cv.get<double*>(8 * cnt);
        }
        tsteps_.clear(); hsteps_.clear(); gsteps_.clear();
        for (auto& kv : tmap) {
            ResampleStep r;
            r.level = std::get<0>(kv.first);
            r.nf = std::get<2>(kv.first);
            r.count = int(kv.second.size());
            r.d_in = cv.get<const double*>(r.count);
            r.d_out = cv.get<double*>(r.count);
            tsteps_.push_back(r);
            ResampleStep h = r;
            h.d_in = cv.get<const double*>(r.count);
            h.d_out = cv.get<double*>(r.count);
            hsteps_.push_back(h);
        }
        for (auto& kv : gmap) {
            ResampleStep r;
            r.level = std::get<0>(kv.first);
            r.nf = std::get<2>(kv.first);
            r.count = int(kv.second.size());
            r.d_in = cv.get<const double*>(r.count);
            r.d_out = cv.get<double*>(r.count);
            gsteps_.push_back(r);
        }
    };
    Carver dry;
    layout(dry);
    arena_bytes_ = dry.off;
    check(cudaMalloc(&arena_, arena_bytes_), "cudaMalloc(arena)");
    Carver real;
    real.base = arena_;
    layout(real);

    // remember which nodes each resample step covers (same iteration order as the layout)
    step_nodes_t_.clear();
    step_nodes_g_.clear();
    for (auto& kv : tmap) step_nodes_t_.push_back(kv.second);
    for (auto& kv : gmap) step_nodes_g_.push_back(kv.second);
    step_index_t_.clear();
    step_index_g_.clear();
    for (auto& kv : tmap) step_index_t_.push_back(std::get<1>(kv.first));
    for (auto& kv : gmap) step_index_g_.push_back(std::get<1>(kv.first));
}

void Hps::upload_tables() {
    const int L = int(mesh_.leaves.size());
    const int nn = n_ * n_;
    // zero the whole arena once (h of the root must read as 0 before any upward pass)
    check(cudaMemsetAsync(arena_, 0, arena_bytes_, st_), "memset(arena)");

    if (solver_type_ == SOLVER_FIVE_POINT) {
        // one variable-coefficient operator per leaf (type index == leaf index)
        std::vector<FpLeaf> fl(L);
        for (int k = 0; k < L; ++k) {
            const double* c = d_coef_ + size_t(k) * 6 * nn;
            fl[k] = FpLeaf{n_, types_[k].dx, types_[k].dy, c, c + nn, c + 5 * nn, fp_band_[k], fp_bcoef_[k],
                           d_fpinfo_ + k};
        }
        check(upload_sync(st_, d_fp_, fl.data(), fl.size() * sizeof(FpLeaf)), "upload fp leaves");
    } else {
        // leaf types: sine basis and inverse eigenvalue table
        std::vector<LeafType> hty(types_.size());
        std::vector<double> V(nn), Dinv(nn);
        for (size_t t = 0; t < types_.size(); ++t) {
            leaf_tables(n_, types_[t].dx, types_[t].dy, lambda_, V.data(), Dinv.data());
            check(upload_sync(st_, d_V_ + t * nn, V.data(), nn * 8), "upload V");
            check(upload_sync(st_, d_Dinv_ + t * nn, Dinv.data(), nn * 8), "upload Dinv");
            hty[t] = LeafType{n_, types_[t].dx, types_[t].dy, d_V_ + t * nn, d_Dinv_ + t * nn};
        }
        check(upload_sync(st_, d_types_, hty.data(), hty.size() * sizeof(LeafType)),
              "upload types");
        if (n_ == 16) leaf_set_basis16(st_);
    }

    std::vector<LeafItem> items;
    for (size_t t = 0; t < types_.size(); ++t)
        for (int u = 0; u < 4 * n_; ++u) items.push_back(LeafItem{int(t), u, nullptr, nullptr, types_[t].T});
    check(upload_sync(st_, d_items_dtn_, items.data(), items.size() * sizeof(LeafItem)),
          "upload dtn items");
    items.clear();
    for (int k = 0; k < L; ++k) {
        const NodeDev& nd = nodes_[mesh_.leaves[k]];
        items.push_back(LeafItem{nd.leaf_type, 0, d_f_ + size_t(k) * nn, nullptr, nd.h});
    }
    check(upload_sync(st_, d_items_neu_, items.data(), items.size() * sizeof(LeafItem)),
          "upload neumann items");
    items.clear();
    for (int k = 0; k < L; ++k) {
        const NodeDev& nd = nodes_[mesh_.leaves[k]];
        items.push_back(LeafItem{nd.leaf_type, 0, d_f_ + size_t(k) * nn, nd.g, d_u_ + size_t(k) * nn});
    }
    check(upload_sync(st_, d_items_solve_, items.data(), items.size() * sizeof(LeafItem)),
          "upload solve items");

    for (auto& g : groups_) {
        const int cnt = int(g.nodes.size());
        std::vector<MergeItem> mi(cnt);
        std::vector<double*> X(cnt), R(cnt), H(cnt), T(cnt);
        std::vector<int*> P(cnt), Q(cnt);
        for (int i = 0; i < cnt; ++i) {
            const int id = g.nodes[i];
            const NodeDev& nd = nodes_[id];
            const MeshNode& mn = mesh_.nodes[id];
            MergeItem& m = mi[i];
            for (int c = 0; c < 4; ++c) {
                const NodeDev& ch = nodes_[mn.child[c]];
                m.Tc[c] = ch.Tc;
                m.hc[c] = ch.hc;
                m.gc[c] = ch.g;
            }
            m.X = nd.X; m.piv = nd.piv; m.perm = nd.perm; m.RHS = nd.RHS; m.H = nd.H; m.T = nd.T;
            m.h = nd.h; m.w = nd.w; m.gf = nd.gf; m.hd = nd.hd;
            X[i] = nd.X; R[i] = nd.RHS; H[i] = nd.H; T[i] = nd.T; P[i] = nd.piv; Q[i] = nd.perm;
        }
        check(upload_sync(st_, g.d_items, mi.data(), cnt * sizeof(MergeItem)), "items");
        check(upload_sync(st_, g.d_X, X.data(), cnt * sizeof(double*)), "X");
        check(upload_sync(st_, g.d_RHS, R.data(), cnt * sizeof(double*)), "RHS");
        check(upload_sync(st_, g.d_H, H.data(), cnt * sizeof(double*)), "H");
        check(upload_sync(st_, g.d_T, T.data(), cnt * sizeof(double*)), "T");
        check(upload_sync(st_, g.d_piv, P.data(), cnt * sizeof(int*)), "piv");
        check(upload_sync(st_, g.d_perm, Q.data(), cnt * sizeof(int*)), "perm");
        // split GEMM tables: row block b of the parent's WESN exterior belongs to child c(b)
        // (W: alpha, gamma; E: beta, omega; S: alpha, beta; N: gamma, omega), whose interfaces are
        // alpha: I0, I2; beta: I1, I2; gamma: I0, I3; omega: I1, I3.
        {
            static const int cb[8] = {0, 2, 1, 3, 0, 1, 2, 3};
            static const int ia[4] = {0, 1, 0, 1}, ib[4] = {2, 2, 3, 3};
            const size_t sz = size_t(g.s);
            std::vector<const double*> gA(8 * cnt), gB(8 * cnt), gB2(8 * cnt);
            std::vector<double*> gC(8 * cnt);
            for (int i = 0; i < cnt; ++i) {
                const NodeDev& nd = nodes_[g.nodes[i]];
                for (int b = 0; b < 8; ++b) {
                    const int c = cb[b];
                    gA[8 * i + b] = nd.H + size_t(b) * sz * 2 * sz;
                    gB[8 * i + b] = nd.RHS + size_t(ia[c]) * sz * 12 * sz;
                    gB2[8 * i + b] = nd.RHS + size_t(ib[c]) * sz * 12 * sz;
                    gC[8 * i + b] = nd.T + size_t(b) * sz * 8 * sz;
                }
            }
            check(upload_sync(st_, g.d_gA, gA.data(), gA.size() * sizeof(void*)), "gA");
            check(upload_sync(st_, g.d_gB, gB.data(), gB.size() * sizeof(void*)), "gB");
            check(upload_sync(st_, g.d_gB2, gB2.data(), gB2.size() * sizeof(void*)), "gB2");
            check(upload_sync(st_, g.d_gC, gC.data(), gC.size() * sizeof(void*)), "gC");
        }
    }
    for (size_t k = 0; k < tsteps_.size(); ++k) {
        const int t = step_index_t_[k];
        std::vector<const double*> in, hin;
        std::vector<double*> out, hout;
        for (int id : step_nodes_t_[k]) {
            const NodeDev& nd = nodes_[id];
            in.push_back(t == 0 ? nd.T : nd.Tsteps[t - 1]);
            out.push_back(nd.Tsteps[t]);
            hin.push_back(t == 0 ? nd.h : nd.hsteps[t - 1]);
            hout.push_back(nd.hsteps[t]);
        }
        const size_t c = in.size();
        check(upload_sync(st_, tsteps_[k].d_in, in.data(), c * sizeof(void*)), "tin");
        check(upload_sync(st_, tsteps_[k].d_out, out.data(), c * sizeof(void*)), "tout");
        check(upload_sync(st_, hsteps_[k].d_in, hin.data(), c * sizeof(void*)), "hin");
        check(upload_sync(st_, hsteps_[k].d_out, hout.data(), c * sizeof(void*)), "hout");
    }
    for (size_t k = 0; k < gsteps_.size(); ++k) {
        const int t = step_index_g_[k];
        std::vector<const double*> in;
        std::vector<double*> out;
        for (int id : step_nodes_g_[k]) {
            const NodeDev& nd = nodes_[id];
            in.push_back(t == 0 ? nd.g : nd.gsteps[t - 1]);
            out.push_back(nd.gsteps[t]);
        }
        const size_t c = in.size();
        check(upload_sync(st_, gsteps_[k].d_in, in.data(), c * sizeof(void*)), "gin");
        check(upload_sync(st_, gsteps_[k].d_out, out.data(), c * sizeof(void*)), "gout");
    }
    check(cudaStreamSynchronize(st_), "upload sync");
}

void Hps::leaf_run(int mode, const LeafItem* items, int nitems) {
    if (solver_type_ == SOLVER_FIVE_POINT) fp_solve(st_, mode, d_fp_, items, nitems, n_);
    else leaf_eigen(st_, mode, d_types_, items, nitems, n_);
}

void Hps::set_coefficients(const double* alpha, const double* beta, const double* lambda) {
    if (solver_type_ != SOLVER_FIVE_POINT)
        throw std::invalid_argument("leaf coefficients apply to the FivePointStencil solver only");
    const size_t nn = size_t(n_) * n_;
    const int L = num_leaves();
    for (int k = 0; k < L; ++k) {
        double* c = d_coef_ + size_t(k) * 6 * nn;
        check(cudaMemcpyAsync(c, alpha + k * nn, nn * 8, cudaMemcpyHostToDevice, st_), "coef alpha");
        check(cudaMemcpyAsync(c + nn, beta + k * 4 * nn, 4 * nn * 8, cudaMemcpyHostToDevice, st_), "coef beta");
        check(cudaMemcpyAsync(c + 5 * nn, lambda + k * nn, nn * 8, cudaMemcpyHostToDevice, st_), "coef lambda");
    }
    check(cudaStreamSynchronize(st_), "coef sync");
    coef_set_ = true;
    built_ = false;
}

void Hps::build_leaf_types() {
    const double n = n_;
    leaf_singular_ = 0;
    if (solver_type_ == SOLVER_FIVE_POINT) {
        if (!coef_set_) throw std::invalid_argument("FivePointStencil: leaf coefficients were not set");
        const double L = num_leaves(), N = n * n;
        check(cudaMemsetAsync(d_fpinfo_, 0, num_leaves() * sizeof(int), st_), "memset fp info");
        pb("leaf_factor");
        fp_factor(st_, d_fp_, num_leaves(), n_);
        pe(L * 8 * (6 * N + N * (2 * n + 1)), L * 2.0 * N * n * n);
        pb("leaf_dtn");
        leaf_run(LEAF_DTN_COLUMN, d_items_dtn_, nitems_dtn_);
        pe(double(types_.size()) * 16 * n * n * 8, double(nitems_dtn_) * (6 * n * n * n + 8 * n * n));
        return;
    }
    // one DtN per distinct leaf geometry, by a pivoted dense LU of its 5-point operator
    std::vector<double> dx, dy;
    std::vector<double*> T;
    for (const auto& ty : types_) {
        dx.push_back(ty.dx);
        dy.push_back(ty.dy);
        T.push_back(ty.T);
    }
    const double nn = n * n, nt = double(types_.size());
    pb("leaf_dtn");
    leaf_singular_ = leaf_dtn_lu(st_, n_, lambda_, dx, dy, T);
    pe(nt * 8 * (2 * nn * nn + 2 * nn * 4 * n + 16 * n * n),
       nt * (2.0 / 3.0 * nn * nn * nn + 2.0 * nn * nn * 4 * n));
}

void Hps::build() {
    root_lu_valid_ = false;
    top_level_ = -1;
    build_leaf_types();
    // the merges of every level (a fixed launch sequence for this tree) replay as a CUDA graph from
    // the third build on (first eager, second captured); the leaf DtN maps above stay eager
    const long long l0 = g_kernel_launches.load();
    graph_build_.run(st_, 1, graphs_ && !prof_, [&] { merge_levels(mesh_.max_level - 1); });
    build_launches_ = g_kernel_launches.load() - l0;
    check(cudaGetLastError(), "build launch");
    check(cudaStreamSynchronize(st_), "build sync");
    singular_ = count_singular(mesh_.max_level) + leaf_singular_;
    if (solver_type_ == SOLVER_FIVE_POINT) {
        std::vector<int> info(num_leaves());
        check(cudaMemcpy(info.data(), d_fpinfo_, info.size() * sizeof(int), cudaMemcpyDeviceToHost), "fp info");
        indefinite_ = 0;
        for (int v : info) {
            singular_ += (v > 0);
            indefinite_ += (v < 0);
        }
    }
    built_ = true;
}

// every merge of the tree levels top .. 0, deepest first (HPSAlgorithm.hpp:497-518 per node): the
// children's T of level top + 1 must be in place
void Hps::merge_levels(int top) {
    for (int lvl = top; lvl >= 0; --lvl) {
        for (size_t k = 0; k < tsteps_.size(); ++k)
            if (tsteps_[k].level == lvl + 1) {
                const double nf = tsteps_[k].nf, cnt = tsteps_[k].count;
                pb("coarsen_T");
                coarsen_T(st_, tsteps_[k].d_in, tsteps_[k].d_out, tsteps_[k].count, tsteps_[k].nf);
                pe(cnt * 8 * (16 * nf * nf + 4 * nf * nf), cnt * 4 * nf * nf * 10);
            }
        for (auto& g : groups_) {
            if (g.level != lvl) continue;
            const int cnt = int(g.nodes.size()), s = g.s, m = 4 * s;
            const double c = cnt, dm = m;
            pb("gather_xht");
            merge_gather_xht(st_, g.d_items, cnt, s);
            pe(c * 8 * (dm * dm + 2 * dm * dm + 4 * dm * dm) * 1.5, 0);
            check(cudaMemsetAsync(g.d_info, 0, cnt * sizeof(int), st_), "memset info");
            pb("getrf");
            dgetrf_batched(st_, m, g.d_X, m, g.d_piv, g.d_info, cnt);
            piv_to_perm(st_, m, g.d_piv, g.d_perm, cnt);
            pe(c * 8 * 2 * dm * dm, c * 2.0 / 3.0 * dm * dm * dm);
            pb("gather_rhs");
            merge_gather_rhs(st_, g.d_items, cnt, s);
            pe(c * 8 * (3 * dm * dm + dm * dm), 0);
            pb("lu_solve");
            dlu_solve_permuted(st_, m, 3 * m, (const double* const*)g.d_X, m, g.d_RHS, 3 * m, cnt);
            pe(c * 8 * (dm * dm + 2 * 3 * dm * dm), c * 2.0 * dm * dm * 3 * dm);
            // T = T_LHS + H S  (HPSAlgorithm.hpp:940-968), S = first 8s columns of RHS; H's zero
            // blocks are skipped: each s-row block of T takes K = 2s (its child's two interfaces)
            pb("gemm_T");
            GemmArgs ga{g.d_gA, 0, 2 * s, g.d_gB, 0, 3 * m, g.d_gC, 0, 2 * m, g.d_gB2, 0, s};
            dgemm_batched(st_, s, 2 * m, 2 * s, 1.0, ga, 1.0, 8 * cnt);
            pe(c * 8 * (dm * dm / 2 + dm * 2 * dm + 2 * 4 * dm * dm), c * 2.0 * (2 * dm) * (2 * dm) * (dm / 2));
        }
    }
}

// interface LUs with a zero pivot among the merges of the levels below `below` (synchronous)
int Hps::count_singular(int below) {
    int bad = 0;
    for (auto& g : groups_) {
        if (g.level >= below) continue;
        std::vector<int> info(g.nodes.size());
        check(cudaMemcpy(info.data(), g.d_info, info.size() * sizeof(int), cudaMemcpyDeviceToHost), "info");
        for (int v : info) bad += (v != 0);
    }
    return bad;
}

void Hps::upwards() {
    const double L = num_leaves(), n = n_;
    pb("leaf_neumann");
    leaf_run(LEAF_NEUMANN, d_items_neu_, num_leaves());
    pe(L * 8 * (n * n + 4 * n), L * (6 * n * n * n + 8 * n * n));
    if (homogeneous_) return;
    upward_levels(mesh_.max_level - 1);
}

// upwards4to1 (HPSAlgorithm.hpp:529-551) for the levels top .. 0: the children's h of level top + 1
// must be in place
void Hps::upward_levels(int top) {
    for (int lvl = top; lvl >= 0; --lvl) {
        for (size_t k = 0; k < hsteps_.size(); ++k)
            if (hsteps_[k].level == lvl + 1) {
                pb("coarsen_h");
                coarsen_vec(st_, hsteps_[k].d_in, hsteps_[k].d_out, hsteps_[k].count, hsteps_[k].nf);
                pe(double(hsteps_[k].count) * 8 * 6 * hsteps_[k].nf, double(hsteps_[k].count) * 4 * hsteps_[k].nf);
            }
        for (auto& g : groups_) {
            if (g.level != lvl) continue;
            const double c = double(g.nodes.size()), s = g.s;
            pb("upward_w");
            upward_hdiff(st_, g.d_items, int(c), g.s);
            upward_w(st_, g.d_items, int(c), g.s);
            pe(c * 8 * (16 * s * s + 8 * s + 4 * s), c * 2 * 16 * s * s);
            pb("upward_h");
            upward_h(st_, g.d_items, int(c), g.s);
            pe(c * 8 * (16 * s * s + 4 * s + 8 * s + 8 * s), c * 2 * 16 * s * s);  // compact H
        }
    }
}

void Hps::root_from_bc() {
    const int m = 4 * nodes_[0].nx;
    // The caller tells whether b is identically zero through bc_general_.
    if (!bc_general_) {
        pb("root_diag");
        root_diag(st_, m, d_bca_, d_bcb_, d_bcr_, nodes_[0].h, nodes_[0].g);
        pe(8.0 * 5 * m, 3.0 * m);
        return;
    }
    pb("root_general");
    if (!d_rootA_) {
        const size_t bytes = align_up(size_t(m) * m * 8) + 3 * align_up(size_t(m) * 8) +
                             2 * align_up(size_t(m) * 4) + 2 * align_up(sizeof(int)) + 4 * align_up(sizeof(void*));
        check(cudaMalloc(&d_rootA_, bytes), "cudaMalloc(root)");
        Carver cv;
        cv.base = reinterpret_cast<char*>(d_rootA_);
        cv.get<double>(size_t(m) * m);
        d_rootrhs_ = cv.get<double>(m);
        d_rootpiv_ = cv.get<int>(m);
        d_rootperm_ = cv.get<int>(m);
        d_rootinfo_ = cv.get<int>(1);
        d_rootflag_ = cv.get<int>(1);
        d_roota_ = cv.get<double>(m);
        d_rootb_ = cv.get<double>(m);
        d_rootA_arr_ = cv.get<double*>(1);
        d_rootrhs_arr_ = cv.get<double*>(1);
        d_rootpiv_arr_ = cv.get<int*>(1);
        d_rootperm_arr_ = cv.get<int*>(1);
        check(upload_sync(st_, d_rootA_arr_, &d_rootA_, sizeof(void*)), "root arr");
        check(upload_sync(st_, d_rootrhs_arr_, &d_rootrhs_, sizeof(void*)), "root arr");
        check(upload_sync(st_, d_rootpiv_arr_, &d_rootpiv_, sizeof(void*)), "root arr");
        check(upload_sync(st_, d_rootperm_arr_, &d_rootperm_, sizeof(void*)), "root arr");
    }
    // g = (diag(a) + diag(b) T)^{-1} (r - diag(b) h)   (HPSAlgorithm.hpp:402-420).  The reference
    // re-assembles and re-factors the 4M x 4M matrix on every solve; here its LU is kept while a and
    // b are bit-identical to the ones it was factored with (and the tree was not rebuilt).
    bool same = false;
    if (root_lu_valid_) {
        root_same(st_, m, d_bca_, d_bcb_, d_roota_, d_rootb_, d_rootflag_);
        check(cudaMemcpyAsync(&root_flag_host_, d_rootflag_, sizeof(int), cudaMemcpyDeviceToHost, st_), "root flag");
        check(cudaStreamSynchronize(st_), "root flag");
        same = root_flag_host_ != 0;
    }
    if (!same) {
        root_assemble(st_, m, d_bca_, d_bcb_, nodes_[0].T, d_rootA_);
        check(cudaMemsetAsync(d_rootinfo_, 0, sizeof(int), st_), "memset root info");
        dgetrf_batched(st_, m, d_rootA_arr_, m, d_rootpiv_arr_, d_rootinfo_, 1);
        piv_to_perm(st_, m, d_rootpiv_arr_, d_rootperm_arr_, 1);
        check(cudaMemcpyAsync(d_roota_, d_bca_, m * sizeof(double), cudaMemcpyDeviceToDevice, st_), "root a");
        check(cudaMemcpyAsync(d_rootb_, d_bcb_, m * sizeof(double), cudaMemcpyDeviceToDevice, st_), "root b");
        root_lu_valid_ = true;
        ++root_factorizations_;
    }
    root_rhs(st_, m, d_bcb_, d_bcr_, nodes_[0].h, d_rootperm_, d_rootrhs_);
    dlu_solve_permuted(st_, m, 1, (const double* const*)d_rootA_arr_, m, d_rootrhs_arr_, 1, 1);
    check(cudaMemcpyAsync(nodes_[0].g, d_rootrhs_, m * sizeof(double), cudaMemcpyDeviceToDevice, st_),
          "root g");
    pe(same ? 8.0 * double(m) * m : 8.0 * 3 * double(m) * m,
       (same ? 0.0 : 2.0 / 3.0 * double(m) * m * m) + 2.0 * double(m) * m);
}

void Hps::downwards() {
    downward_levels(mesh_.max_level, false);
    if (homogeneous_) fill_zero(st_, d_f_, (long long)num_leaves() * n_ * n_);
    const double L = num_leaves(), n = n_;
    pb("leaf_solve");
    leaf_run(LEAF_SOLVE, d_items_solve_, num_leaves());
    pe(L * 8 * (2 * n * n + 4 * n), L * 8 * n * n * n);
}

// split1to4 (HPSAlgorithm.hpp:562-577) from the root down to the nodes of level `bottom`; with
// `uncoarsen_bottom` their g is also brought to their own size (uncoarsen_, :1165-1183)
void Hps::downward_levels(int bottom, bool uncoarsen_bottom) {
    for (int lvl = 0; lvl <= bottom; ++lvl) {
        if (lvl == bottom && !uncoarsen_bottom) break;
        for (size_t k = 0; k < gsteps_.size(); ++k)
            if (gsteps_[k].level == lvl) {
                pb("uncoarsen_g");
                uncoarsen_vec(st_, gsteps_[k].d_in, gsteps_[k].d_out, gsteps_[k].count, gsteps_[k].nf);
                pe(double(gsteps_[k].count) * 8 * 6 * gsteps_[k].nf, double(gsteps_[k].count) * 8 * gsteps_[k].nf);
            }
        if (lvl == bottom) break;
        for (auto& g : groups_) {
            if (g.level != lvl) continue;
            const double c = double(g.nodes.size()), s = g.s;
            pb("downward");
            downward(st_, g.d_items, int(c), g.s, homogeneous_ ? 0 : 1);
            pe(c * 8 * (32 * s * s + 8 * s + 4 * s + 16 * s), c * 2 * 32 * s * s);
        }
    }
}

void Hps::solve_async() {
    const long long key = (homogeneous_ ? 1 : 0) | (bc_general_ ? 2 : 0);
    // the general root solve decides on the host whether its cached LU still applies
    graph_solve_.run(st_, key, graphs_ && !prof_ && !bc_general_, [&] {
        upwards();
        root_from_bc();
        downwards();
    });
}

void GraphCache::clear() {
    for (auto& e : entries_)
        if (e.exec) cudaGraphExecDestroy(e.exec);
    entries_.clear();
    if (cap_) cudaStreamDestroy(cap_);
    cap_ = nullptr;
}

double Hps::build_flops() const {
    double f = 0;
    for (const auto& g : groups_) {
        const double m = 4.0 * g.s, cnt = double(g.nodes.size());
        f += cnt * (2.0 / 3.0 * m * m * m + 2.0 * m * m * (3 * m) + 2.0 * (2 * m) * (2 * m) * (m / 2));
    }
    return f;
}

double Hps::solve_bytes() const {
    double b = 0;
    for (const auto& g : groups_) {
        const double s = g.s, cnt = double(g.nodes.size());
        // X^{-1} (16 s^2) + compact H (16 s^2) + S (32 s^2)
        b += cnt * 8.0 * (16 * s * s + 16 * s * s + 32 * s * s);
    }
    b += double(num_leaves()) * n_ * n_ * 8.0 * 3;  // f read twice, u written
    return b;
}

double Hps::solve_flops() const {
    double f = 0;
    for (const auto& g : groups_) {
        const double s = g.s, cnt = double(g.nodes.size());
        f += cnt * 2.0 * (16 * s * s + 16 * s * s + 32 * s * s);
    }
    f += double(num_leaves()) * (8.0 * n_ * n_ * n_ + 6.0 * n_ * n_ * n_);
    return f;
}

}  // namespace efgb
