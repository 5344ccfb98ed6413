// Host side of the mixed-precision many-RHS solver (see ef_mixed.cu for the method).
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include "ef_hps.hpp"

namespace efgb {

namespace {

struct MxCarver {
    char* base = nullptr;
    size_t off = 0;
    template <class T>
    T* get(size_t count) {
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += (std::max<size_t>(count, 1) * sizeof(T) + 255) / 256 * 256;
        return p;
    }
};

void ck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

}  // namespace

MixedSolver::MixedSolver(Hps& hps, int bmax) : H_(hps), bmax_(bmax) {
    if (!hps.built()) throw std::invalid_argument("mixed solver: build the FP64 tree first");
    if (hps.solver_type() != SOLVER_FISHPACK90)
        throw std::invalid_argument("mixed solver: FISHPACK90 (constant coefficient) leaves only");
    if (bmax < 1 || bmax > 1024) throw std::invalid_argument("mixed solver: bmax must be in [1, 1024]");
    const int N = hps.num_nodes(), L = hps.num_leaves(), n = hps.leaf_n();
    const size_t nn = size_t(n) * n, B = size_t(bmax);
    const int M = hps.root_M();
    const Mesh& mesh = hps.mesh();
    mn_.assign(N, MNode());

    auto layout = [&](MxCarver& cv) {
        // interface states first, contiguous (cleared at every solve)
        const size_t ug0 = cv.off;
        for (int id = 0; id < N; ++id)
            if (!mesh.nodes[id].leaf()) mn_[id].uG = cv.get<double>(4 * size_t(hps.nodes_[id].s) * B);
        uG_bytes_ = cv.off - ug0;
        uG_begin_ = cv.base ? cv.base + ug0 : nullptr;
        for (int id = 0; id < N; ++id) {
            const NodeDev& nd = hps.nodes_[id];
            MNode& m = mn_[id];
            if (mesh.nodes[id].leaf()) {
                m.g32 = cv.get<float>(4 * size_t(n) * B);
                m.h32 = cv.get<float>(4 * size_t(n) * B);
                m.g64 = cv.get<double>(4 * size_t(n) * B);
                m.h64 = cv.get<double>(4 * size_t(n) * B);
            } else {
                const size_t s = nd.s;
                m.S = cv.get<float>(32 * s * s);
                m.Xi = cv.get<float>(16 * s * s);
                m.H32 = cv.get<float>(16 * s * s);
                m.h32 = cv.get<float>(8 * s * B);
                m.hd32 = cv.get<float>(4 * s * B);
                m.w32 = cv.get<float>(4 * s * B);
                m.m32 = cv.get<float>(4 * s * B);
                m.g32 = cv.get<float>(4 * size_t(nd.size) * B);
                m.g64 = cv.get<double>(4 * size_t(nd.size) * B);
                m.h64 = cv.get<double>(8 * s * B);
            }
            m.hs32.clear(); m.gs32.clear(); m.hs64.clear(); m.gs64.clear();
            for (int t = 0; t < nd.ncoarsen; ++t) {
                const size_t nc = size_t(nd.nx >> t) / 2;
                m.hs32.push_back(cv.get<float>(4 * nc * B));
                m.hs64.push_back(cv.get<double>(4 * nc * B));
                const int cf = nd.ncoarsen - (t + 1);
                m.gs32.push_back(cv.get<float>(4 * size_t(nd.nx >> cf) * B));
                m.gs64.push_back(cv.get<double>(4 * size_t(nd.nx >> cf) * B));
            }
            m.hc32 = nd.ncoarsen ? m.hs32.back() : m.h32;
            m.hc64 = nd.ncoarsen ? m.hs64.back() : m.h64;
            m.gf32 = nd.ncoarsen ? m.gs32.back() : m.g32;
            m.gf64 = nd.ncoarsen ? m.gs64.back() : m.g64;
        }
        q32_ = cv.get<float>(B * L * nn);
        u64_ = cv.get<double>(B * L * nn);
        f_ = cv.get<double>(B * L * nn);
        a_ = cv.get<double>(B * 4 * M);
        r_ = cv.get<double>(B * 4 * M);
        rmax_ = cv.get<double>(B * kMaxPasses);
        d_types32_ = cv.get<LeafType32>(hps.types_.size());
        d_leaves_ = cv.get<MixLeaf>(L);
        groups_.assign(hps.groups_.size(), MGroup());
        for (size_t gi = 0; gi < hps.groups_.size(); ++gi) {
            const Group& g = hps.groups_[gi];
            groups_[gi].level = g.level;
            groups_[gi].s = g.s;
            groups_[gi].cnt = int(g.nodes.size());
            groups_[gi].d_items = cv.get<MixItem>(g.nodes.size());
            groups_[gi].d_conv = cv.get<MixConv>(g.nodes.size());
        }
        hsteps_.assign(hps.step_nodes_t_.size(), MStep());
        for (size_t k = 0; k < hsteps_.size(); ++k) {
            MStep& st = hsteps_[k];
            st.level = hps.hsteps_[k].level;
            st.nf = hps.hsteps_[k].nf;
            st.count = hps.hsteps_[k].count;
            st.in32 = cv.get<void*>(st.count);
            st.out32 = cv.get<void*>(st.count);
            st.in64 = cv.get<void*>(st.count);
            st.out64 = cv.get<void*>(st.count);
        }
        gsteps_.assign(hps.step_nodes_g_.size(), MStep());
        for (size_t k = 0; k < gsteps_.size(); ++k) {
            MStep& st = gsteps_[k];
            st.level = hps.gsteps_[k].level;
            st.nf = hps.gsteps_[k].nf;
            st.count = hps.gsteps_[k].count;
            st.in32 = cv.get<void*>(st.count);
            st.out32 = cv.get<void*>(st.count);
            st.in64 = cv.get<void*>(st.count);
            st.out64 = cv.get<void*>(st.count);
        }
    };
    MxCarver dry;
    layout(dry);
    bytes_ = dry.off;
    ck(cudaMalloc(&arena_, bytes_), "cudaMalloc(mixed arena)");
    MxCarver real;
    real.base = arena_;
    layout(real);
    cudaStream_t st = hps.stream();
    ck(cudaMemsetAsync(arena_, 0, bytes_, st), "memset(mixed arena)");

    // leaf tables in FP32
    std::vector<LeafType32> t32(hps.types_.size());
    {
        std::vector<double> V(nn), D(nn);
        std::vector<float> Vf(nn), Df(nn);
        float* tab = nullptr;
        ck(cudaMalloc(&tab, 2 * nn * t32.size() * sizeof(float)), "cudaMalloc(fp32 tables)");
        tables_ = tab;
        for (size_t t = 0; t < t32.size(); ++t) {
            leaf_tables(n, hps.types_[t].dx, hps.types_[t].dy, hps.lambda_, V.data(), D.data());
            for (size_t e = 0; e < nn; ++e) { Vf[e] = float(V[e]); Df[e] = float(D[e]); }
            ck(cudaMemcpy(tab + 2 * nn * t, Vf.data(), nn * 4, cudaMemcpyHostToDevice), "upload V32");
            ck(cudaMemcpy(tab + 2 * nn * t + nn, Df.data(), nn * 4, cudaMemcpyHostToDevice), "upload D32");
            t32[t] = LeafType32{n, float(hps.types_[t].dx), float(hps.types_[t].dy), tab + 2 * nn * t,
                                tab + 2 * nn * t + nn};
        }
        ck(cudaMemcpy(d_types32_, t32.data(), t32.size() * sizeof(LeafType32), cudaMemcpyHostToDevice), "types32");
    }
    std::vector<MixLeaf> leaves(L);
    for (int k = 0; k < L; ++k) {
        const int id = mesh.leaves[k];
        leaves[k] = MixLeaf{hps.nodes_[id].leaf_type, mn_[id].g32, mn_[id].h32, mn_[id].g64, mn_[id].h64};
    }
    ck(cudaMemcpy(d_leaves_, leaves.data(), L * sizeof(MixLeaf), cudaMemcpyHostToDevice), "mix leaves");
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        const Group& g = hps.groups_[gi];
        std::vector<MixItem> items(g.nodes.size());
        std::vector<MixConv> conv(g.nodes.size());
        for (size_t i = 0; i < g.nodes.size(); ++i) {
            const int id = g.nodes[i];
            const MNode& m = mn_[id];
            MixItem& it = items[i];
            it.S = m.S; it.Xi = m.Xi; it.H = m.H32;
            it.h = m.h32; it.hd = m.hd32; it.w = m.w32; it.m = m.m32; it.gf = m.gf32; it.uG = m.uG;
            it.gf64 = m.gf64; it.h64 = m.h64; it.mout = m.m32;
            for (int c = 0; c < 4; ++c) {
                const MNode& ch = mn_[mesh.nodes[id].child[c]];
                it.hc[c] = ch.hc32;
                it.gc[c] = ch.g32;
                it.gc64[c] = ch.g64;
                it.hc64[c] = ch.hc64;
            }
            conv[i] = MixConv{hps.nodes_[id].RHS, hps.nodes_[id].H, m.S, m.Xi, m.H32};
        }
        ck(cudaMemcpy(groups_[gi].d_items, items.data(), items.size() * sizeof(MixItem), cudaMemcpyHostToDevice), "mix items");
        ck(cudaMemcpy(groups_[gi].d_conv, conv.data(), conv.size() * sizeof(MixConv), cudaMemcpyHostToDevice), "mix conv");
    }
    auto fill_steps = [&](std::vector<MStep>& steps, const std::vector<std::vector<int>>& nodes,
                          const std::vector<int>& index, bool up) {
        for (size_t k = 0; k < steps.size(); ++k) {
            const int t = index[k];
            std::vector<void*> i32, o32, i64, o64;
            for (int id : nodes[k]) {
                const MNode& m = mn_[id];
                if (up) {
                    i32.push_back(t == 0 ? (void*)m.h32 : (void*)m.hs32[t - 1]);
                    o32.push_back(m.hs32[t]);
                    i64.push_back(t == 0 ? (void*)m.h64 : (void*)m.hs64[t - 1]);
                    o64.push_back(m.hs64[t]);
                } else {
                    i32.push_back(t == 0 ? (void*)m.g32 : (void*)m.gs32[t - 1]);
                    o32.push_back(m.gs32[t]);
                    i64.push_back(t == 0 ? (void*)m.g64 : (void*)m.gs64[t - 1]);
                    o64.push_back(m.gs64[t]);
                }
            }
            const size_t c = i32.size() * sizeof(void*);
            ck(cudaMemcpy(steps[k].in32, i32.data(), c, cudaMemcpyHostToDevice), "steps");
            ck(cudaMemcpy(steps[k].out32, o32.data(), c, cudaMemcpyHostToDevice), "steps");
            ck(cudaMemcpy(steps[k].in64, i64.data(), c, cudaMemcpyHostToDevice), "steps");
            ck(cudaMemcpy(steps[k].out64, o64.data(), c, cudaMemcpyHostToDevice), "steps");
        }
    };
    fill_steps(hsteps_, hps.step_nodes_t_, hps.step_index_t_, true);
    fill_steps(gsteps_, hps.step_nodes_g_, hps.step_index_g_, false);
    // FP32 operator copies
    for (auto& g : groups_) mx_convert(st, g.d_conv, g.cnt, g.s);
    ck(cudaGetLastError(), "mixed convert");
    ck(cudaStreamSynchronize(st), "mixed setup");
}

MixedSolver::~MixedSolver() {
    if (arena_) cudaFree(arena_);
    if (tables_) cudaFree(tables_);
}

void MixedSolver::residual(int B, double* rmax) {
    Hps& h = H_;
    cudaStream_t st = h.stream();
    const int maxL = h.mesh().max_level;
    // exact Dirichlet data of every node from the root data and the interface state
    for (int lvl = 0; lvl < maxL; ++lvl) {
        for (auto& s : gsteps_)
            if (s.level == lvl) mx_uncoarsen(st, true, s.in64, s.out64, s.count, s.nf, B);
        for (auto& g : groups_)
            if (g.level == lvl) mx_scatter64(st, g.d_items, g.cnt, g.s, B);
    }
    mx_leaf_residual(st, h.d_types_, d_leaves_, h.num_leaves(), B, h.lambda_, f_, u64_, q32_, rmax);
    for (int lvl = maxL - 1; lvl >= 0; --lvl) {
        for (auto& s : hsteps_)
            if (s.level == lvl + 1) mx_coarsen(st, true, s.in64, s.out64, s.count, s.nf, B);
        for (auto& g : groups_)
            if (g.level == lvl) mx_flux_up(st, g.d_items, g.cnt, g.s, B);
    }
}

void MixedSolver::pass(int B) {
    Hps& h = H_;
    cudaStream_t st = h.stream();
    const int maxL = h.mesh().max_level;
    const int L = h.num_leaves(), n = h.leaf_n();
    mx_leaf32(st, LEAF_NEUMANN, d_types32_, d_leaves_, L, B, n, q32_, nullptr);
    for (int lvl = maxL - 1; lvl >= 0; --lvl) {
        for (auto& s : hsteps_)
            if (s.level == lvl + 1) mx_coarsen(st, false, s.in32, s.out32, s.count, s.nf, B);
        for (auto& g : groups_)
            if (g.level == lvl) mx_up(st, g.d_items, g.cnt, g.s, B);
    }
    // homogeneous root data for the correction
    ck(cudaMemsetAsync(mn_[0].g32, 0, sizeof(float) * 4 * size_t(h.root_M()) * B, st), "root g32");
    for (int lvl = 0; lvl < maxL; ++lvl) {
        for (auto& s : gsteps_)
            if (s.level == lvl) mx_uncoarsen(st, false, s.in32, s.out32, s.count, s.nf, B);
        for (auto& g : groups_)
            if (g.level == lvl) mx_down(st, g.d_items, g.cnt, g.s, B);
    }
    mx_leaf32(st, LEAF_SOLVE, d_types32_, d_leaves_, L, B, n, q32_, u64_);
}

void MixedSolver::solve(int B, int sweeps) {
    if (B < 1 || B > bmax_) throw std::invalid_argument("mixed solver: batch size out of range");
    if (sweeps < 0 || sweeps + 1 > kMaxPasses) throw std::invalid_argument("mixed solver: too many sweeps");
    Hps& h = H_;
    cudaStream_t st = h.stream();
    const size_t cells = size_t(h.num_leaves()) * h.leaf_n() * h.leaf_n();
    ck(cudaMemsetAsync(u64_, 0, sizeof(double) * cells * B, st), "clear u");
    ck(cudaMemsetAsync(uG_begin_, 0, uG_bytes_, st), "clear interface state");
    ck(cudaMemsetAsync(rmax_, 0, sizeof(double) * size_t(bmax_) * kMaxPasses, st), "clear residuals");
    mx_root(st, 4 * h.root_M(), B, a_, r_, mn_[0].g64);
    for (int p = 0; p <= sweeps; ++p) {
        residual(B, rmax_ + size_t(p) * bmax_);
        pass(B);
    }
}

}  // namespace efgb
