// Host side of the mixed-precision many-RHS solver (see ef_mixed.cu for the method).
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>

#include <cudaTypedefs.h>

#include "ef_hps.hpp"

namespace efgb {

namespace {
// c = m 2^(e - 63) with m a signed 63-bit significand (|m| in [2^62, 2^63), exact); c = 0 gives m = 0
void significand63(double c, long long& m, int& e) {
    int ex = 0;
    const double fr = std::frexp(c, &ex);  // c = fr 2^ex, |fr| in [0.5, 1)
    m = c == 0.0 ? 0ll : (long long)std::ldexp(fr, 63);
    e = c == 0.0 ? 0 : ex;
}
}  // namespace

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

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda)
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        ck(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q),
           "driver entry point cuTensorMapEncodeTiled");
        if (q != cudaDriverEntryPointSuccess || !p) throw std::runtime_error("cuTensorMapEncodeTiled unavailable");
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// row-major FP32 matrix [rows][cols] read in boxes of 32 columns x box_rows rows, 128-byte swizzle
CUtensorMap make_map(float* base, long long rows, int cols, int box_rows) {
    CUtensorMap tm;
    const cuuint64_t dims[2] = {cuuint64_t(cols), cuuint64_t(rows)};
    const cuuint64_t strides[1] = {cuuint64_t(cols) * sizeof(float)};
    const cuuint32_t box[2] = {32u, cuuint32_t(box_rows)};
    const cuuint32_t estr[2] = {1u, 1u};
    const CUresult r = encode_tiled()(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                                      CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")");
    return tm;
}

}  // namespace

MixedSolver::MixedSolver(Hps& hps, int bmax, const MixedSolver* share)
    : H_(hps), bmax_(bmax), st_(hps.stream()), share_(share) {
    if (share && &share->H_ != &hps) throw std::invalid_argument("mixed solver: operators shared across trees");
    if (!hps.built() && !hps.built32()) throw std::invalid_argument("mixed solver: build the tree first");
    const bool fp = hps.solver_type() == SOLVER_FIVE_POINT;
    if (bmax < 1 || bmax > 1024) throw std::invalid_argument("mixed solver: bmax must be in [1, 1024]");
    const int N = hps.num_nodes(), L = hps.num_leaves(), n = hps.leaf_n();
    if ((long long)L * bmax >= (1LL << 31) || 12LL * hps.node(0).nx * bmax >= (1LL << 31))
        throw std::invalid_argument("mixed solver: leaves x bmax too large for 32-bit item indices");
    if (fp && n > 32)
        throw std::invalid_argument("mixed solver: FivePointStencil leaves of at most 32 x 32 cells");
    if (n % 4 != 0 || n > 64)
        throw std::invalid_argument("mixed solver: the leaf size must be a multiple of 4 and at most 64");
    const size_t nn = size_t(n) * n, B = size_t(bmax);
    const int M = hps.root_M();
    const Mesh& mesh = hps.mesh();
    mn_.assign(N, MNode());

    // a tree without coarsening steps copies rows unchanged from level to level: the residual reads
    // the leaves' Dirichlet rows where they live and takes every interface mismatch straight from
    // two leaf edge-flux rows (tables traced below)
    const bool direct = hps.step_nodes_t_.empty() && hps.step_nodes_g_.empty() && !g_level_interface.load();
    long long nmis = 0;
    for (int id = 0; id < N && direct; ++id)
        if (!mesh.nodes[id].leaf()) nmis += 4LL * hps.nodes_[id].s;
    const int nroot = direct && N > 1 ? 8 * hps.nodes_[0].s : 0;
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
        d_err_ = cv.get<int>(1);
        rleaf_ = cv.get<float>(B * L);
        d_coef_ = cv.get<MixCoef>(hps.types_.size());
        d_types32_ = cv.get<LeafType32>(hps.types_.size());
        d_leaves_ = cv.get<MixLeaf>(L);
        d_gsrc_ = cv.get<MxRow>(size_t(L) * 4 * n);
        d_mis_ = cv.get<MxMis>(size_t(nmis));
        d_add_ = cv.get<MxAdd>(size_t(nmis));
        d_rootsrc_ = cv.get<MxRow>(size_t(nroot));
        if (fp) {
            // FP32 band factors and FP64 stencil tables, shared by the lanes of one tree
            d_fps_ = cv.get<MixFp>(L);
            fp_band32_ = share ? share->fp_band32_ : cv.get<float>(size_t(L) * 4 * nn * n);
            fp_bcoef32_ = share ? share->fp_bcoef32_ : cv.get<float>(size_t(L) * 4 * n);
            fp_coef64_ = share ? share->fp_coef64_ : cv.get<double>(size_t(L) * 5 * nn);
        }
        groups_.assign(hps.groups_.size(), MGroup());
        for (size_t gi = 0; gi < hps.groups_.size(); ++gi) {
            const Group& g = hps.groups_[gi];
            groups_[gi].level = g.level;
            groups_[gi].s = g.s;
            groups_[gi].cnt = int(g.nodes.size());
            groups_[gi].d_items = cv.get<MixItem>(g.nodes.size());
            groups_[gi].d_conv = cv.get<MixConv>(g.nodes.size());
            // FP32 operators of the group back to back: one row-major matrix per kind (or the
            // operators of the lane this one shares them with)
            const size_t s = g.s, cnt = g.nodes.size();
            float* S = share ? share->groups_[gi].S32 : cv.get<float>(cnt * 32 * s * s);
            float* Xi = share ? share->groups_[gi].Xi32 : cv.get<float>(cnt * 16 * s * s);
            float* H32 = share ? share->groups_[gi].H32 : cv.get<float>(cnt * 16 * s * s);
            groups_[gi].S32 = S;
            groups_[gi].Xi32 = Xi;
            groups_[gi].H32 = H32;
            // bf16 planes of the tensor-core path (3 x the FP32 element count up to the padding of
            // the last row tile and K chunk, 2 bytes each) (per kind: W, H, DOWN)
            for (int kind = 0; kind < 3; ++kind)
                groups_[gi].tc[kind] = hps.tensor_cores() != 0 && mx_tc_supported(kind, g.s);
            if (groups_[gi].tc[2])
                groups_[gi].S3 = share ? share->groups_[gi].S3
                                       : (void*)cv.get<uint16_t>(size_t(mx_tc_plane_elems(cnt * 4 * s, int(8 * s))));
            if (groups_[gi].tc[0])
                groups_[gi].Xi3 = share ? share->groups_[gi].Xi3
                                        : (void*)cv.get<uint16_t>(size_t(mx_tc_plane_elems(cnt * 4 * s, int(4 * s))));
            if (groups_[gi].tc[1])
                groups_[gi].H3 = share ? share->groups_[gi].H3
                                       : (void*)cv.get<uint16_t>(size_t(mx_tc_plane_elems(cnt * 8 * s, int(2 * s))));
            for (size_t i = 0; i < cnt; ++i) {
                MNode& m = mn_[g.nodes[i]];
                m.S = S ? S + i * 32 * s * s : nullptr;
                m.Xi = Xi ? Xi + i * 16 * s * s : nullptr;
                m.H32 = H32 ? H32 + i * 16 * s * s : nullptr;
            }
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
    cudaStream_t st = st_;
    ck(cudaMemsetAsync(arena_, 0, bytes_, st), "memset(mixed arena)");

    if (fp) {
        std::vector<MixFp> fl(L);
        for (int k = 0; k < L; ++k)
            fl[k] = MixFp{fp_band32_ + size_t(k) * 4 * nn * n, fp_bcoef32_ + size_t(k) * 4 * n,
                          fp_coef64_ + size_t(k) * 5 * nn, 2.0 / hps.types_[k].dx, 2.0 / hps.types_[k].dy};
        ck(upload_sync(st_, d_fps_, fl.data(), L * sizeof(MixFp)), "mixed fp leaves");
        if (!share) mx_fp_convert(st, hps.d_fp_, d_fps_, L, n);
    }
    // leaf tables in FP32 (constant-coefficient leaves)
    std::vector<LeafType32> t32(fp ? 0 : hps.types_.size());
    if (!fp) {
        std::vector<double> V(nn), D(nn);
        std::vector<float> Vf(nn), Df(nn);
        float* tab = nullptr;
        ck(cudaMalloc(&tab, 2 * nn * t32.size() * sizeof(float)), "cudaMalloc(fp32 tables)");
        tables_ = tab;
        for (size_t t = 0; t < t32.size(); ++t) {
            leaf_tables(n, hps.types_[t].dx, hps.types_[t].dy, hps.lambda_, V.data(), D.data());
            for (size_t e = 0; e < nn; ++e) { Vf[e] = float(V[e]); Df[e] = float(D[e]); }
            ck(upload_sync(st_, tab + 2 * nn * t, Vf.data(), nn * 4), "upload V32");
            ck(upload_sync(st_, tab + 2 * nn * t + nn, Df.data(), nn * 4), "upload D32");
            t32[t] = LeafType32{n, float(hps.types_[t].dx), float(hps.types_[t].dy), tab + 2 * nn * t,
                                tab + 2 * nn * t + nn};
        }
        ck(upload_sync(st_, d_types32_, t32.data(), t32.size() * sizeof(LeafType32)), "types32");
        if (n == 16) mx_set_basis16(st_, Vf.data());  // V depends on n only: the last type's copy serves all
        std::vector<MixCoef> co(hps.types_.size());
        for (size_t t = 0; t < co.size(); ++t) {
            const double dx = hps.types_[t].dx, dy = hps.types_[t].dy;
            const double cx = 1.0 / (dx * dx), cy = 1.0 / (dy * dy), lm = hps.lambda_;
            MixCoef& c = co[t];
            c.dtn_x = 2.0 / dx;
            c.dtn_y = 2.0 / dy;
            significand63(cx, c.cxm, c.ecx);
            significand63(cy, c.cym, c.ecy);
            significand63(lm, c.lmm, c.elm);
            c.iso = cx == cy ? 1 : 0;
            c.cx32 = float(cx);
            c.cy32 = float(cy);
            if (!c.iso || c.lmm) res_form_ = 1;
        }
        ck(upload_sync(st_, d_coef_, co.data(), co.size() * sizeof(MixCoef)), "mixed coefs");
    }
    // where each leaf's Dirichlet rows live, and the rows of every interface mismatch: traced
    // through the index maps of the per-level kernels (exterior rows to the children, the parent's
    // interface state to both sides; upward, exterior fluxes from the children)
    direct_ = direct;
    nmis_ = nmis;
    nroot_ = nroot;
    {
        // rows are named by buffer and row: their addresses depend on the block's request count
        auto row = [&](const void* buf, size_t r) {
            const size_t off = size_t(reinterpret_cast<const char*>(buf) - arena_);
            if (off % 256 != 0 || off / 256 > 0xffffffffull) throw std::logic_error("mixed solver: arena row");
            return MxRow{unsigned(off / 256), unsigned(r)};
        };
        const size_t n4 = 4 * size_t(n);
        std::vector<MxRow> gtab(size_t(L) * n4);
        if (direct) {
            std::vector<int> order{0};  // breadth first: parents before children
            for (size_t i = 0; i < order.size(); ++i)
                if (!mesh.nodes[order[i]].leaf())
                    for (int c = 0; c < 4; ++c) order.push_back(mesh.nodes[order[i]].child[c]);
            std::vector<std::vector<MxRow>> gt(N), ht(N);
            gt[0].resize(N > 1 ? 8 * size_t(hps.nodes_[0].s) : n4);
            for (size_t p = 0; p < gt[0].size(); ++p) gt[0][p] = row(mn_[0].g64, p);
            for (int id : order) {
                if (mesh.nodes[id].leaf()) continue;
                const int s = hps.nodes_[id].s;
                const int* ch = mesh.nodes[id].child;
                for (int c = 0; c < 4; ++c) gt[ch[c]].assign(4 * size_t(s), MxRow{0u, 0u});
                for (int p = 0; p < 8 * s; ++p) {
                    int c, q;
                    mx_ext_map(p, s, c, q);
                    gt[ch[c]][q] = gt[id][p];
                }
                for (int r = 0; r < 4 * s; ++r) {
                    const int I = r / s, o = r - I * s;
                    const MxRow v = row(mn_[id].uG, size_t(r));
                    gt[ch[mx_lower_child(I)]][mx_q_lower(I, o, s)] = v;
                    gt[ch[mx_upper_child(I)]][mx_q_upper(I, o, s)] = v;
                }
                std::vector<MxRow>().swap(gt[id]);
            }
            std::vector<MxMis> mis;
            mis.reserve(size_t(nmis));
            // the FP64 state update of a pass: a node's interface row and the lower child's
            // Dirichlet row into which DOWN writes the pass's value
            std::vector<MxAdd> adds;
            adds.reserve(size_t(nmis));
            for (int id : order) {
                if (mesh.nodes[id].leaf()) continue;
                const int s = hps.nodes_[id].s;
                const int* ch = mesh.nodes[id].child;
                for (int r = 0; r < 4 * s; ++r) {
                    const int I = r / s, o = r - I * s;
                    adds.push_back(MxAdd{row(mn_[id].uG, size_t(r)), row(mn_[ch[mx_lower_child(I)]].g32, size_t(mx_q_lower(I, o, s)))});
                }
            }
            if ((long long)adds.size() != nmis) throw std::logic_error("mixed solver: state rows not traced");
            ck(upload_sync(st_, d_add_, adds.data(), adds.size() * sizeof(MxAdd)), "state rows");
            for (auto it = order.rbegin(); it != order.rend(); ++it) {
                const int id = *it;
                if (mesh.nodes[id].leaf()) {
                    ht[id].resize(n4);
                    for (size_t k = 0; k < n4; ++k) ht[id][k] = row(mn_[id].h64, k);
                    continue;
                }
                const int s = hps.nodes_[id].s;
                const int* ch = mesh.nodes[id].child;
                ht[id].resize(8 * size_t(s));
                for (int e = 0; e < 8 * s; ++e) {
                    int c, q;
                    mx_ext_map(e, s, c, q);
                    ht[id][e] = ht[ch[c]][q];
                }
                for (int r = 0; r < 4 * s; ++r) {
                    const int I = r / s, o = r - I * s;
                    mis.push_back(MxMis{row(mn_[id].m32, size_t(r)), ht[ch[mx_lower_child(I)]][mx_q_lower(I, o, s)],
                                        ht[ch[mx_upper_child(I)]][mx_q_upper(I, o, s)]});
                }
                for (int c = 0; c < 4; ++c) std::vector<MxRow>().swap(ht[ch[c]]);
            }
            for (int k = 0; k < L; ++k) {
                const auto& g = gt[mesh.leaves[k]];
                if (g.size() != n4) throw std::logic_error("mixed solver: leaf Dirichlet rows not traced");
                std::copy(g.begin(), g.end(), gtab.begin() + size_t(k) * n4);
            }
            if ((long long)mis.size() != nmis) throw std::logic_error("mixed solver: interface rows not traced");
            ck(upload_sync(st_, d_mis_, mis.data(), mis.size() * sizeof(MxMis)), "mismatch rows");
            if (nroot) ck(upload_sync(st_, d_rootsrc_, ht[0].data(), size_t(nroot) * sizeof(MxRow)), "root rows");
        } else {
            for (int k = 0; k < L; ++k)
                for (size_t j = 0; j < n4; ++j) gtab[size_t(k) * n4 + j] = row(mn_[mesh.leaves[k]].g64, j);
        }
        ck(upload_sync(st_, d_gsrc_, gtab.data(), gtab.size() * sizeof(MxRow)), "leaf Dirichlet rows");
    }
    std::vector<MixLeaf> leaves(L);
    for (int k = 0; k < L; ++k) {
        const int id = mesh.leaves[k];
        leaves[k] = MixLeaf{hps.nodes_[id].leaf_type, mn_[id].g32, mn_[id].h32, mn_[id].g64, mn_[id].h64,
                            d_gsrc_ + size_t(k) * 4 * n, arena_};
    }
    ck(upload_sync(st_, d_leaves_, leaves.data(), L * sizeof(MixLeaf)), "mix leaves");
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        const Group& g = hps.groups_[gi];
        std::vector<MixItem> items(g.nodes.size());
        std::vector<MixConv> conv(g.nodes.size());
        for (size_t i = 0; i < g.nodes.size(); ++i) {
            const int id = g.nodes[i];
            const MNode& m = mn_[id];
            MixItem& it = items[i];
            it.S = m.S; it.Xi = m.Xi; it.H = m.H32;
            // uG null: the DOWN epilogues leave the FP64 state to mx_state_add (trees without coarsening)
            it.h = m.h32; it.hd = m.hd32; it.w = m.w32; it.m = m.m32; it.gf = m.gf32; it.uG = direct_ ? nullptr : m.uG;
            it.gf64 = m.gf64; it.h64 = m.h64; it.mout = m.m32;
            for (int c = 0; c < 4; ++c) {
                const MNode& ch = mn_[mesh.nodes[id].child[c]];
                it.hc[c] = ch.hc32;
                it.gc[c] = ch.g32;
                it.gc64[c] = ch.g64;
                it.hc64[c] = ch.hc64;
            }
            conv[i] = hps.built32() ? MixConv{nullptr, nullptr, m.S, m.Xi, m.H32, hps.n32_[id].RHS, hps.n32_[id].H}
                                    : MixConv{hps.nodes_[id].RHS, hps.nodes_[id].H, m.S, m.Xi, m.H32, nullptr, nullptr};
        }
        ck(upload_sync(st_, groups_[gi].d_items, items.data(), items.size() * sizeof(MixItem)), "mix items");
        ck(upload_sync(st_, groups_[gi].d_conv, conv.data(), conv.size() * sizeof(MixConv)), "mix conv");
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
            ck(upload_sync(st_, steps[k].in32, i32.data(), c), "steps");
            ck(upload_sync(st_, steps[k].out32, o32.data(), c), "steps");
            ck(upload_sync(st_, steps[k].in64, i64.data(), c), "steps");
            ck(upload_sync(st_, steps[k].out64, o64.data(), c), "steps");
        }
    };
    fill_steps(hsteps_, hps.step_nodes_t_, hps.step_index_t_, true);
    fill_steps(gsteps_, hps.step_nodes_g_, hps.step_index_g_, false);
    // FP32 operator copies and the TMA descriptors that stream them
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        MGroup& g = groups_[gi];
        if (share) {
            g.tmS = share->groups_[gi].tmS;
            g.tmXi = share->groups_[gi].tmXi;
            g.tmH = share->groups_[gi].tmH;
            continue;
        }
        mx_convert(st, g.d_conv, g.cnt, g.s);
        const long long cnt = g.cnt, s = g.s;
        if (mx_tile_rows(0, g.s) == 0 || mx_tile_rows(1, g.s) == 0)
            throw std::invalid_argument("mixed solver: interface size not a multiple of 4");
        g.tmS = make_map(g.S32, cnt * 4 * s, int(8 * s), mx_tile_rows(0, g.s));
        g.tmXi = make_map(g.Xi32, cnt * 4 * s, int(4 * s), mx_tile_rows(0, g.s));
        g.tmH = make_map(g.H32, cnt * 8 * s, int(2 * s), mx_tile_rows(1, g.s));
        // (the arena was zeroed: the planes' padding rows and columns stay zero)
        if (g.tc[2]) mx_tc_split(st, 2, g.S32, g.S3, cnt * 4 * s, int(8 * s), g.s);
        if (g.tc[0]) mx_tc_split(st, 0, g.Xi32, g.Xi3, cnt * 4 * s, int(4 * s), g.s);
        if (g.tc[1]) mx_tc_split(st, 1, g.H32, g.H3, cnt * 8 * s, int(2 * s), g.s);
    }
    ck(cudaGetLastError(), "mixed convert");
    ck(cudaStreamSynchronize(st), "mixed setup");
    if (hps.mx_split_.size() != groups_.size() || hps.mx_split_tc_ != hps.tensor_cores()) tune();
}

void Hps::set_mx_plan(const std::vector<std::array<int, 3>>& codes) {
    if (codes.size() != groups_.size())
        throw std::invalid_argument("gemm plan: one row per node group (" + std::to_string(groups_.size()) + ")");
    static const char* kinds[3] = {"W", "H", "DOWN"};
    for (size_t gi = 0; gi < codes.size(); ++gi)
        for (int kind = 0; kind < 3; ++kind) {
            const int c = codes[gi][kind], s = groups_[gi].s;
            if (c < -8 || c > 8) throw std::invalid_argument("gemm plan: codes lie in [-8, 8]");
            if (c >= 0) continue;
            const int k = -c;
            if (tensor_cores_ == 0 || !mx_tc_supported(kind, s) || (k & (k - 1)) != 0 || k > mx_tc_max_split(kind, s))
                throw std::invalid_argument(std::string("gemm plan: no tensor-core ") + kinds[kind] + " GEMM with K split " +
                                            std::to_string(k) + " at s = " + std::to_string(s));
        }
    mx_split_ = codes;
    mx_split_tc_ = tensor_cores_;
}

void MixedSolver::tune() {
    // per group and kind, the fastest of the CUDA-core GEMM (K split 1, 2, 4, ...: code > 0) and the
    // tensor-core GEMM (code < 0: split -code), timed with CUDA events on a block of min(bmax, 32)
    Hps& h = H_;
    const int B = std::min(bmax_, 32);
    std::vector<std::array<int, 3>> best(groups_.size(), std::array<int, 3>{1, 1, 1});
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ck(cudaEventCreate(&e0), "tune event");
    ck(cudaEventCreate(&e1), "tune event");
    auto time_code = [&](const MGroup& g, int kind, int code) {
        node_gemm(st_, g, kind, B, code);  // warm-up
        ck(cudaEventRecord(e0, st_), "tune event");
        for (int r = 0; r < 3; ++r) node_gemm(st_, g, kind, B, code);
        ck(cudaEventRecord(e1, st_), "tune event");
        ck(cudaEventSynchronize(e1), "tune sync");
        float ms = 0.f;
        ck(cudaEventElapsedTime(&ms, e0, e1), "tune time");
        return ms;
    };
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        const MGroup& g = groups_[gi];
        for (int kind = 0; kind < 3; ++kind) {
            float best_ms = 1e30f;
            int best_code = 1;
            const bool forced = g.tc[kind] && h.tensor_cores() == 2;
            for (int pass = forced ? 1 : 0; pass < (g.tc[kind] ? 2 : 1); ++pass) {
                const bool tc = pass == 1;
                const int kmax = tc ? mx_tc_max_split(kind, g.s) : mx_gemm_max_split(kind, g.s);
                float path_ms = 1e30f;
                int path_code = 0;
                for (int ks = 1; ks <= kmax; ks *= 2) {
                    float ms;
                    try {
                        ms = time_code(g, kind, tc ? -ks : ks);
                    } catch (const std::runtime_error&) {
                        // a launch shape the device refuses (e.g. a cluster that does not fit): skip it
                        (void)cudaGetLastError();
                        continue;
                    }
                    if (ms < path_ms * 0.97f) {  // a larger split must win clearly
                        path_ms = ms;
                        path_code = tc ? -ks : ks;
                    }
                }
                if (path_ms < best_ms) {
                    best_ms = path_ms;
                    best_code = path_code;
                }
            }
            best[gi][kind] = best_code;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ck(cudaGetLastError(), "mixed tune");
    if (take_error()) throw std::runtime_error("mixed solver: an operator tile copy did not complete while tuning");
    // the tuning launches wrote the pass buffers and the interface state: start clean
    ck(cudaMemsetAsync(arena_, 0, size_t(uG_begin_ - arena_) + uG_bytes_, st_), "clear after tune");
    h.mx_split_ = best;
    h.mx_split_tc_ = h.tensor_cores();
}

// Bytes a node GEMM launch moves at the least: the operator (FP32, or the three bf16 planes of the
// tensor-core form), the right-hand side block and what the epilogue reads and writes per node --
// W: hd in, w out; H: w in, hc in, h out; DOWN: gf in, w in, both children's interface rows out,
// the FP64 interface state read and written.
double MixedSolver::gemm_bytes(const MGroup& g, int kind, int B, int code) const {
    const double c = g.cnt, s = g.s, eb = (g.tc[kind] && code < 0) ? 6.0 : 4.0;
    const double op = (kind == 2 ? 32.0 : 16.0) * s * s * eb;
    // per request: W 4s in + 4s out (FP32); H 8s + 8s in, 8s out; DOWN 8s + 4s in, 2 x 4s out, 4s
    // FP64 read and written
    const double vec = kind == 0 ? 32.0 * s : kind == 1 ? 96.0 * s : (32.0 + 16.0 + 32.0 + (direct_ ? 0.0 : 64.0)) * s;
    return c * (op + vec * B);
}

void MixedSolver::node_gemm(cudaStream_t st, const MGroup& g, int kind, int B, int code) {
    if (g.tc[kind] && code < 0) {
        const void* planes = kind == 0 ? g.Xi3 : (kind == 1 ? g.H3 : g.S3);
        mx_gemm_tc(st, kind, planes, g.d_items, g.cnt, g.s, B, d_err_, -code);
    } else {
        const int ksplit = code < 0 ? 0 : code;
        const CUtensorMap& tm = kind == 0 ? g.tmXi : (kind == 1 ? g.tmH : g.tmS);
        mx_gemm(st, kind, tm, g.d_items, g.cnt, g.s, B, d_err_, ksplit);
    }
}

std::vector<std::array<int, 5>> MixedSolver::gemm_plan() const {
    std::vector<std::array<int, 5>> out;
    const Hps& h = H_;
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        const std::array<int, 3> c = h.mx_split_.size() == groups_.size() ? h.mx_split_[gi] : std::array<int, 3>{0, 0, 0};
        out.push_back({groups_[gi].level, groups_[gi].s, c[0], c[1], c[2]});
    }
    return out;
}

MixedSolver::~MixedSolver() {
    if (arena_) cudaFree(arena_);
    if (tables_) cudaFree(tables_);
    if (robin_mem_) cudaFree(robin_mem_);
}

void MixedSolver::set_root_operator(const double* a, const double* b) {
    Hps& h = H_;
    const int m = 4 * h.root_M();
    bool general = false;
    for (int i = 0; i < m; ++i)
        if (b[i] != 0.0) { general = true; break; }
    graphs_.clear();  // the captured sequences change with the root operator
    if (!general) {
        robin_ = false;
        return;
    }
    if (!h.built()) throw std::invalid_argument("mixed solver: Robin root data need the FP64 build (root T)");
    cudaStream_t st = st_;
    const size_t mm = size_t(m) * m;
    auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    if (!robin_mem_) {
        const size_t bytes = up(2 * m * 8) + up(m * 4) + up(mm * 4) + 2 * up(size_t(m) * bmax_ * 4) + up(3 * sizeof(void*));
        ck(cudaMalloc(&robin_mem_, bytes), "cudaMalloc(mixed Robin root)");
        char* p = robin_mem_;
        ra64_ = reinterpret_cast<double*>(p); rb64_ = ra64_ + m; p += up(2 * m * 8);
        rb32_ = reinterpret_cast<float*>(p); p += up(m * 4);
        Z32_ = reinterpret_cast<float*>(p); p += up(mm * 4);
        rho32_ = reinterpret_cast<float*>(p); p += up(size_t(m) * bmax_ * 4);
        rhs32_ = reinterpret_cast<float*>(p); p += up(size_t(m) * bmax_ * 4);
        zA_ = reinterpret_cast<const float**>(p);
        zB_ = reinterpret_cast<const float**>(p + sizeof(void*));
        zC_ = reinterpret_cast<float**>(p + 2 * sizeof(void*));
        const void* ptrs[3] = {Z32_, rhs32_, mn_[0].g32};
        ck(upload_sync(st, zA_, ptrs, sizeof(ptrs)), "Robin GEMM pointers");
    }
    std::vector<float> b32(m);
    for (int i = 0; i < m; ++i) b32[i] = float(b[i]);
    ck(upload_sync(st, ra64_, a, m * 8), "Robin a");
    ck(upload_sync(st, rb64_, b, m * 8), "Robin b");
    ck(upload_sync(st, rb32_, b32.data(), m * 4), "Robin b32");
    // Z = (diag a + diag b T)^{-1} in FP64 (LU with partial pivoting, then the solve of P I), kept in FP32
    char* tmp = nullptr;
    const size_t tbytes = 2 * up(mm * 8) + 2 * up(size_t(m) * 4) + up(4) + up(4 * sizeof(void*));
    ck(cudaMalloc(&tmp, tbytes), "cudaMalloc(Robin factor)");
    double* A = reinterpret_cast<double*>(tmp);
    double* Z = reinterpret_cast<double*>(tmp + up(mm * 8));
    int* piv = reinterpret_cast<int*>(tmp + 2 * up(mm * 8));
    int* perm = reinterpret_cast<int*>(tmp + 2 * up(mm * 8) + up(size_t(m) * 4));
    int* info = reinterpret_cast<int*>(tmp + 2 * up(mm * 8) + 2 * up(size_t(m) * 4));
    void** arr = reinterpret_cast<void**>(tmp + 2 * up(mm * 8) + 2 * up(size_t(m) * 4) + up(4));
    int bad = 0;
    try {
        const void* pa[4] = {A, Z, piv, perm};
        ck(upload_sync(st, arr, pa, sizeof(pa)), "Robin pointers");
        ck(cudaMemsetAsync(info, 0, sizeof(int), st), "Robin info");
        root_assemble(st, m, ra64_, rb64_, h.root_T(), A);
        dgetrf_batched(st, m, reinterpret_cast<double* const*>(arr), m, reinterpret_cast<int* const*>(arr + 2), info, 1);
        piv_to_perm(st, m, reinterpret_cast<int* const*>(arr + 2), reinterpret_cast<int* const*>(arr + 3), 1);
        mx_perm_identity(st, m, perm, Z);
        dlu_solve_permuted(st, m, m, reinterpret_cast<const double* const*>(arr), m,
                           reinterpret_cast<double* const*>(arr + 1), m, 1);
        const double* zin[1] = {Z};
        float* zout[1] = {Z32_};
        void** cv = arr;  // reuse the pointer slots for the narrowing copy
        ck(cudaStreamSynchronize(st), "Robin factor");
        ck(upload_sync(st, cv, zin, sizeof(zin)), "Robin narrow in");
        ck(upload_sync(st, cv + 1, zout, sizeof(zout)), "Robin narrow out");
        narrow_batched(st, reinterpret_cast<const double* const*>(cv), reinterpret_cast<float* const*>(cv + 1),
                       (long long)mm, 1);
        ck(cudaMemcpyAsync(&bad, info, sizeof(int), cudaMemcpyDeviceToHost, st), "Robin info");
        ck(cudaStreamSynchronize(st), "Robin set-up");
    } catch (...) {
        cudaStreamSynchronize(st);
        cudaFree(tmp);
        throw;
    }
    cudaFree(tmp);
    if (bad) throw std::invalid_argument("mixed solver: diag(a) + diag(b) T_root is singular");
    robin_ = true;
}

void MixedSolver::residual(int B, double* rmax, bool zero_state, bool fused) {
    Hps& h = H_;
    cudaStream_t st = st_;
    const int maxL = h.mesh().max_level;
    const double L = h.num_leaves(), nn = double(h.leaf_n()) * h.leaf_n();
    // exact Dirichlet data of every node from the root data and the interface state (read in place
    // by the leaves on a tree without coarsening steps)
    if (!direct_) {
        h.pb("mx_interface", st);
        for (int lvl = 0; lvl < maxL; ++lvl) {
            for (auto& s : gsteps_)
                if (s.level == lvl) mx_uncoarsen(st, true, s.in64, s.out64, s.count, s.nf, B);
            for (auto& g : groups_)
                if (g.level == lvl) mx_scatter64(st, g.d_items, g.cnt, g.s, B);
        }
        h.pe(0, 0, st);
    }
    if (fused && zero_state) {
        // f read once for the zero-state residual and the first pass's Neumann step
        const double items = L * B;
        h.pb("mx_leaf_first", st);
        mx_leaf16_first(st, d_types32_, d_coef_, d_leaves_, h.num_leaves(), B, f_, q32_, rleaf_, rmax, d_gsrc_, arena_);
        h.pe(items * (nn * 12.0 + 4 * 16 * 20.0), items * 2.0 * (3 * nn * 16 + 4 * nn), st);
    } else if (fused) {
        // the exact residual and the next pass's Neumann step from registers
        const double items = L * B;
        h.pb("mx_leaf_residual", st);
        mx_leaf16_residual_neumann(st, d_types32_, d_coef_, d_leaves_, h.num_leaves(), B, f_, u64_, q32_, rleaf_, rmax,
                                   d_gsrc_, arena_);
        h.pe(items * (nn * 20.0 + 4 * 16 * 20.0), items * (nn * 6.0 + 2.0 * (3 * nn * 16 + 4 * nn)), st);
    } else {
        h.pb("mx_leaf_residual", st);
        if (d_fps_)
            mx_fp_residual(st, d_fps_, d_leaves_, h.num_leaves(), B, h.leaf_n(), zero_state ? 1 : 0, f_, u64_, q32_,
                           rleaf_, rmax);
        else
            mx_leaf_residual(st, d_coef_, res_form_, d_leaves_, h.num_leaves(), B, h.leaf_n(), zero_state ? 1 : 0, f_,
                             u64_, q32_, rleaf_, rmax, d_gsrc_, arena_);
        // f and the state in, r out; per item the 4n Dirichlet values in, the 4n edge fluxes out (FP64)
        h.pe(L * B * (nn * (zero_state ? 12.0 : 20.0) + 4.0 * h.leaf_n() * 16), zero_state ? 0.0 : L * B * nn * 6.0, st);
    }
    h.pb("mx_interface", st);
    if (direct_) {
        mx_mismatch(st, arena_, d_mis_, nmis_, B);
        if (robin_) mx_gather_rows64(st, arena_, d_rootsrc_, mn_[0].h64, nroot_, B);
    } else {
        for (int lvl = maxL - 1; lvl >= 0; --lvl) {
            for (auto& s : hsteps_)
                if (s.level == lvl + 1) mx_coarsen(st, true, s.in64, s.out64, s.count, s.nf, B);
            for (auto& g : groups_)
                if (g.level == lvl) mx_flux_up(st, g.d_items, g.cnt, g.s, B);
        }
    }
    // residual of the Robin root condition from the state's root data and exact boundary flux
    if (robin_) mx_root_residual(st, 4 * h.root_M(), B, ra64_, rb64_, r_, mn_[0].g64, mn_[0].h64, rho32_);
    h.pe(0, 0, st);
}

void MixedSolver::pass(int B, bool first, bool neumann_done, bool last) {
    Hps& h = H_;
    cudaStream_t st = st_;
    const int maxL = h.mesh().max_level;
    const int L = h.num_leaves(), n = h.leaf_n();
    const double items = double(L) * B, nn = double(n) * n;
    if (!neumann_done) {
        h.pb("mx_leaf_neumann", st);
        if (d_fps_) mx_fp_leaf32(st, LEAF_NEUMANN, d_fps_, d_leaves_, L, B, n, q32_, nullptr, 0);
        else mx_leaf32(st, LEAF_NEUMANN, d_types32_, d_leaves_, L, B, n, q32_, nullptr, 0);
        h.pe(items * (nn * 4 + 4 * n * 4), items * 2.0 * (3 * nn * n + 4 * nn), st);
    }
    for (int lvl = maxL - 1; lvl >= 0; --lvl) {
        h.pb("mx_interface", st);
        for (auto& s : hsteps_)
            if (s.level == lvl + 1) mx_coarsen(st, false, s.in32, s.out32, s.count, s.nf, B);
        for (auto& g : groups_)
            if (g.level == lvl) mx_hdiff(st, g.d_items, g.cnt, g.s, B);
        h.pe(0, 0, st);
        for (size_t gi = 0; gi < groups_.size(); ++gi) {
            const MGroup& g = groups_[gi];
            if (g.level != lvl) continue;
            const double c = g.cnt, s2 = double(g.s) * g.s;
            const std::array<int, 3> ks = h.mx_split_.empty() ? std::array<int, 3>{0, 0, 0} : h.mx_split_[gi];
            h.pb("mx_gemm_w", st);
            node_gemm(st, g, 0, B, ks[0]);
            h.pe(gemm_bytes(g, 0, B, ks[0]), c * 2.0 * 16 * s2 * B, st);
            h.pb("mx_gemm_h", st);
            node_gemm(st, g, 1, B, ks[1]);
            h.pe(gemm_bytes(g, 1, B, ks[1]), c * 2.0 * 16 * s2 * B, st);
        }
    }
    const int mroot = 4 * h.root_M();
    if (robin_) {
        // the correction's root data dg = Z (rho - b h_p), added to the state's root data
        h.pb("mx_root", st);
        mx_root_rhs(st, mroot, B, rb32_, rho32_, mn_[0].h32, rhs32_);
        GemmArgs32 ga{zA_, 0, mroot, zB_, 0, B, zC_, 0, B};
        sgemm_batched(st, mroot, B, mroot, 1.0f, ga, 0.0f, 1);
        mx_root_update(st, mroot, B, mn_[0].g32, mn_[0].g64);
        h.pe(double(mroot) * mroot * 4, 2.0 * double(mroot) * mroot * B, st);
    } else {
        // homogeneous root data for the correction
        ck(cudaMemsetAsync(mn_[0].g32, 0, sizeof(float) * size_t(mroot) * B, st), "root g32");
    }
    for (int lvl = 0; lvl < maxL; ++lvl) {
        h.pb("mx_interface", st);
        for (auto& s : gsteps_)
            if (s.level == lvl) mx_uncoarsen(st, false, s.in32, s.out32, s.count, s.nf, B);
        h.pe(0, 0, st);
        for (size_t gi = 0; gi < groups_.size(); ++gi) {
            const MGroup& g = groups_[gi];
            if (g.level != lvl) continue;
            const double c = g.cnt, s2 = double(g.s) * g.s;
            const int code = h.mx_split_.empty() ? 0 : h.mx_split_[gi][2];
            // the exterior rows go to the children unchanged (a streaming launch: in the GEMM's
            // epilogue the copy's latency sat on the epilogue warps), the GEMM writes the interface rows
            h.pb("mx_exterior", st);
            mx_ext32(st, g.d_items, g.cnt, g.s, B);
            h.pe(c * 8 * g.s * B * 8.0, 0, st);
            h.pb("mx_gemm_down", st);
            node_gemm(st, g, 2, B, code);
            h.pe(gemm_bytes(g, 2, B, code), c * 2.0 * 32 * s2 * B, st);
        }
    }
    if (direct_ && !last) {
        // the pass's interface values into the FP64 state of every node, in one launch (no residual
        // reads the state after the last pass)
        h.pb("mx_interface", st);
        mx_state_add(st, arena_, d_add_, nmis_, B);
        h.pe(double(nmis_) * B * 20.0, 0, st);
    }
    h.pb("mx_leaf_solve", st);
    if (d_fps_) mx_fp_leaf32(st, LEAF_SOLVE, d_fps_, d_leaves_, L, B, n, q32_, u64_, first ? 0 : 1);
    else mx_leaf32(st, LEAF_SOLVE, d_types32_, d_leaves_, L, B, n, q32_, u64_, first ? 0 : 1);
    // q in, the FP64 state written (and read when accumulating), the Dirichlet rows in
    h.pe(items * (nn * (first ? 12.0 : 20.0) + 4.0 * n * 4), items * 2.0 * 4 * nn * n, st);
}

void MixedSolver::solve(int B, int sweeps) {
    if (B < 1 || B > bmax_) throw std::invalid_argument("mixed solver: batch size out of range");
    if (sweeps < 0 || sweeps + 1 > kMaxPasses) throw std::invalid_argument("mixed solver: too many sweeps");
    Hps& h = H_;
    graphs_.run(st_, (long long)B * 64 + sweeps, h.graphs() && !h.prof_, [&] {
        cudaStream_t s = st_;
        ck(cudaMemsetAsync(uG_begin_, 0, uG_bytes_, s), "clear interface state");
        ck(cudaMemsetAsync(rmax_, 0, sizeof(double) * size_t(bmax_) * kMaxPasses, s), "clear residuals");
        if (robin_) ck(cudaMemsetAsync(mn_[0].g64, 0, sizeof(double) * 4 * size_t(h.root_M()) * B, s), "root g64");
        else mx_root(s, 4 * h.root_M(), B, a_, r_, mn_[0].g64);
        // 16 x 16 constant-coefficient leaves fuse each residual with the next Neumann step (the
        // exact residual in its form 0: square cells, lambda = 0); the general-leaf-residual option
        // keeps them apart, with the same bits
        const bool fuse = !d_fps_ && h.leaf_n() == 16 && !g_general_residual.load();
        for (int p = 0; p <= sweeps; ++p) {
            const bool f = fuse && (p == 0 || res_form_ == 0);
            residual(B, rmax_ + size_t(p) * bmax_, p == 0, f);
            pass(B, p == 0, f, p == sweeps);
        }
    });
}

int MixedSolver::take_error() {
    int v = 0;
    ck(cudaMemcpyAsync(&v, d_err_, sizeof(int), cudaMemcpyDeviceToHost, st_), "mixed error flag");
    ck(cudaStreamSynchronize(st_), "mixed solver");
    if (v) ck(cudaMemsetAsync(d_err_, 0, sizeof(int), st_), "mixed error flag");
    return v;
}

}  // namespace efgb
