// Mixed-precision build (no counterpart in the reference): the merges of HPSAlgorithm.hpp:497-1009
// with FP32 operators -- coarsening L21 T L12, the X / H / T_LHS gathers, LU of X, [S | X^{-1}] by
// two triangular solves and T = T_LHS + H S -- on the same plan and index maps as the FP64 build.
// The interface matrices of the top tree levels, whose conditioning grows with the interface
// length, are factored in FP64 (the gathered X widened, factored with partial pivoting, the factors
// rounded back to FP32).  The FP32 S, X^{-1} and H feed the mixed block solver, whose FP64
// residual makes the result independent of the operators' precision.
#include <algorithm>
#include <stdexcept>
#include <string>

#include "ef_hps.hpp"

namespace efgb {

namespace {

struct Carver32 {
    char* base = nullptr;
    size_t off = 0;
    template <class T>
    T* get(size_t count) {
        T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
        off += (std::max<size_t>(count, 1) * sizeof(T) + 255) / 256 * 256;
        return p;
    }
};

void ck32(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

template <class T>
void upload(cudaStream_t st, T* dst, const std::vector<T>& src, const char* what) {
    if (!src.empty()) ck32(upload_sync(st, dst, src.data(), src.size() * sizeof(T)), what);
}

}  // namespace

void Hps::allocate32() {
    const int N = int(nodes_.size());
    const int nn = n_ * n_;
    std::vector<float*> typeT(types_.size());
    auto layout = [&](Carver32& cv) {
        for (size_t t = 0; t < types_.size(); ++t) typeT[t] = cv.get<float>(size_t(16) * nn);
        n32_.assign(N, Node32());
        for (int id = 0; id < N; ++id) {
            const NodeDev& nd = nodes_[id];
            Node32& m = n32_[id];
            if (mesh_.nodes[id].leaf()) {
                m.T = typeT[nd.leaf_type];
            } else {
                const size_t s = nd.s;
                m.T = cv.get<float>(64 * s * s);
                m.X = cv.get<float>(16 * s * s);
                m.RHS = cv.get<float>(48 * s * s);
                m.H = cv.get<float>(16 * s * s);
            }
            for (int t = 0; t < nd.ncoarsen; ++t) {
                const size_t nc = size_t(nd.nx >> t) / 2;
                m.Tsteps.push_back(cv.get<float>(16 * nc * nc));
            }
            m.Tc = nd.ncoarsen ? m.Tsteps.back() : m.T;
        }
        g32_.assign(groups_.size(), Group32());
        for (size_t gi = 0; gi < groups_.size(); ++gi) {
            const int cnt = int(groups_[gi].nodes.size());
            Group32& g = g32_[gi];
            g.d_items = cv.get<MergeItem32>(cnt);
            g.d_X = cv.get<float*>(cnt);
            g.d_RHS = cv.get<float*>(cnt);
            g.d_gA = cv.get<const float*>(8 * cnt);
            g.d_gB = cv.get<const float*>(8 * cnt);
            g.d_gB2 = cv.get<const float*>(8 * cnt);
            g.d_gC = cv.get<float*>(8 * cnt);
        }
        t32_.assign(tsteps_.size(), Step32());
        for (size_t k = 0; k < tsteps_.size(); ++k) {
            t32_[k].d_in = cv.get<const float*>(tsteps_[k].count);
            t32_[k].d_out = cv.get<float*>(tsteps_[k].count);
        }
        d_tT64_ = cv.get<const double*>(types_.size());
        d_tT32_ = cv.get<float*>(types_.size());
    };
    Carver32 dry;
    layout(dry);
    arena32_bytes_ = dry.off;
    ck32(cudaMalloc(&arena32_, arena32_bytes_), "cudaMalloc(FP32 operators)");
    Carver32 real;
    real.base = arena32_;
    layout(real);

    // pointer tables
    std::vector<const double*> t64(types_.size());
    for (size_t t = 0; t < types_.size(); ++t) t64[t] = types_[t].T;
    upload(st_, d_tT64_, t64, "type T64");
    upload(st_, d_tT32_, typeT, "type T32");
    static const int cb[8] = {0, 2, 1, 3, 0, 1, 2, 3};
    static const int ia[4] = {0, 1, 0, 1}, ib[4] = {2, 2, 3, 3};
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        const Group& g = groups_[gi];
        const int cnt = int(g.nodes.size());
        const size_t sz = size_t(g.s);
        std::vector<MergeItem32> mi(cnt);
        std::vector<float*> X(cnt), R(cnt);
        std::vector<const float*> gA(8 * cnt), gB(8 * cnt), gB2(8 * cnt);
        std::vector<float*> gC(8 * cnt);
        for (int i = 0; i < cnt; ++i) {
            const int id = g.nodes[i];
            const Node32& m = n32_[id];
            const NodeDev& nd = nodes_[id];
            MergeItem32 it{};
            for (int c = 0; c < 4; ++c) it.Tc[c] = n32_[mesh_.nodes[id].child[c]].Tc;
            it.X = m.X;
            it.piv = nd.piv;
            it.perm = nd.perm;
            it.RHS = m.RHS;
            it.H = m.H;
            it.T = m.T;
            mi[i] = it;
            X[i] = m.X;
            R[i] = m.RHS;
            for (int b = 0; b < 8; ++b) {
                const int c = cb[b];
                gA[8 * i + b] = m.H + size_t(b) * sz * 2 * sz;
                gB[8 * i + b] = m.RHS + size_t(ia[c]) * sz * 12 * sz;
                gB2[8 * i + b] = m.RHS + size_t(ib[c]) * sz * 12 * sz;
                gC[8 * i + b] = m.T + size_t(b) * sz * 8 * sz;
            }
        }
        const Group32& g3 = g32_[gi];
        upload(st_, g3.d_items, mi, "items32");
        upload(st_, g3.d_X, X, "X32");
        upload(st_, g3.d_RHS, R, "RHS32");
        upload(st_, g3.d_gA, gA, "gA32");
        upload(st_, g3.d_gB, gB, "gB32");
        upload(st_, g3.d_gB2, gB2, "gB2_32");
        upload(st_, g3.d_gC, gC, "gC32");
    }
    for (size_t k = 0; k < tsteps_.size(); ++k) {
        const int t = step_index_t_[k];
        std::vector<const float*> in;
        std::vector<float*> out;
        for (int id : step_nodes_t_[k]) {
            const Node32& m = n32_[id];
            in.push_back(t == 0 ? m.T : m.Tsteps[t - 1]);
            out.push_back(m.Tsteps[t]);
        }
        upload(st_, t32_[k].d_in, in, "tin32");
        upload(st_, t32_[k].d_out, out, "tout32");
    }
}

void Hps::build_mixed(int fp64_levels) {
    top_level_ = -1;
    if (fp64_levels < 0) throw std::invalid_argument("mixed build: fp64_levels must be >= 0");
    if (!arena32_) allocate32();
    build_leaf_types();
    const int n = n_;
    pb("mx_build_leaf_convert");
    narrow_batched(st_, d_tT64_, d_tT32_, 16LL * n * n, int(types_.size()));
    pe(double(types_.size()) * 16 * n * n * 12, 0);
    const int maxL = mesh_.max_level;
    for (int lvl = maxL - 1; lvl >= 0; --lvl) {
        for (size_t k = 0; k < tsteps_.size(); ++k)
            if (tsteps_[k].level == lvl + 1) {
                const double nf = tsteps_[k].nf, cnt = tsteps_[k].count;
                pb("mx_build_coarsen_T");
                coarsen_T32(st_, t32_[k].d_in, t32_[k].d_out, tsteps_[k].count, tsteps_[k].nf);
                pe(cnt * 4 * (16 * nf * nf + 4 * nf * nf), cnt * 4 * nf * nf * 10);
            }
        for (size_t gi = 0; gi < groups_.size(); ++gi) {
            const Group& g = groups_[gi];
            if (g.level != lvl) continue;
            const Group32& g3 = g32_[gi];
            const int cnt = int(g.nodes.size()), s = g.s, m = 4 * s;
            const double c = cnt, dm = m;
            pb("mx_build_gather");
            merge_gather_xht32(st_, g3.d_items, cnt, s);
            pe(c * 4 * (dm * dm + 2 * dm * dm + 4 * dm * dm) * 1.5, 0);
            ck32(cudaMemsetAsync(g.d_info, 0, cnt * sizeof(int), st_), "memset info");
            if (lvl < fp64_levels) {
                pb("mx_build_getrf_fp64");
                widen_batched(st_, (const float* const*)g3.d_X, g.d_X, (long long)m * m, cnt);
                dgetrf_batched(st_, m, g.d_X, m, g.d_piv, g.d_info, cnt);
                narrow_batched(st_, (const double* const*)g.d_X, g3.d_X, (long long)m * m, cnt);
                pe(c * 12 * 2 * dm * dm, c * 2.0 / 3.0 * dm * dm * dm);
            } else {
                pb("mx_build_getrf");
                sgetrf_batched(st_, m, g3.d_X, m, g.d_piv, g.d_info, cnt);
                pe(c * 4 * 2 * dm * dm, c * 2.0 / 3.0 * dm * dm * dm);
            }
            piv_to_perm(st_, m, g.d_piv, g.d_perm, cnt);
            pb("mx_build_gather");
            merge_gather_rhs32(st_, g3.d_items, cnt, s);
            pe(c * 4 * (3 * dm * dm + dm * dm), 0);
            pb("mx_build_lu_solve");
            slu_solve_permuted(st_, m, 3 * m, (const float* const*)g3.d_X, m, g3.d_RHS, 3 * m, cnt);
            pe(c * 4 * (dm * dm + 2 * 3 * dm * dm), c * 2.0 * dm * dm * 3 * dm);
            pb("mx_build_gemm_T");
            GemmArgs32 ga{g3.d_gA, 0, 2 * s, g3.d_gB, 0, 3 * m, g3.d_gC, 0, 2 * m, g3.d_gB2, 0, s};
            sgemm_batched(st_, s, 2 * m, 2 * s, 1.0f, ga, 1.0f, 8 * cnt);
            pe(c * 4 * (dm * dm / 2 + dm * 2 * dm + 2 * 4 * dm * dm), c * 2.0 * (2 * dm) * (2 * dm) * (dm / 2));
        }
    }
    ck32(cudaGetLastError(), "mixed build launch");
    ck32(cudaStreamSynchronize(st_), "mixed build sync");
    singular_ = leaf_singular_;
    for (auto& g : groups_) {
        std::vector<int> info(g.nodes.size());
        ck32(cudaMemcpy(info.data(), g.d_info, info.size() * sizeof(int), cudaMemcpyDeviceToHost), "info");
        for (int v : info) singular_ += (v != 0);
    }
    built32_ = true;
}

}  // namespace efgb
