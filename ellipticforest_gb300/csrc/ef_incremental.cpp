// Local re-factorisation after a mesh change (no counterpart in the reference, which rebuilds every
// merge): the operators of a merge node -- T, [S | X^{-1}], the compact H and the LU of X -- depend
// only on the node's subtree (its leaves, their geometry, the coarsening among its descendants).  A
// node of the new tree whose subtree is the same in the old tree copies them; only the others merge,
// with the same grouped kernels restricted to the changed nodes of each group.  The result equals a
// fresh build() bit for bit.
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "ef_hps.hpp"

namespace efgb {

namespace {

void cki(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
}

uint64_t mix64(uint64_t h, uint64_t v) {
    h ^= v + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h * 0xff51afd7ed558ccdull;
}

// subtree signature of every node: its quad and its children's signatures (leaves: the quad)
std::vector<uint64_t> signatures(const Mesh& m) {
    std::vector<uint64_t> sig(m.nodes.size(), 0);
    for (int id = int(m.nodes.size()) - 1; id >= 0; --id) {  // pre-order: children after parents
        const MeshNode& nd = m.nodes[id];
        uint64_t h = mix64(mix64(mix64(1469598103934665603ull, uint64_t(nd.level)), uint64_t(nd.ix)), uint64_t(nd.iy));
        if (!nd.leaf())
            for (int c = 0; c < 4; ++c) h = mix64(h, sig[nd.child[c]]);
        else
            h = mix64(h, 0x5bd1e995ull);
        sig[id] = h;
    }
    return sig;
}

}  // namespace

void Hps::build_from(const Hps& old) {
    if (solver_type_ != SOLVER_FISHPACK90 || old.solver_type_ != SOLVER_FISHPACK90)
        throw std::invalid_argument("incremental build: constant-coefficient (FISHPACK90) leaves only");
    if (!old.built_) throw std::invalid_argument("incremental build: the old tree is not built");
    if (old.n_ != n_ || old.lambda_ != lambda_ || old.mesh_.xl != mesh_.xl || old.mesh_.xu != mesh_.xu ||
        old.mesh_.yl != mesh_.yl || old.mesh_.yu != mesh_.yu)
        throw std::invalid_argument("incremental build: domain, patch size or lambda differ");
    root_lu_valid_ = false;
    top_level_ = -1;
    const std::vector<uint64_t> sn = signatures(mesh_), so = signatures(old.mesh_);
    std::map<std::tuple<int, int64_t, int64_t>, int> old_id;
    for (int id = 0; id < int(old.mesh_.nodes.size()); ++id) {
        const MeshNode& nd = old.mesh_.nodes[id];
        old_id[{nd.level, nd.ix, nd.iy}] = id;
    }
    // which merge nodes reuse the old operators
    std::vector<int> src(nodes_.size(), -1);
    reused_ = 0;
    for (int id = 0; id < int(nodes_.size()); ++id) {
        const MeshNode& nd = mesh_.nodes[id];
        if (nd.leaf()) continue;
        auto it = old_id.find({nd.level, nd.ix, nd.iy});
        if (it == old_id.end() || so[it->second] != sn[id] || old.mesh_.nodes[it->second].leaf()) continue;
        if (old.nodes_[it->second].s != nodes_[id].s) continue;
        src[id] = it->second;
        ++reused_;
    }
    // device tables: per group the changed nodes' merge items, pointer arrays and split-GEMM tables,
    // and one batched copy list for the reused nodes
    struct Sub {
        int cnt = 0;
        size_t items = 0, X = 0, RHS = 0, piv = 0, perm = 0, info = 0, gA = 0, gB = 0, gB2 = 0, gC = 0;
    };
    std::vector<Sub> sub(groups_.size());
    std::vector<unsigned char> host;
    auto reserve = [&](size_t bytes) {
        const size_t off = (host.size() + 255) / 256 * 256;
        host.resize(off + bytes);
        return off;
    };
    std::vector<std::vector<int>> dirty(groups_.size());
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        for (int id : groups_[gi].nodes)
            if (src[id] < 0) dirty[gi].push_back(id);
        Sub& s = sub[gi];
        s.cnt = int(dirty[gi].size());
        if (!s.cnt) continue;
        s.items = reserve(s.cnt * sizeof(MergeItem));
        s.X = reserve(s.cnt * sizeof(double*));
        s.RHS = reserve(s.cnt * sizeof(double*));
        s.piv = reserve(s.cnt * sizeof(int*));
        s.perm = reserve(s.cnt * sizeof(int*));
        s.info = reserve(s.cnt * sizeof(int));
        s.gA = reserve(8 * s.cnt * sizeof(void*));
        s.gB = reserve(8 * s.cnt * sizeof(void*));
        s.gB2 = reserve(8 * s.cnt * sizeof(void*));
        s.gC = reserve(8 * s.cnt * sizeof(void*));
    }
    // copies: (dst, src, doubles) per reused node and buffer
    std::vector<const double*> csrc;
    std::vector<double*> cdst;
    std::vector<long long> clen;
    for (int id = 0; id < int(nodes_.size()); ++id) {
        if (src[id] < 0) continue;
        const NodeDev& a = nodes_[id];
        const NodeDev& b = old.nodes_[src[id]];
        const long long s = a.s;
        cdst.push_back(a.T); csrc.push_back(b.T); clen.push_back(64 * s * s);
        cdst.push_back(a.RHS); csrc.push_back(b.RHS); clen.push_back(48 * s * s);
        cdst.push_back(a.H); csrc.push_back(b.H); clen.push_back(16 * s * s);
        cdst.push_back(a.X); csrc.push_back(b.X); clen.push_back(16 * s * s);
    }
    const size_t ncopy = cdst.size();
    const size_t c_src = reserve(ncopy * sizeof(void*)), c_dst = reserve(ncopy * sizeof(void*)),
                 c_len = reserve(ncopy * sizeof(long long));
    unsigned char* dev = nullptr;
    cki(cudaMalloc(&dev, host.size() + 256), "cudaMalloc(incremental tables)");
    static const int cb[8] = {0, 2, 1, 3, 0, 1, 2, 3};
    static const int ia[4] = {0, 1, 0, 1}, ib[4] = {2, 2, 3, 3};
    std::vector<MergeItem> all_items;
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        const Sub& s = sub[gi];
        if (!s.cnt) continue;
        // the full group's items, then the changed subset
        all_items.resize(groups_[gi].nodes.size());
        cki(cudaMemcpy(all_items.data(), groups_[gi].d_items, all_items.size() * sizeof(MergeItem), cudaMemcpyDeviceToHost),
            "items");
        std::map<int, int> pos;
        for (size_t i = 0; i < groups_[gi].nodes.size(); ++i) pos[groups_[gi].nodes[i]] = int(i);
        const size_t sz = size_t(groups_[gi].s);
        for (int k = 0; k < s.cnt; ++k) {
            const int id = dirty[gi][k];
            const NodeDev& nd = nodes_[id];
            std::memcpy(&host[s.items + k * sizeof(MergeItem)], &all_items[pos[id]], sizeof(MergeItem));
            std::memcpy(&host[s.X + k * sizeof(void*)], &nd.X, sizeof(void*));
            std::memcpy(&host[s.RHS + k * sizeof(void*)], &nd.RHS, sizeof(void*));
            std::memcpy(&host[s.piv + k * sizeof(void*)], &nd.piv, sizeof(void*));
            std::memcpy(&host[s.perm + k * sizeof(void*)], &nd.perm, sizeof(void*));
            for (int b = 0; b < 8; ++b) {
                const int c = cb[b];
                const double* A = nd.H + size_t(b) * sz * 2 * sz;
                const double* Bp = nd.RHS + size_t(ia[c]) * sz * 12 * sz;
                const double* B2 = nd.RHS + size_t(ib[c]) * sz * 12 * sz;
                double* Cp = nd.T + size_t(b) * sz * 8 * sz;
                std::memcpy(&host[s.gA + (8 * k + b) * sizeof(void*)], &A, sizeof(void*));
                std::memcpy(&host[s.gB + (8 * k + b) * sizeof(void*)], &Bp, sizeof(void*));
                std::memcpy(&host[s.gB2 + (8 * k + b) * sizeof(void*)], &B2, sizeof(void*));
                std::memcpy(&host[s.gC + (8 * k + b) * sizeof(void*)], &Cp, sizeof(void*));
            }
        }
    }
    for (size_t k = 0; k < ncopy; ++k) {
        std::memcpy(&host[c_src + k * sizeof(void*)], &csrc[k], sizeof(void*));
        std::memcpy(&host[c_dst + k * sizeof(void*)], &cdst[k], sizeof(void*));
        std::memcpy(&host[c_len + k * sizeof(long long)], &clen[k], sizeof(long long));
    }
    cki(upload_sync(st_, dev, host.data(), host.size()), "incremental tables");
    auto at = [&](size_t off) { return dev + off; };

    build_leaf_types();
    // the reused operators first: parents read their children's T when they merge
    copy_batched(st_, reinterpret_cast<const double* const*>(at(c_src)), reinterpret_cast<double* const*>(at(c_dst)),
                 reinterpret_cast<const long long*>(at(c_len)), int(ncopy));
    const int maxL = mesh_.max_level;
    for (int lvl = maxL - 1; lvl >= 0; --lvl) {
        for (size_t k = 0; k < tsteps_.size(); ++k)
            if (tsteps_[k].level == lvl + 1) coarsen_T(st_, tsteps_[k].d_in, tsteps_[k].d_out, tsteps_[k].count, tsteps_[k].nf);
        for (size_t gi = 0; gi < groups_.size(); ++gi) {
            const Group& g = groups_[gi];
            if (g.level != lvl) continue;
            const Sub& sb = sub[gi];
            if (!sb.cnt) continue;
            const int cnt = sb.cnt, s = g.s, m = 4 * s;
            auto* items = reinterpret_cast<const MergeItem*>(at(sb.items));
            auto* X = reinterpret_cast<double* const*>(at(sb.X));
            auto* RHS = reinterpret_cast<double* const*>(at(sb.RHS));
            auto* piv = reinterpret_cast<int* const*>(at(sb.piv));
            auto* perm = reinterpret_cast<int* const*>(at(sb.perm));
            int* info = reinterpret_cast<int*>(at(sb.info));
            merge_gather_xht(st_, items, cnt, s);
            cki(cudaMemsetAsync(info, 0, cnt * sizeof(int), st_), "memset info");
            dgetrf_batched(st_, m, X, m, piv, info, cnt);
            piv_to_perm(st_, m, piv, perm, cnt);
            merge_gather_rhs(st_, items, cnt, s);
            dlu_solve_permuted(st_, m, 3 * m, (const double* const*)X, m, RHS, 3 * m, cnt);
            GemmArgs ga{reinterpret_cast<const double* const*>(at(sb.gA)), 0, 2 * s,
                        reinterpret_cast<const double* const*>(at(sb.gB)), 0, 3 * m,
                        reinterpret_cast<double* const*>(at(sb.gC)), 0, 2 * m,
                        reinterpret_cast<const double* const*>(at(sb.gB2)), 0, s};
            dgemm_batched(st_, s, 2 * m, 2 * s, 1.0, ga, 1.0, 8 * cnt);
        }
    }
    cki(cudaGetLastError(), "incremental build launch");
    cki(cudaStreamSynchronize(st_), "incremental build sync");
    singular_ = leaf_singular_;
    for (size_t gi = 0; gi < groups_.size(); ++gi) {
        const Sub& sb = sub[gi];
        if (!sb.cnt) continue;
        std::vector<int> info(sb.cnt);
        cki(cudaMemcpy(info.data(), at(sb.info), sb.cnt * sizeof(int), cudaMemcpyDeviceToHost), "info");
        for (int v : info) singular_ += (v != 0);
    }
    cudaFree(dev);
    built_ = true;
}

}  // namespace efgb
