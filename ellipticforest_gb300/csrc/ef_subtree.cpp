// Subtree split of one tree over several GPUs (no counterpart in this form in the reference, whose
// MPI build broadcasts whole child patches across the process boundary inside merge4to1:
// src/Quadtree.hpp:470-496, :146-148).
//
// With P = 4^k processes, process p owns the level-k subtree p: it builds, upward-passes and solves
// it as a tree of its own (a Mesh whose root is that node, so every patch box, leaf DtN and merge is
// the one of the full tree).  One process holds a handle on the full mesh and runs only the top k
// levels on the gathered level-k operators:
//   build : T of every level-k node (4m x 4m, m = the node's side)  ->  merges of levels k-1 .. 0
//   solve : h of every level-k node (4m)  ->  upward pass of levels k-1 .. 0, root data, downward
//           pass to level k  ->  g of every level-k node (4m), which its owner's subtree solves with
//           as Dirichlet root data.
// The kernels see the same operands as in a single-handle build and solve, so the results are the
// same bit for bit.  The exchange itself (gather of T and h, scatter of g) is the caller's: any
// transport works (NCCL or plain peer copies on device memory, or host memory).
#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "ef_hps.hpp"
#include "ef_mesh.hpp"

namespace efgb {

std::vector<int> level_nodes(const Mesh& m, int level) {
    std::vector<int> ids;
    for (int id = 0; id < int(m.nodes.size()); ++id)
        if (m.nodes[id].level == level) ids.push_back(id);
    return ids;  // pre-order = z-order among the nodes of one level
}

Mesh subtree_mesh(const Mesh& m, int level, int index) {
    const std::vector<int> ids = level_nodes(m, level);
    if (index < 0 || index >= int(ids.size()))
        throw std::invalid_argument("subtree: index out of range (" + std::to_string(ids.size()) +
                                    " nodes at level " + std::to_string(level) + ")");
    const MeshNode& top = m.nodes[ids[index]];
    std::vector<Quad> leaves;
    for (int leaf : m.leaves) {
        const MeshNode& nd = m.nodes[leaf];
        if (nd.level < level) continue;
        const int d = nd.level - level;
        if ((nd.ix >> d) != top.ix || (nd.iy >> d) != top.iy) continue;
        leaves.push_back(Quad{d, nd.ix - (top.ix << d), nd.iy - (top.iy << d)});
    }
    // the node's box, halved by the same midpoint rule as in the full mesh, reproduces every patch
    // box of the subtree exactly
    return Mesh::from_leaves(top.xl, top.xu, top.yl, top.yu, m.nx, m.ny, leaves);
}

std::vector<int> Hps::split_nodes(int level) const {
    if (level < 1) throw std::invalid_argument("subtree split: the level must be at least 1");
    for (int leaf : mesh_.leaves)
        if (mesh_.nodes[leaf].level <= level)
            throw std::invalid_argument("subtree split: every leaf must lie below the split level " +
                                        std::to_string(level));
    return level_nodes(mesh_, level);
}

std::vector<int> Hps::split_sizes(int level) const {
    std::vector<int> out;
    for (int id : split_nodes(level)) out.push_back(4 * nodes_[id].nx);
    return out;
}

void Hps::build_top(int level, const double* const* T_host) {
    const std::vector<int> ids = split_nodes(level);
    root_lu_valid_ = false;
    built_ = false;
    for (size_t k = 0; k < ids.size(); ++k) {
        const NodeDev& nd = nodes_[ids[k]];
        const size_t m = 4 * size_t(nd.nx);
        if (!T_host[k]) throw std::invalid_argument("build_top: null T block");
        check(cudaMemcpyAsync(nd.T, T_host[k], m * m * sizeof(double), cudaMemcpyHostToDevice, st_), "copy T block");
    }
    merge_levels(level - 1);
    check(cudaGetLastError(), "top build launch");
    check(cudaStreamSynchronize(st_), "top build sync");
    singular_ = count_singular(level);
    top_level_ = level;
    built_ = true;
}

void Hps::upwards_top(int level, const double* const* h_host) {
    if (top_level_ != level) throw std::invalid_argument("upwards_top: the tree was not built with build_top at this level");
    const std::vector<int> ids = split_nodes(level);
    for (size_t k = 0; k < ids.size(); ++k) {
        const NodeDev& nd = nodes_[ids[k]];
        if (!h_host[k]) throw std::invalid_argument("upwards_top: null h block");
        check(cudaMemcpyAsync(nd.h, h_host[k], 4 * size_t(nd.nx) * sizeof(double), cudaMemcpyHostToDevice, st_),
              "copy h block");
    }
    upward_levels(level - 1);
    check(cudaGetLastError(), "top upward launch");
    check(cudaStreamSynchronize(st_), "top upward sync");
}

void Hps::solve_top(int level, double* const* g_host) {
    if (top_level_ != level) throw std::invalid_argument("solve_top: the tree was not built with build_top at this level");
    const std::vector<int> ids = split_nodes(level);
    root_from_bc();
    downward_levels(level, true);
    for (size_t k = 0; k < ids.size(); ++k) {
        const NodeDev& nd = nodes_[ids[k]];
        if (!g_host[k]) throw std::invalid_argument("solve_top: null g block");
        check(cudaMemcpyAsync(g_host[k], nd.gf, 4 * size_t(nd.nx) * sizeof(double), cudaMemcpyDeviceToHost, st_),
              "copy g block");
    }
    check(cudaGetLastError(), "top solve launch");
    check(cudaStreamSynchronize(st_), "top solve sync");
}

}  // namespace efgb
