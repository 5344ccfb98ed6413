// Host-side quadtree of the GB300 HPS solver.
//
// Replaces the p4est-backed Mesh/Quadtree pair of the reference (src/Mesh.hpp:111-180,
// src/Quadtree.hpp:120-360) with a flat node array: no p4est, no MPI, no path-string map on the
// hot path.  Node 0 is the root; nodes are stored in pre-order (children in z-order 0=SW, 1=SE,
// 2=NW, 3=NE, as p4est_quadrant_child_id numbers them), so leaves appear in the same order as
// Quadtree::traversePreOrder visits them.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace efgb {

struct Quad {
    int level;
    int64_t ix, iy;
};

struct MeshNode {
    int level = 0;
    int64_t ix = 0, iy = 0;      // integer coordinates at `level`
    int parent = -1;
    int child[4] = {-1, -1, -1, -1};
    int leaf_index = -1;         // position in leaf order, -1 for internal nodes
    // Patch box from repeated midpoint halving (FiniteVolumeNodeFactory.cpp:15-66).
    double xl = 0, xu = 0, yl = 0, yu = 0;
    bool leaf() const { return child[0] < 0; }
};

class Mesh {
public:
    double xl = 0, xu = 0, yl = 0, yu = 0;  // root box
    int nx = 0, ny = 0;                      // cells per leaf patch side
    std::vector<MeshNode> nodes;             // pre-order
    std::vector<int> leaves;                 // node ids of leaves, pre-order
    int max_level = 0;

    // p4est_new_ext(min_level, uniform) + recursive p4est_refine with the cell-centre test of
    // Mesh.hpp:135-162 + p4est_balance(P4EST_CONNECT_CORNER).
    static Mesh refine_by_function(double xl, double xu, double yl, double yu, int nx, int ny,
                                   int min_level, int max_level,
                                   const std::function<bool(double, double)>& fn);
    static Mesh uniform(double xl, double xu, double yl, double yu, int nx, int ny, int level);
    static Mesh from_leaves(double xl, double xu, double yl, double yu, int nx, int ny,
                            const std::vector<Quad>& leaves);

    std::string path(int node) const;  // p4est_quadrant_path (P4est.cpp:35-43)

private:
    void build_nodes(const std::vector<Quad>& leaves);
};

// Node ids at `level` in pre-order (z-order), and the mesh of the subtree under the index-th of
// them: its root box is that node's box and its leaves keep their patch boxes bit for bit.
std::vector<int> level_nodes(const Mesh& m, int level);
Mesh subtree_mesh(const Mesh& m, int level, int index);

// Coarsest refinement of `leaves` in which face- and corner-neighbours differ by at most one level.
std::vector<Quad> corner_balance(const std::vector<Quad>& leaves);

}  // namespace efgb
