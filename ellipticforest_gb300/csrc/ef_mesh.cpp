// Host-side quadtree: refinement, 2:1 corner balance and node layout.
// Restates src/Mesh.hpp:111-180 (refineByFunction), the p4est calls it makes, and the node
// geometry of src/Patches/FiniteVolume/FiniteVolumeNodeFactory.cpp:15-66.
#include "ef_mesh.hpp"

#include <algorithm>
#include <stdexcept>
#include <unordered_set>

namespace efgb {

namespace {

constexpr int kMaxLevel = 30;                      // P4EST_MAXLEVEL
constexpr double kRootLen = double(1LL << kMaxLevel);  // P4EST_ROOT_LEN

inline uint64_t key_of(int level, int64_t ix, int64_t iy) {
    return (uint64_t(level) << 58) | (uint64_t(ix) << 29) | uint64_t(iy);
}

// Bilinear vertex interpolation of one square tree: p4est_qcoord_to_vertex on the connectivity
// built by p4est_connectivity_new_square_domain (P4est.cpp:7-33).
void qcoord_to_vertex(double xl, double xu, double yl, double yu, int64_t qx, int64_t qy,
                      double* vx, double* vy) {
    const double wx1 = double(qx) / kRootLen, wx0 = 1.0 - wx1;
    const double wy1 = double(qy) / kRootLen, wy0 = 1.0 - wy1;
    const double X[4] = {xl, xu, xl, xu};
    const double Y[4] = {yl, yl, yu, yu};
    const double wy[2] = {wy0, wy1}, wx[2] = {wx0, wx1};
    double ax = 0.0, ay = 0.0;
    int k = 0;
    for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a, ++k) {
            const double f = wy[b] * wx[a];
            ax += f * X[k];
            ay += f * Y[k];
        }
    *vx = ax;
    *vy = ay;
}

// The p4est_refine callback of Mesh.hpp:135-162.
bool refine_test(const std::function<bool(double, double)>& fn, double xl, double xu, double yl,
                 double yu, int nx, int ny, const Quad& q, int max_level) {
    if (q.level >= max_level) return false;
    const int64_t qlen = int64_t(1) << (kMaxLevel - q.level);
    double x0, y0, x1, y1;
    qcoord_to_vertex(xl, xu, yl, yu, q.ix * qlen, q.iy * qlen, &x0, &y0);
    qcoord_to_vertex(xl, xu, yl, yu, q.ix * qlen + qlen, q.iy * qlen + qlen, &x1, &y1);
    const double dx = (x1 - x0) / nx, dy = (y1 - y0) / ny;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            if (fn(x0 + (i + 0.5) * dx, y0 + (j + 0.5) * dy)) return true;
    return false;
}

}  // namespace

std::vector<Quad> corner_balance(const std::vector<Quad>& in) {
    std::unordered_set<uint64_t> set;
    set.reserve(in.size() * 2);
    for (const Quad& q : in) set.insert(key_of(q.level, q.ix, q.iy));

    auto find_leaf = [&](int level, int64_t ix, int64_t iy, Quad* out) {
        for (int l = level; l >= 0; --l) {
            const int s = level - l;
            if (set.count(key_of(l, ix >> s, iy >> s))) {
                *out = Quad{l, ix >> s, iy >> s};
                return true;
            }
        }
        return false;
    };

    bool changed = true;
    while (changed) {
        changed = false;
        std::vector<Quad> cur;
        cur.reserve(set.size());
        for (uint64_t k : set)
            cur.push_back(Quad{int(k >> 58), int64_t((k >> 29) & ((1ULL << 29) - 1)),
                               int64_t(k & ((1ULL << 29) - 1))});
        std::sort(cur.begin(), cur.end(), [](const Quad& a, const Quad& b) {
            if (a.level != b.level) return a.level > b.level;
            if (a.ix != b.ix) return a.ix < b.ix;
            return a.iy < b.iy;
        });
        for (const Quad& q : cur) {
            if (!set.count(key_of(q.level, q.ix, q.iy))) continue;
            if (q.level < 2) continue;
            const int64_t n = int64_t(1) << q.level;
            for (int dxo = -1; dxo <= 1; ++dxo)
                for (int dyo = -1; dyo <= 1; ++dyo) {
                    if (!dxo && !dyo) continue;
                    const int64_t jx = q.ix + dxo, jy = q.iy + dyo;
                    if (jx < 0 || jy < 0 || jx >= n || jy >= n) continue;
                    Quad nb;
                    if (!find_leaf(q.level, jx, jy, &nb)) continue;
                    if (nb.level >= q.level - 1) continue;
                    set.erase(key_of(nb.level, nb.ix, nb.iy));
                    for (int c = 0; c < 4; ++c)
                        set.insert(key_of(nb.level + 1, 2 * nb.ix + (c & 1), 2 * nb.iy + (c >> 1)));
                    changed = true;
                }
        }
    }
    std::vector<Quad> out;
    out.reserve(set.size());
    for (uint64_t k : set)
        out.push_back(Quad{int(k >> 58), int64_t((k >> 29) & ((1ULL << 29) - 1)),
                           int64_t(k & ((1ULL << 29) - 1))});
    return out;
}

Mesh Mesh::refine_by_function(double xl, double xu, double yl, double yu, int nx, int ny,
                              int min_level, int max_level,
                              const std::function<bool(double, double)>& fn) {
    if (nx <= 0 || ny <= 0 || min_level < 0 || max_level > 28 || min_level > max_level)
        throw std::invalid_argument("refine_by_function: bad arguments");
    std::vector<Quad> leaves, stack;
    const int64_t m = int64_t(1) << min_level;
    for (int64_t ix = 0; ix < m; ++ix)
        for (int64_t iy = 0; iy < m; ++iy) stack.push_back(Quad{min_level, ix, iy});
    while (!stack.empty()) {
        Quad q = stack.back();
        stack.pop_back();
        if (refine_test(fn, xl, xu, yl, yu, nx, ny, q, max_level)) {
            for (int c = 0; c < 4; ++c)
                stack.push_back(Quad{q.level + 1, 2 * q.ix + (c & 1), 2 * q.iy + (c >> 1)});
        } else {
            leaves.push_back(q);
        }
    }
    return from_leaves(xl, xu, yl, yu, nx, ny, corner_balance(leaves));
}

Mesh Mesh::uniform(double xl, double xu, double yl, double yu, int nx, int ny, int level) {
    if (level < 0 || level > 14) throw std::invalid_argument("uniform: bad level");
    std::vector<Quad> leaves;
    const int64_t m = int64_t(1) << level;
    for (int64_t ix = 0; ix < m; ++ix)
        for (int64_t iy = 0; iy < m; ++iy) leaves.push_back(Quad{level, ix, iy});
    return from_leaves(xl, xu, yl, yu, nx, ny, leaves);
}

Mesh Mesh::from_leaves(double xl, double xu, double yl, double yu, int nx, int ny,
                       const std::vector<Quad>& leaves) {
    Mesh m;
    m.xl = xl; m.xu = xu; m.yl = yl; m.yu = yu;
    m.nx = nx; m.ny = ny;
    m.build_nodes(leaves);
    return m;
}

void Mesh::build_nodes(const std::vector<Quad>& leaf_list) {
    std::unordered_set<uint64_t> leafset, internal;
    for (const Quad& q : leaf_list) {
        leafset.insert(key_of(q.level, q.ix, q.iy));
        for (int l = q.level - 1; l >= 0; --l) {
            const int s = q.level - l;
            internal.insert(key_of(l, q.ix >> s, q.iy >> s));
        }
    }
    for (uint64_t k : leafset)
        if (internal.count(k)) throw std::invalid_argument("mesh: leaf set is not a partition");
    nodes.clear();
    leaves.clear();
    max_level = 0;
    // Pre-order construction with the NodeFactory's midpoint geometry.
    struct Item { int level; int64_t ix, iy; int parent; int sibling; };
    std::vector<Item> stack{{0, 0, 0, -1, 0}};
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        MeshNode nd;
        nd.level = it.level;
        nd.ix = it.ix;
        nd.iy = it.iy;
        nd.parent = it.parent;
        if (it.parent < 0) {
            nd.xl = xl; nd.xu = xu; nd.yl = yl; nd.yu = yu;
        } else {
            const MeshNode& p = nodes[it.parent];
            const double xm = (p.xl + p.xu) / 2.0, ym = (p.yl + p.yu) / 2.0;
            const int s = it.sibling;
            nd.xl = (s & 1) ? xm : p.xl;
            nd.xu = (s & 1) ? p.xu : xm;
            nd.yl = (s & 2) ? ym : p.yl;
            nd.yu = (s & 2) ? p.yu : ym;
        }
        const int id = int(nodes.size());
        if (it.parent >= 0) nodes[it.parent].child[it.sibling] = id;
        const uint64_t k = key_of(it.level, it.ix, it.iy);
        if (leafset.count(k)) {
            nd.leaf_index = int(leaves.size());
            leaves.push_back(id);
            max_level = std::max(max_level, it.level);
            nodes.push_back(nd);
        } else if (internal.count(k)) {
            nodes.push_back(nd);
            for (int c = 3; c >= 0; --c)
                stack.push_back(Item{it.level + 1, 2 * it.ix + (c & 1), 2 * it.iy + (c >> 1), id, c});
        } else {
            throw std::invalid_argument("mesh: leaves do not cover the root");
        }
    }
}

std::string Mesh::path(int node) const {
    std::string p;
    int cur = node;
    while (nodes[cur].parent >= 0) {
        const MeshNode& nd = nodes[cur];
        const int cid = int((nd.ix & 1) | ((nd.iy & 1) << 1));
        p.insert(p.begin(), char('0' + cid));
        cur = nd.parent;
    }
    return "0" + p;
}

}  // namespace efgb
