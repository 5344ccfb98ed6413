// Quadtree and mesh of the C++ drop-in: Node<T>, AbstractNodeFactory<T>, FiniteVolumeNodeFactory,
// Quadtree<T> and Mesh<T> with the reference's traversal and refinement API (src/QuadNode.hpp,
// src/AbstractNodeFactory.hpp, src/Quadtree.hpp:236-360, src/Mesh.hpp:111-180,
// src/Patches/FiniteVolume/FiniteVolumeNodeFactory.cpp:15-93).  The tree shape comes from the
// library's refine-and-balance (ef_mesh_create_refined); the nodes are host objects for drivers.
#pragma once

#include "VTK.hpp"

#include <algorithm>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "FiniteVolume.hpp"

namespace EllipticForest {

template <typename T>
class Node : public MPI::MPIObject {
public:
    T data;
    std::string path;
    int level = 0;
    int pfirst = 0;
    int plast = 0;
    bool leaf = false;

    Node() : MPIObject(MPI_COMM_WORLD) {}
    Node(MPI::Communicator comm, T d, std::string p, int lvl, int pf, int pl)
        : MPIObject(comm), data(std::move(d)), path(std::move(p)), level(lvl), pfirst(pf), plast(pl) {}
    bool isOwned() const { return true; }
    std::string str() const {
        return "node: path = " + path + ", level = " + std::to_string(level) + ", ranks = [" +
               std::to_string(pfirst) + "-" + std::to_string(plast) + "]";
    }
};

template <typename T>
class AbstractNodeFactory {
public:
    virtual ~AbstractNodeFactory() = default;
    virtual Node<T>* createNode(T data, std::string path, int level, int pfirst, int plast) = 0;
    virtual Node<T>* createChildNode(Node<T>* parent, int sibling_id, int pfirst, int plast) = 0;
    virtual Node<T>* createParentNode(std::vector<Node<T>*> children, int pfirst, int plast) = 0;
};

// FiniteVolumeNodeFactory.cpp:11-93: children split the parent box at its midpoints, keeping nx.
class FiniteVolumeNodeFactory : public MPI::MPIObject, public AbstractNodeFactory<FiniteVolumePatch> {
public:
    FiniteVolumeNodeFactory() = default;
    explicit FiniteVolumeNodeFactory(MPI::Communicator comm) : MPIObject(comm) {}

    Node<FiniteVolumePatch>* createNode(FiniteVolumePatch data, std::string path, int level, int pfirst,
                                        int plast) override {
        return new Node<FiniteVolumePatch>(getComm(), data, path, level, pfirst, plast);
    }
    Node<FiniteVolumePatch>* createChildNode(Node<FiniteVolumePatch>* parent, int sibling_id, int pfirst,
                                             int plast) override {
        auto& pg = parent->data.grid();
        const int nx = int(pg.nx()), ny = int(pg.ny());
        const double xl = pg.xLower(), xu = pg.xUpper(), yl = pg.yLower(), yu = pg.yUpper();
        const double xm = (xl + xu) / 2.0, ym = (yl + yu) / 2.0;
        FiniteVolumeGrid g;
        switch (sibling_id) {
            case 0: g = FiniteVolumeGrid(getComm(), nx, xl, xm, ny, yl, ym); break;
            case 1: g = FiniteVolumeGrid(getComm(), nx, xm, xu, ny, yl, ym); break;
            case 2: g = FiniteVolumeGrid(getComm(), nx, xl, xm, ny, ym, yu); break;
            default: g = FiniteVolumeGrid(getComm(), nx, xm, xu, ny, ym, yu); break;
        }
        return new Node<FiniteVolumePatch>(getComm(), FiniteVolumePatch(getComm(), g),
                                           parent->path + std::to_string(sibling_id), parent->level + 1, pfirst,
                                           plast);
    }
    Node<FiniteVolumePatch>* createParentNode(std::vector<Node<FiniteVolumePatch>*> ch, int pfirst,
                                              int plast) override {
        auto& g0 = ch[0]->data.grid();
        FiniteVolumeGrid g(getComm(), int(g0.nx()), g0.xLower(), ch[1]->data.grid().xUpper(), int(g0.ny()),
                           g0.yLower(), ch[2]->data.grid().yUpper());
        return new Node<FiniteVolumePatch>(getComm(), FiniteVolumePatch(getComm(), g),
                                           ch[0]->path.substr(0, ch[0]->path.size() - 1), ch[0]->level - 1,
                                           pfirst, plast);
    }
};

template <typename T>
class Quadtree : public MPI::MPIObject {
public:
    using NodeMap = std::map<std::string, Node<T>*>;
    NodeMap map;

    Quadtree() = default;
    Quadtree(const Quadtree&) = delete;
    Quadtree& operator=(const Quadtree&) = delete;
    Quadtree(Quadtree&& o) noexcept : map(std::move(o.map)) { o.map.clear(); }
    Quadtree& operator=(Quadtree&& o) noexcept {
        if (this != &o) {
            clear();
            map = std::move(o.map);
            o.map.clear();
        }
        return *this;
    }
    ~Quadtree() { clear(); }

    void clear() {
        for (auto& kv : map) delete kv.second;
        map.clear();
    }

    T& root() { return map.at("0")->data; }

    void traversePreOrder(std::function<int(Node<T>*)> visit) { pre(map.at("0"), visit); }
    void traversePreOrder(std::function<void(T&)> visit) {
        pre(map.at("0"), [&](Node<T>* n) { visit(n->data); return 1; });
    }
    void traversePostOrder(std::function<int(Node<T>*)> visit) { post(map.at("0"), visit); }
    void traversePostOrder(std::function<void(T&)> visit) {
        post(map.at("0"), [&](Node<T>* n) { visit(n->data); return 1; });
    }

    // Quadtree.hpp:322-360: families in post-order (merge) or pre-order (split)
    void merge(std::function<int(Node<T>*)> leaf, std::function<int(Node<T>*, std::vector<Node<T>*>)> family) {
        mergeRec(map.at("0"), leaf, family);
    }
    void split(std::function<int(Node<T>*)> leaf, std::function<int(Node<T>*, std::vector<Node<T>*>)> family) {
        splitRec(map.at("0"), leaf, family);
    }

    std::vector<Node<T>*> children(Node<T>* n) {
        std::vector<Node<T>*> c(4);
        for (int i = 0; i < 4; ++i) c[i] = map.at(n->path + std::to_string(i));
        return c;
    }

private:
    void pre(Node<T>* n, const std::function<int(Node<T>*)>& v) {
        v(n);
        if (!n->leaf)
            for (auto* c : children(n)) pre(c, v);
    }
    void post(Node<T>* n, const std::function<int(Node<T>*)>& v) {
        if (!n->leaf)
            for (auto* c : children(n)) post(c, v);
        v(n);
    }
    void mergeRec(Node<T>* n, const std::function<int(Node<T>*)>& leaf,
                  const std::function<int(Node<T>*, std::vector<Node<T>*>)>& family) {
        if (n->leaf) { leaf(n); return; }
        auto ch = children(n);
        for (auto* c : ch) mergeRec(c, leaf, family);
        family(n, ch);
    }
    void splitRec(Node<T>* n, const std::function<int(Node<T>*)>& leaf,
                  const std::function<int(Node<T>*, std::vector<Node<T>*>)>& family) {
        if (n->leaf) { leaf(n); return; }
        auto ch = children(n);
        family(n, ch);
        for (auto* c : ch) splitRec(c, leaf, family);
    }
};

template <typename PatchType>
class Mesh : public MPI::MPIObject {
public:
    Quadtree<PatchType> quadtree;

    Mesh() : MPIObject(MPI_COMM_WORLD) {}
    Mesh(const Mesh&) = delete;
    Mesh& operator=(const Mesh&) = delete;
    ~Mesh() {
        if (handle_) ef_mesh_destroy(handle_);
    }

    // Mesh.hpp:111-180: uniform to min_level, refine every patch with a cell centre where fn holds
    // (up to max_level), 2:1 corner balance; then the node tree with the factory's geometry.
    void refineByFunction(std::function<bool(double x, double y)> fn, double threshold, int min_level,
                          int max_level, PatchType& root_patch, AbstractNodeFactory<PatchType>& node_factory) {
        (void)threshold;  // the reference stores it but its refinement test is fn alone
        auto& g = root_patch.grid();
        ef_mesh* h = nullptr;
        efCheck(ef_mesh_create_refined(g.xLower(), g.xUpper(), g.yLower(), g.yUpper(), int(g.nx()), int(g.ny()),
                                       min_level, max_level, &Mesh::tramp, &fn, &h),
                "Mesh::refineByFunction");
        adopt(h, root_patch, node_factory);
    }

    void iteratePatches(std::function<void(PatchType&)> fn) {
        quadtree.traversePreOrder([&](Node<PatchType>* n) {
            if (n->leaf) fn(n->data);
            return 1;
        });
    }
    void iterateCells(std::function<void(double, double)> fn) {
        iteratePatches([&](PatchType& p) {
            auto& g = p.grid();
            for (std::size_t i = 0; i < g.nx(); ++i)
                for (std::size_t j = 0; j < g.ny(); ++j) fn(g(0, i), g(1, j));
        });
    }

    ef_mesh* handle() const { return handle_; }
    // leaves in pre-order (the order of the library's leaf arrays)
    std::vector<Node<PatchType>*>& leaves() { return leaves_; }

    // Mesh.hpp:357-390: cell data for toVTK, in leaf order with cell index j + i*ny (as vectorU)
    void addMeshFunction(Vector<double>& meshFunction) {
        const std::string nm = meshFunction.name().empty() ? "mesh_function_" + std::to_string(mesh_functions_.size())
                                                           : meshFunction.name();
        mesh_functions_.push_back(VTKCellArray{nm, meshFunction.data()});
    }
    void addMeshFunction(std::function<double(double x, double y)> meshFunction, std::string meshFunctionName) {
        VTKCellArray a{meshFunctionName, {}};
        iterateCells([&](double x, double y) { a.values.push_back(meshFunction(x, y)); });
        mesh_functions_.push_back(std::move(a));
    }
    void clearMeshFunctions() { mesh_functions_.clear(); }

    // Mesh.hpp:398-424: <base>-mesh[-NNNN].pvtu with its piece <base>-mesh[-NNNN]-0.vtu (one quad per
    // leaf cell, the added mesh functions as cell data) and <base>-quadtree[-NNNN].vtu (one quad per leaf
    // patch, its level and leaf index as cell data).
    void toVTK(std::string baseFilename, int number = -1) {
        std::string tag;
        if (number != -1) {
            char buffer[32];
            std::snprintf(buffer, sizeof(buffer), "-%04i", number);
            tag = buffer;
        }
        std::vector<double> cells, boxes;
        std::vector<double> level, index;
        for (std::size_t k = 0; k < leaves_.size(); ++k) {
            auto& g = leaves_[k]->data.grid();
            const double dx = g.dx(), dy = g.dy();
            for (std::size_t i = 0; i < g.nx(); ++i)
                for (std::size_t j = 0; j < g.ny(); ++j) {
                    const double x0 = g.xLower() + i * dx, y0 = g.yLower() + j * dy;
                    const double q[8] = {x0, y0, x0 + dx, y0, x0 + dx, y0 + dy, x0, y0 + dy};
                    cells.insert(cells.end(), q, q + 8);
                }
            const double b[8] = {g.xLower(), g.yLower(), g.xUpper(), g.yLower(), g.xUpper(), g.yUpper(), g.xLower(),
                                 g.yUpper()};
            boxes.insert(boxes.end(), b, b + 8);
            level.push_back(double(leaves_[k]->level));
            index.push_back(double(k));
        }
        const std::string mesh = baseFilename + "-mesh" + tag;
        const std::size_t slash = mesh.find_last_of('/');
        writeQuadVTU(mesh + "-0.vtu", cells, mesh_functions_);
        writePVTU(mesh + ".pvtu", (slash == std::string::npos ? mesh : mesh.substr(slash + 1)) + "-0.vtu",
                  mesh_functions_);
        writeQuadVTU(baseFilename + "-quadtree" + tag + ".vtu", boxes,
                     {VTKCellArray{"level", level}, VTKCellArray{"leaf", index}});
    }

private:
    static int tramp(double x, double y, void* ctx) {
        return (*static_cast<std::function<bool(double, double)>*>(ctx))(x, y) ? 1 : 0;
    }

    void adopt(ef_mesh* h, PatchType& root_patch, AbstractNodeFactory<PatchType>& factory) {
        if (handle_) ef_mesh_destroy(handle_);
        handle_ = h;
        quadtree.clear();
        leaves_.clear();
        int nl = 0;
        efCheck(ef_mesh_num_leaves(h, &nl), "Mesh::refineByFunction");
        std::vector<std::string> leaf_paths(nl);
        for (int k = 0; k < nl; ++k) {
            int level = 0;
            long long ix = 0, iy = 0;
            efCheck(ef_mesh_leaf(h, k, &level, &ix, &iy, nullptr), "Mesh::refineByFunction");
            std::string p;
            for (int l = level; l > 0; --l) {
                const int s = level - l;
                p.insert(p.begin(), char('0' + int(((ix >> s) & 1) | (((iy >> s) & 1) << 1))));
            }
            leaf_paths[k] = "0" + p;
        }
        // every prefix of a leaf path is a node (p4est_search_all visits them all)
        std::vector<std::string> paths;
        std::map<std::string, bool> seen;
        for (auto& lp : leaf_paths)
            for (std::size_t k = 1; k <= lp.size(); ++k) {
                const std::string pre = lp.substr(0, k);
                if (!seen.count(pre)) { seen[pre] = true; paths.push_back(pre); }
            }
        std::sort(paths.begin(), paths.end(), [](const std::string& a, const std::string& b) {
            return a.size() != b.size() ? a.size() < b.size() : a < b;
        });
        for (auto& p : paths) {
            Node<PatchType>* nd = (p == "0") ? factory.createNode(root_patch, "0", 0, 0, 0)
                                             : factory.createChildNode(quadtree.map.at(p.substr(0, p.size() - 1)),
                                                                       p.back() - '0', 0, 0);
            quadtree.map[p] = nd;
        }
        for (auto& lp : leaf_paths) {
            quadtree.map.at(lp)->leaf = true;
            leaves_.push_back(quadtree.map.at(lp));
        }
    }

    ef_mesh* handle_ = nullptr;
    std::vector<Node<PatchType>*> leaves_;
    std::vector<VTKCellArray> mesh_functions_;
};

}  // namespace EllipticForest
