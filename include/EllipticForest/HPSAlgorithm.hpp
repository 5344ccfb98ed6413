// HPSAlgorithm<PatchGridType, PatchSolverType, PatchType, NumericalType> of the C++ drop-in
// (src/HPSAlgorithm.hpp:26-596): the same constructor, stages and callbacks, running on one GB300
// through the C ABI.  Operators stay in device memory owned by the handle; leaf vectorF/vectorU
// are materialised on the host patches as the reference's drivers read them.
#pragma once

#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>

#include "Mesh.hpp"

namespace EllipticForest {

enum BoundaryConditionType { Dirichlet = 0, Neumann = 1, Robin = 2 };

template <typename PatchGridType, typename PatchSolverType, typename PatchType, typename NumericalType>
class HPSAlgorithm : public MPI::MPIObject {
public:
    Mesh<PatchType>& mesh;
    PatchSolverType& patch_solver;
    bool isBuilt = false;

    HPSAlgorithm(MPI::Communicator comm, Mesh<PatchType>& mesh, PatchSolverType& patch_solver)
        : MPIObject(comm), mesh(mesh), patch_solver(patch_solver) {}
    virtual ~HPSAlgorithm() {
        if (h_) ef_hps_destroy(h_);
    }
    HPSAlgorithm(const HPSAlgorithm&) = delete;
    HPSAlgorithm& operator=(const HPSAlgorithm&) = delete;

    // HPSAlgorithm.hpp:91-106
    virtual void setupStage() {
        EllipticForestApp& app = EllipticForestApp::getInstance();
        app.logHead("Begin HPS Setup Stage");
        app.addTimer("setup-stage");
        app.timers["setup-stage"].start();
        app.timers["setup-stage"].stop();
        app.logHead("End HPS Setup Stage");
    }

    // HPSAlgorithm.hpp:120-161: leaf DtN maps and every 4-to-1 merge, grouped per tree level on
    // the GPU.  The option keys are read as the reference reads them (std::get<bool> throws
    // std::bad_variant_access when a key was not set to a bool).
    virtual void buildStage() {
        EllipticForestApp& app = EllipticForestApp::getInstance();
        app.logHead("Begin HPS Build Stage");
        app.addTimer("build-stage");
        app.timers["build-stage"].start();
        const bool cache_ops = std::get<bool>(app.options["cache-operators"]);
        ensureHandle();
        efCheck(ef_hps_set_option(h_, "cache-operators", cache_ops ? 1 : 0), "HPSAlgorithm::buildStage");
        const int st = ef_hps_build(h_);
        if (st == EF_ERR_SINGULAR) {
            // the reference prints the dgesv INFO and continues (Matrix.hpp:897-900)
            std::fprintf(stderr, "[EllipticForest::HPSAlgorithm::buildStage] %s\n", ef_last_error());
        } else {
            efCheck(st, "HPSAlgorithm::buildStage");
        }
        // mergePatch_ (HPSAlgorithm.hpp:1004-1009): the root patch grid spans the merged patches
        auto& rg = mesh.quadtree.root().grid();
        mesh.quadtree.root().grid() = FiniteVolumeGrid(getComm(), M_, rg.xLower(), rg.xUpper(), M_, rg.yLower(),
                                                       rg.yUpper());
        isBuilt = true;
        app.timers["build-stage"].stop();
        app.logHead("End HPS Build Stage");
    }

    // HPSAlgorithm.hpp:178-216: the callback sets vectorF on every leaf patch
    virtual void upwardsStage(std::function<void(PatchType& leafPatch)> rhs_patch_function) {
        EllipticForestApp& app = EllipticForestApp::getInstance();
        app.logHead("Begin HPS Upwards Stage");
        app.addTimer("upwards-stage");
        app.timers["upwards-stage"].start();
        std::vector<double> f;
        f.reserve(std::size_t(num_leaves_) * n_ * n_);
        for (auto* leaf : mesh.leaves()) {
            rhs_patch_function(leaf->data);
            auto& fv = leaf->data.vectorF();
            if (fv.size() != std::size_t(n_) * n_) throw std::invalid_argument("[upwardsStage] vectorF has the wrong size");
            f.insert(f.end(), fv.data().begin(), fv.data().end());
        }
        runUpwards(f);
        app.timers["upwards-stage"].stop();
        app.logHead("End HPS Upwards Stage");
    }

    // HPSAlgorithm.hpp:225-272: f sampled at the leaf cell centres, index j + i*ny
    virtual void upwardsStage(std::function<double(double, double)> rhs_function) {
        EllipticForestApp& app = EllipticForestApp::getInstance();
        app.logHead("Begin HPS Upwards Stage");
        app.addTimer("upwards-stage");
        app.timers["upwards-stage"].start();
        std::vector<double> f;
        f.reserve(std::size_t(num_leaves_ > 0 ? num_leaves_ : 1) * n_ * n_);
        for (auto* leaf : mesh.leaves()) {
            auto& grid = leaf->data.grid();
            Vector<double> fv(grid.nx() * grid.ny());
            for (std::size_t i = 0; i < grid.nx(); ++i) {
                const double x = grid(0, i);
                for (std::size_t j = 0; j < grid.ny(); ++j) fv[j + i * grid.ny()] = rhs_function(x, grid(1, j));
            }
            f.insert(f.end(), fv.data().begin(), fv.data().end());
            leaf->data.vectorF() = std::move(fv);
        }
        runUpwards(f);
        app.timers["upwards-stage"].stop();
        app.logHead("End HPS Upwards Stage");
    }

    // HPSAlgorithm.hpp:291-324: the callback sets vectorG (4M, WESN) on the root patch
    virtual void solveStage(std::function<void(PatchType& rootPatch)> boundary_data_function) {
        EllipticForestApp& app = EllipticForestApp::getInstance();
        app.logHead("Begin HPS Solve Stage");
        app.addTimer("solve-stage");
        app.timers["solve-stage"].start();
        requireBuilt();
        PatchType& root = mesh.quadtree.root();
        boundary_data_function(root);
        if (root.vectorG().size() != 4 * std::size_t(M_)) throw std::invalid_argument("[solveStage] root g has the wrong size");
        setOptions();
        efCheck(ef_hps_solve_root_dirichlet(h_, root.vectorG().dataPointer()), "HPSAlgorithm::solveStage");
        fetchLeafSolutions();
        app.timers["solve-stage"].stop();
        app.logHead("End HPS Solve Stage");
    }

    // HPSAlgorithm.hpp:343-445: a u + b du/dn = r sampled at the root face centres
    virtual void solveStage(std::function<NumericalType(int side, NumericalType x, NumericalType y,
                                                        NumericalType* a, NumericalType* b)>
                                boundary_analytical_function) {
        EllipticForestApp& app = EllipticForestApp::getInstance();
        app.logHead("Begin HPS Solve Stage");
        app.addTimer("solve-stage");
        app.timers["solve-stage"].start();
        requireBuilt();
        auto& rg = mesh.quadtree.root().grid();
        const int M = M_;
        std::vector<double> a(4 * M), b(4 * M), r(4 * M);
        for (int side = 0; side < 4; ++side)
            for (int i = 0; i < M; ++i) {
                double x, y;
                if (side == 0) { x = rg.xLower(); y = rg(1, i); }
                else if (side == 1) { x = rg.xUpper(); y = rg(1, i); }
                else if (side == 2) { x = rg(0, i); y = rg.yLower(); }
                else { x = rg(0, i); y = rg.yUpper(); }
                NumericalType av = 0, bv = 0;
                r[side * M + i] = boundary_analytical_function(side, x, y, &av, &bv);
                a[side * M + i] = av;
                b[side * M + i] = bv;
            }
        setOptions();
        efCheck(ef_hps_solve(h_, a.data(), b.data(), r.data()), "HPSAlgorithm::solveStage");
        fetchLeafSolutions();
        app.timers["solve-stage"].stop();
        app.logHead("End HPS Solve Stage");
    }

    // The per-node hooks of the reference (HPSAlgorithm.hpp:497-596).  On the GPU every tree level
    // is merged, upward-passed and split by grouped kernels over all of its nodes, and the operators
    // stay in device memory, so there is no per-node call a subclass could take over.  The hooks are
    // therefore `final`: a subclass that overrides one (as the reference allows) fails to compile
    // ("overriding final function") instead of being silently ignored.  Calling one directly throws.
    virtual void merge4to1(PatchType& tau, PatchType& alpha, PatchType& beta, PatchType& gamma,
                           PatchType& omega) final {
        noPerNodeHook("merge4to1");
    }
    virtual void upwards4to1(PatchType& tau, PatchType& alpha, PatchType& beta, PatchType& gamma,
                             PatchType& omega) final {
        noPerNodeHook("upwards4to1");
    }
    virtual void split1to4(PatchType& tau, PatchType& alpha, PatchType& beta, PatchType& gamma,
                           PatchType& omega) final {
        noPerNodeHook("split1to4");
    }
    virtual void leafSolve(PatchType& patch) final { noPerNodeHook("leafSolve"); }

    ef_hps* handle() { return h_; }

private:
    [[noreturn]] static void noPerNodeHook(const char* name) {
        throw std::logic_error(std::string("[HPSAlgorithm::") + name +
                               "] per-node hooks do not run on the GPU path: every tree level runs as grouped kernels");
    }
    void ensureHandle() {
        if (h_) return;
        efCheck(ef_hps_create(mesh.handle(), patch_solver.efType(), patch_solver.efLambda(), &h_),
                "HPSAlgorithm: create");
        long long bytes = 0;
        efCheck(ef_hps_info(h_, &num_leaves_, &n_, &M_, &bytes), "HPSAlgorithm: info");
        if (patch_solver.solver_type == FiniteVolumeSolverType::FivePointStencil) {
            // variable coefficients sampled on every leaf (FiniteVolumeSolver.cpp:66-79)
            const std::size_t nn = std::size_t(n_) * n_;
            std::vector<double> a(num_leaves_ * nn), b(4 * num_leaves_ * nn), l(num_leaves_ * nn);
            std::size_t k = 0;
            for (auto* leaf : mesh.leaves()) {
                patch_solver.sampleCoefficients(leaf->data.grid(), a.data() + k * nn, b.data() + 4 * k * nn,
                                                l.data() + k * nn);
                ++k;
            }
            efCheck(ef_hps_set_coefficients(h_, a.data(), b.data(), l.data()), "HPSAlgorithm: coefficients");
        }
    }
    void requireBuilt() {
        if (!h_ || !isBuilt) throw std::logic_error("[HPSAlgorithm] build stage must run first");
    }
    void setOptions() {
        EllipticForestApp& app = EllipticForestApp::getInstance();
        efCheck(ef_hps_set_option(h_, "homogeneous-rhs", std::get<bool>(app.options["homogeneous-rhs"]) ? 1 : 0),
                "HPSAlgorithm: options");
    }
    void runUpwards(const std::vector<double>& f) {
        requireBuilt();
        setOptions();
        efCheck(ef_hps_upwards(h_, f.data()), "HPSAlgorithm::upwardsStage");
    }
    void fetchLeafSolutions() {
        std::vector<double> u(std::size_t(num_leaves_) * n_ * n_);
        efCheck(ef_hps_get_leaf_u(h_, u.data()), "HPSAlgorithm: leaf solutions");
        const std::size_t nn = std::size_t(n_) * n_;
        auto& leaves = mesh.leaves();
        for (std::size_t k = 0; k < leaves.size(); ++k)
            leaves[k]->data.vectorU() = Vector<double>(std::vector<double>(u.begin() + k * nn, u.begin() + (k + 1) * nn));
    }

    ef_hps* h_ = nullptr;
    int num_leaves_ = 0, n_ = 0, M_ = 0;
};

}  // namespace EllipticForest
