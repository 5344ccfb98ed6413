// Driver written against the C++ drop-in exactly as a reference user would (the API sequence of
// the reference's examples/elliptic-single: app + options, grid and root patch, node factory,
// Mesh::refineByFunction, FiniteVolumeSolver, HPSAlgorithm setup/build/upwards/solve, traversal of
// the leaf patches, Mesh::toVTK).  Solves  u_xx + u_yy = f  with u = sin x + sin y and writes the
// leaf solutions (pre-order leaf order, cell j + i*ny) to the file given by --out=<path>, and the VTK
// files <path>-vtk-mesh.pvtu / -mesh-0.vtu / -quadtree.vtu.
#include <cmath>
#include <cstdio>
#include <string>

#include <EllipticForest.hpp>
#include <Patches/FiniteVolume/FiniteVolume.hpp>

namespace ef = EllipticForest;

static double uExact(double x, double y) { return std::sin(x) + std::sin(y); }
static double fRHS(double x, double y) { return -uExact(x, y); }

template <class T>
static T opt(ef::EllipticForestApp& app, const char* key, T fallback) {
    if (!app.options.optionExists(key)) app.options.setOption(key, fallback);
    return std::get<T>(app.options[key]);
}

int main(int argc, char** argv) {
    ef::EllipticForestApp app(&argc, &argv);
    app.logger.quiet = true;
    app.options.setOption("cache-operators", false);
    app.options.setOption("homogeneous-rhs", false);
    const double threshold = opt<double>(app, "refinement-threshold", 1.2);
    const int min_level = opt<int>(app, "min-level", 0);
    const int max_level = opt<int>(app, "max-level", 3);
    const int nx = opt<int>(app, "nx", 16);
    const double lo = opt<double>(app, "x-lower", -10.0), hi = opt<double>(app, "x-upper", 10.0);
    const std::string out = opt<std::string>(app, "out", std::string("u.bin"));

    ef::FiniteVolumeGrid grid(MPI_COMM_WORLD, nx, lo, hi, nx, lo, hi);
    ef::FiniteVolumePatch root_patch(MPI_COMM_WORLD, grid);
    ef::FiniteVolumeNodeFactory node_factory(MPI_COMM_WORLD);
    ef::Mesh<ef::FiniteVolumePatch> mesh{};
    mesh.refineByFunction([&](double x, double y) { return std::fabs(fRHS(x, y)) > threshold; }, threshold,
                          min_level, max_level, root_patch, node_factory);

    ef::FiniteVolumeSolver solver{};
    solver.solver_type = ef::FiniteVolumeSolverType::FISHPACK90;
    solver.alpha_function = [](double, double) { return 1.0; };
    solver.beta_function = [](double, double) { return 1.0; };
    solver.lambda_function = [](double, double) { return 0.0; };

    ef::HPSAlgorithm<ef::FiniteVolumeGrid, ef::FiniteVolumeSolver, ef::FiniteVolumePatch, double> HPS(
        MPI_COMM_WORLD, mesh, solver);
    HPS.setupStage();
    HPS.buildStage();
    HPS.upwardsStage([&](double x, double y) { return fRHS(x, y); });
    HPS.solveStage([&](int side, double x, double y, double* a, double* b) {
        *a = 1.0;
        *b = 0.0;
        return uExact(x, y);
    });

    ef::Vector<double> uMesh{};
    double err = 0.0;
    int nleaves = 0;
    mesh.quadtree.traversePreOrder([&](ef::Node<ef::FiniteVolumePatch>* node) {
        if (node->leaf) {
            auto& patch = node->data;
            auto& g = patch.grid();
            for (std::size_t i = 0; i < g.nx(); ++i)
                for (std::size_t j = 0; j < g.ny(); ++j)
                    err = std::max(err, std::fabs(patch.vectorU()[j + i * g.ny()] - uExact(g(0, i), g(1, j))));
            uMesh.append(patch.vectorU());
            ++nleaves;
        }
        return 1;
    });
    // Mesh::toVTK as in the reference's examples: the leaf solution and the exact solution as cell data
    uMesh.name() = "u";
    mesh.addMeshFunction(uMesh);
    mesh.addMeshFunction([](double x, double y) { return uExact(x, y); }, "u_exact");
    mesh.toVTK(out + "-vtk");
    std::FILE* fp = std::fopen(out.c_str(), "wb");
    if (!fp) return 2;
    std::fwrite(uMesh.dataPointer(), sizeof(double), uMesh.size(), fp);
    std::fclose(fp);
    std::printf("{\"leaves\": %d, \"dofs\": %zu, \"max_err\": %.17g, \"build_s\": %.6f, \"solve_s\": %.6f}\n",
                nleaves, uMesh.size(), err, app.timers["build-stage"].time(), app.timers["solve-stage"].time());
    return 0;
}
