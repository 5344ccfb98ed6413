// Finite-volume plugin of the C++ drop-in: FiniteVolumeGrid, FiniteVolumePatch, FiniteVolumeSolver
// and FiniteVolumeNodeFactory with the reference's names and signatures
// (src/Patches/FiniteVolume/*.hpp).  The solver's numerical work runs in the GB300 library through
// the C ABI (ef_fv_build_d2n / ef_fv_solve / ef_fv_map_d2n).
#pragma once

#include <string>

#include "Core.hpp"

namespace EllipticForest {

enum DimensionIndex { X = 0, Y = 1 };
constexpr int XDIM = 0;
constexpr int YDIM = 1;

using Analytical2DFunction = std::function<double(double, double)>;

enum FiniteVolumeSolverType { FivePointStencil, FISHPACK90 };

// FiniteVolumeGrid.cpp:9-36
class FiniteVolumeGrid : public MPI::MPIObject {
public:
    FiniteVolumeGrid() : MPIObject(MPI_COMM_SELF) {}
    FiniteVolumeGrid(MPI::Communicator comm, int nx, double x_lower, double x_upper, int ny, double y_lower,
                     double y_upper)
        : MPIObject(comm), nx_(nx), x_lower_(x_lower), x_upper_(x_upper), dx_((x_upper - x_lower) / nx),
          ny_(ny), y_lower_(y_lower), y_upper_(y_upper), dy_((y_upper - y_lower) / ny) {}

    double point(DimensionIndex dim, int index) const {
        if (dim == DimensionIndex::X) return (x_lower_ + dx_ / 2) + index * dx_;
        if (dim == DimensionIndex::Y) return (y_lower_ + dy_ / 2) + index * dy_;
        throw std::invalid_argument("Invalid `dim` argument.");
    }
    double operator()(std::size_t dim, std::size_t index) const { return point(DimensionIndex(dim), int(index)); }
    std::string name() const { return "FiniteVolumeGrid"; }
    std::size_t nx() const { return nx_; }
    std::size_t ny() const { return ny_; }
    double xLower() const { return x_lower_; }
    double xUpper() const { return x_upper_; }
    double yLower() const { return y_lower_; }
    double yUpper() const { return y_upper_; }
    double dx() const { return dx_; }
    double dy() const { return dy_; }

private:
    int nx_ = 0;
    double x_lower_ = 0, x_upper_ = 0, dx_ = 0;
    int ny_ = 0;
    double y_lower_ = 0, y_upper_ = 0, dy_ = 0;
};

// FiniteVolumePatch.hpp:19-73: leaf data live on the host patches; operators stay on the device.
class FiniteVolumePatch : public MPI::MPIObject {
public:
    int n_coarsens = 0;

    FiniteVolumePatch() : MPIObject(MPI_COMM_WORLD) {}
    explicit FiniteVolumePatch(MPI::Communicator comm) : MPIObject(comm), grid_(comm, 0, 0, 0, 0, 0, 0) {}
    FiniteVolumePatch(MPI::Communicator comm, FiniteVolumeGrid grid) : MPIObject(comm), grid_(grid) {}

    std::string name() const { return "FiniteVolumePatch"; }
    FiniteVolumeGrid& grid() { return grid_; }
    int size() { return int(grid_.nx() / std::pow(2, n_coarsens)); }  // Patch.hpp:99-101

    Matrix<double>& matrixX() { return X_; }
    Matrix<double>& matrixH() { return H_; }
    Matrix<double>& matrixS() { return S_; }
    Matrix<double>& matrixT() { return T_; }
    Vector<double>& vectorU() { return u_; }
    Vector<double>& vectorG() { return g_; }
    Vector<double>& vectorV() { return v_; }
    Vector<double>& vectorF() { return f_; }
    Vector<double>& vectorH() { return h_; }
    Vector<double>& vectorW() { return w_; }

private:
    FiniteVolumeGrid grid_;
    Matrix<double> X_, H_, S_, T_;
    Vector<double> u_, g_, v_, f_, h_, w_;
};

// FiniteVolumeSolver.hpp:53-162
class FiniteVolumeSolver : public MPI::MPIObject {
public:
    FiniteVolumeSolverType solver_type = FiniteVolumeSolverType::FivePointStencil;
    Analytical2DFunction alpha_function;
    Analytical2DFunction beta_function;
    Analytical2DFunction lambda_function;
    Analytical2DFunction rhs_function;

    FiniteVolumeSolver() : MPIObject(MPI_COMM_SELF) {}
    FiniteVolumeSolver(MPI::Communicator comm, Analytical2DFunction alpha, Analytical2DFunction beta,
                       Analytical2DFunction lambda, Analytical2DFunction rhs)
        : MPIObject(comm), alpha_function(alpha), beta_function(beta), lambda_function(lambda), rhs_function(rhs) {}

    std::string name() const { return "FiniteVolumeSolver"; }
    int gridIndex2MatrixIndex(int i, int j, int nx, int ny) const { return j + i * ny; }

    // library code of the solver type
    int efType() const {
        return solver_type == FiniteVolumeSolverType::FISHPACK90 ? EF_SOLVER_FISHPACK90 : EF_SOLVER_FIVE_POINT;
    }
    double efLambda() const { return lambda_function ? lambda_function(0, 0) : 0.0; }

    // FivePointStencil coefficients of one patch sampled at the points of FiniteVolumeSolver.cpp:66-79:
    // alpha(x_i, y_j); beta at x_i -/+ dx/2.0 and y_j -/+ dy/2.0 (all W, then E, S, N); lambda(x_i, y_j)
    void sampleCoefficients(FiniteVolumeGrid& grid, double* alpha, double* beta, double* lambda) const {
        const std::size_t nx = grid.nx(), ny = grid.ny(), N = nx * ny;
        const double dx = grid.dx(), dy = grid.dy();
        for (std::size_t i = 0; i < nx; ++i)
            for (std::size_t j = 0; j < ny; ++j) {
                const double xi = grid(0, i), yj = grid(1, j);
                const std::size_t c = j + i * ny;
                alpha[c] = alpha_function(xi, yj);
                beta[c] = beta_function(xi - dx / 2.0, yj);
                beta[N + c] = beta_function(xi + dx / 2.0, yj);
                beta[2 * N + c] = beta_function(xi, yj - dy / 2.0);
                beta[3 * N + c] = beta_function(xi, yj + dy / 2.0);
                lambda[c] = lambda_function(xi, yj);
            }
    }

    Vector<double> solve(FiniteVolumeGrid& grid, Vector<double>& dirichlet_data, Vector<double>& rhs_data) {
        const int n = int(grid.nx());
        checkSizes(grid, dirichlet_data, rhs_data);
        Vector<double> u(std::size_t(n) * n);
        if (solver_type == FiniteVolumeSolverType::FivePointStencil) {
            Coef c(grid, *this);
            efCheck(ef_fv5_solve(n, grid.xLower(), grid.xUpper(), grid.yLower(), grid.yUpper(), c.a.data(),
                                 c.b.data(), c.l.data(), dirichlet_data.dataPointer(), rhs_data.dataPointer(),
                                 u.dataPointer()),
                    "FiniteVolumeSolver::solve");
        } else {
            efCheck(ef_fv_solve(efType(), n, grid.xLower(), grid.xUpper(), grid.yLower(), grid.yUpper(), efLambda(),
                                dirichlet_data.dataPointer(), rhs_data.dataPointer(), u.dataPointer()),
                    "FiniteVolumeSolver::solve");
        }
        return u;
    }
    Vector<double> mapD2N(FiniteVolumeGrid& grid, Vector<double>& dirichlet_data, Vector<double>& rhs_data) {
        const int n = int(grid.nx());
        checkSizes(grid, dirichlet_data, rhs_data);
        Vector<double> h(4 * std::size_t(n));
        if (solver_type == FiniteVolumeSolverType::FivePointStencil) {
            Coef c(grid, *this);
            efCheck(ef_fv5_map_d2n(n, grid.xLower(), grid.xUpper(), grid.yLower(), grid.yUpper(), c.a.data(),
                                   c.b.data(), c.l.data(), dirichlet_data.dataPointer(), rhs_data.dataPointer(),
                                   h.dataPointer()),
                    "FiniteVolumeSolver::mapD2N");
        } else {
            efCheck(ef_fv_map_d2n(efType(), n, grid.xLower(), grid.xUpper(), grid.yLower(), grid.yUpper(),
                                  efLambda(), dirichlet_data.dataPointer(), rhs_data.dataPointer(), h.dataPointer()),
                    "FiniteVolumeSolver::mapD2N");
        }
        return h;
    }
    Matrix<double> buildD2N(FiniteVolumeGrid& grid) {
        const int n = int(grid.nx());
        Matrix<double> T(4 * std::size_t(n), 4 * std::size_t(n));
        if (solver_type == FiniteVolumeSolverType::FivePointStencil) {
            Coef c(grid, *this);
            efCheck(ef_fv5_build_d2n(n, grid.xLower(), grid.xUpper(), grid.yLower(), grid.yUpper(), c.a.data(),
                                     c.b.data(), c.l.data(), T.dataPointer()),
                    "FiniteVolumeSolver::buildD2N");
        } else {
            efCheck(ef_fv_build_d2n(efType(), n, grid.xLower(), grid.xUpper(), grid.yLower(), grid.yUpper(),
                                    efLambda(), T.dataPointer()),
                    "FiniteVolumeSolver::buildD2N");
        }
        return T;
    }
    Vector<double> particularNeumannData(FiniteVolumeGrid& grid, Vector<double>& rhs_data) {
        Vector<double> g0(2 * grid.nx() + 2 * grid.ny(), 0.0);
        return mapD2N(grid, g0, rhs_data);
    }

private:
    struct Coef {
        std::vector<double> a, b, l;
        Coef(FiniteVolumeGrid& g, const FiniteVolumeSolver& s)
            : a(g.nx() * g.ny()), b(4 * g.nx() * g.ny()), l(g.nx() * g.ny()) {
            s.sampleCoefficients(g, a.data(), b.data(), l.data());
        }
    };
    static void checkSizes(FiniteVolumeGrid& grid, Vector<double>& g, Vector<double>& f) {
        if (grid.nx() != grid.ny()) throw std::invalid_argument("[FiniteVolumeSolver] square patches only");
        if (g.size() != 4 * grid.nx() || f.size() != grid.nx() * grid.ny())
            throw std::invalid_argument("[FiniteVolumeSolver] size mismatch of Dirichlet or RHS data");
    }
};

}  // namespace EllipticForest
