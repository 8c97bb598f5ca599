// pressuresolver.cpp -- drop-in PressureSolver (see pressuresolver.h): the
// reference's interface, solved by libgfs's MICCG(0) on the GPU.
#include "pressuresolver.h"

#include <cmath>
#include <cstdlib>
#include <sstream>

#include "gfs_dropin.h"

// ------------------------------------------------------------------ VectorXd
// The reference's small vector type (pressuresolver.cpp:20-81), kept because
// callers size and read the pressure through it.

VectorXd::VectorXd() {}

VectorXd::VectorXd(int size) : _vector(size, 0.0) {}

VectorXd::VectorXd(int size, double fill) : _vector(size, fill) {}

VectorXd::VectorXd(VectorXd &vector) : _vector(vector._vector) {}

VectorXd::~VectorXd() {}

const double VectorXd::operator[](int i) const {
    FLUIDSIM_ASSERT(i >= 0 && i < (int)_vector.size());
    return _vector[i];
}

double &VectorXd::operator[](int i) {
    FLUIDSIM_ASSERT(i >= 0 && i < (int)_vector.size());
    return _vector[i];
}

void VectorXd::fill(double fill) { std::fill(_vector.begin(), _vector.end(), fill); }

double VectorXd::dot(VectorXd &vector) {
    FLUIDSIM_ASSERT(_vector.size() == vector._vector.size());
    double sum = 0.0;
    for (size_t i = 0; i < _vector.size(); i++) sum += _vector[i] * vector._vector[i];
    return sum;
}

double VectorXd::absMaxCoeff() {
    double m = -std::numeric_limits<double>::infinity();
    for (double v : _vector) m = std::max(m, std::fabs(v));
    return m;
}

// -------------------------------------------------------- MatrixCoefficients

MatrixCoefficients::MatrixCoefficients() {}

MatrixCoefficients::MatrixCoefficients(int size) : cells(size, MatrixCell()) {}

MatrixCoefficients::~MatrixCoefficients() {}

const MatrixCell MatrixCoefficients::operator[](int i) const {
    FLUIDSIM_ASSERT(i >= 0 && i < (int)cells.size());
    return cells[i];
}

MatrixCell &MatrixCoefficients::operator[](int i) {
    FLUIDSIM_ASSERT(i >= 0 && i < (int)cells.size());
    return cells[i];
}

// ------------------------------------------------------------ PressureSolver

PressureSolver::PressureSolver() {}

PressureSolver::~PressureSolver() {}

void PressureSolver::setPrecision(int precision) {
    FLUIDSIM_ASSERT(precision == GFS_PRECISION_PLAIN || precision == GFS_PRECISION_MIXED);
    _precision = precision;
}

void PressureSolver::solve(PressureSolverParameters params, VectorXd &pressure) {
    // PressureSolver::solve (pressuresolver.cpp:116-137): pressure is pre-sized
    // to the fluid cells and starts from zero
    GridIndexVector *cells = params.fluidCells;
    FLUIDSIM_ASSERT(pressure.size() == (unsigned int)cells->size());
    pressure.fill(0.0);
    if (cells->size() == 0) {
        return;
    }

    gfs_ctx *ctx = gfs_dropin::context();
    gfs_dropin::check(ctx ? 0 : GFS_ERR_CUDA, "PressureSolver::solve (no CUDA device)");

    FluidMaterialGrid *mgrid = params.materialGrid;
    int ni = mgrid->width, nj = mgrid->height, nk = mgrid->depth;
    std::vector<uint8_t> mat;
    gfs_dropin::material_to_flat(mgrid, mat);
    gfs_dropin::FlatMAC mac;
    gfs_dropin::mac_to_flat(params.velocityField, mac);
    FLUIDSIM_ASSERT(mac.ni == ni && mac.nj == nj && mac.nk == nk);

    // libgfs numbers the unknowns as the fluid cells of the material grid in
    // k -> j -> i order; map them to the caller's fluidCells order
    std::vector<int32_t> index((size_t)ni * nj * nk, -1);
    int32_t next = 0;
    for (size_t q = 0; q < mat.size(); q++) {
        if (mat[q] == 1) index[q] = next++;
    }
    // (checked in every build: the mapping below indexes with it)
    if ((size_t)next != cells->size()) {
        std::cerr << "PressureSolver::solve: " << cells->size() << " fluid cells listed, " << next
                  << " fluid cells in the material grid" << std::endl;
        std::abort();
    }
    int64_t count = next;
    int iterations = 0;
    double residual = 0.0;
    std::vector<double> solved((size_t)count);
    gfs_dropin::check(gfs_pressure_solve(ctx, ni, nj, nk, params.cellwidth, params.density, params.deltaTime,
                                         mat.data(), mac.u.data(), mac.v.data(), mac.w.data(), _precision,
                                         _pressureSolveTolerance, _maxCGIterations, solved.data(), &count,
                                         &iterations, &residual),
                      "PressureSolver::solve");
    for (size_t q = 0; q < cells->size(); q++) {
        GridIndex g = cells->at(q);
        int32_t at = -1;
        if (g.i >= 0 && g.j >= 0 && g.k >= 0 && g.i < ni && g.j < nj && g.k < nk)
            at = index[(size_t)g.i + (size_t)ni * ((size_t)g.j + (size_t)nj * (size_t)g.k)];
        if (at < 0) {
            std::cerr << "PressureSolver::solve: listed cell (" << g.i << ", " << g.j << ", " << g.k
                      << ") is not a fluid cell of the material grid" << std::endl;
            std::abort();
        }
        pressure[(int)q] = solved[(size_t)at];
    }
    _lastIterations = iterations;
    _lastResidual = residual;

    // the reference's log lines (pressuresolver.cpp:474-498)
    if (params.logfile != nullptr && iterations >= 0) {
        if (iterations >= _maxCGIterations) {
            params.logfile->log("Iterations limit reached.\t Estimated error : ", residual, 1);
        } else {
            params.logfile->log("CG Iterations: ", iterations, 1);
        }
    }
}
