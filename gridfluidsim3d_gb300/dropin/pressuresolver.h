// pressuresolver.h -- drop-in replacement of GridFluidSim3D's PressureSolver
// (src/pressuresolver.h) that solves on a GB300 through libgfs.
//
// The public surface is the reference's: PressureSolverParameters
// (pressuresolver.h:38-47), VectorXd (:54-76), MatrixCell / MatrixCoefficients
// (:82-108) and PressureSolver::solve (:117).  solve() runs the same MICCG(0)
// system (gfs_pressure_solve) and fills `pressure` in the order of
// params.fluidCells.  setPrecision() is an addition: GFS_PRECISION_PLAIN (the
// default) reproduces the reference's FP64 arithmetic; GFS_PRECISION_MIXED runs
// the FP32 inner solve with FP64 refinement to the same stopping rule.
#ifndef PRESSURESOLVER_H
#define PRESSURESOLVER_H

#include <vector>
#include <stdio.h>
#include <iostream>
#include <limits>
#include <algorithm>

#include "macvelocityfield.h"
#include "logfile.h"
#include "grid3d.h"
#include "array3d.h"
#include "fluidmaterialgrid.h"
#include "gridindexvector.h"
#include "fluidsimassert.h"

struct PressureSolverParameters {
    double cellwidth;
    double density;
    double deltaTime;

    GridIndexVector *fluidCells;
    FluidMaterialGrid *materialGrid;
    MACVelocityField *velocityField;
    LogFile *logfile;
};

class VectorXd
{
public:
    VectorXd();
    VectorXd(int size);
    VectorXd(int size, double fill);
    VectorXd(VectorXd &vector);
    ~VectorXd();

    const double operator [](int i) const;
    double& operator[](int i);

    inline size_t size() {
        return _vector.size();
    }

    void fill(double fill);
    double dot(VectorXd &vector);
    double absMaxCoeff();

    std::vector<double> _vector;
};

struct MatrixCell {
    char diag;
    char plusi;
    char plusj;
    char plusk;

    MatrixCell() : diag(0x00), plusi(0x00), plusj(0x00), plusk(0x00) {}
};

class MatrixCoefficients
{
public:
    MatrixCoefficients();
    MatrixCoefficients(int size);
    ~MatrixCoefficients();

    const MatrixCell operator [](int i) const;
    MatrixCell& operator [](int i);

    inline size_t size() {
        return cells.size();
    }

    std::vector<MatrixCell> cells;
};

class PressureSolver
{
public:
    PressureSolver();
    ~PressureSolver();

    void solve(PressureSolverParameters params, VectorXd &pressure);

    // Not in the reference: choose the arithmetic (GFS_PRECISION_PLAIN = 0,
    // GFS_PRECISION_MIXED = 1) and read back the last solve's statistics.
    void setPrecision(int precision);
    int getLastIterationCount() { return _lastIterations; }
    double getLastMaxResidual() { return _lastResidual; }

private:
    int _precision = 0;
    int _lastIterations = 0;
    double _lastResidual = 0.0;
    // the reference's constants (pressuresolver.h:159-160)
    double _pressureSolveTolerance = 1e-6;
    int _maxCGIterations = 200;
};

#endif
