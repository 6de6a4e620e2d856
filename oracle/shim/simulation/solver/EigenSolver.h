// Shim for the reference build only (oracle/_ref): the reference's Eigen solvers
// (include/simulation/solver/EigenSolver.h) need the empty Eigen submodule.  Same class names, bodies abort;
// the oracle selects only the CG and Jacobi solvers.
#pragma once
#include <cstdlib>
#include "simulation/solver/ISolver.h"
class EigenCGSolver2D : public ISolverCPU2D {
public:
    EigenCGSolver2D(int w, int h) : ISolverCPU2D(w, h) { std::abort(); }
    float solve(IGrid2D*) override { std::abort(); }
};
class EigenBiCGSTABSolver2D : public ISolverCPU2D {
public:
    EigenBiCGSTABSolver2D(int w, int h) : ISolverCPU2D(w, h) { std::abort(); }
    float solve(IGrid2D*) override { std::abort(); }
};
