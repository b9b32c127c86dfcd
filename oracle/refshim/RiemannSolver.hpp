// TEST INFRASTRUCTURE (oracle build of the reference).  Stands in for the
// third-party RiemannSolver.hpp (bwvdnbro/python_finite_volume_solver, master,
// unpinned; fetched by demonstrator/Makefile:93-94 and absent here) with the
// oracle's own restatement of Toro's exact solver, so that the reference build
// and the oracle port use the same Riemann arithmetic.  Call site:
// demonstrator/src/Riemann.cpp:84-94.
#pragma once
#include "../riemann_exact.hpp"

class RiemannSolver {
public:
    explicit RiemannSolver(double gamma) : rs_(gamma, 1e-10, 100) {}
    int solve(double rhoL, double uL, double PL, double rhoR, double uR, double PR,
              double &rhoSol, double &uSol, double &PSol) const {
        return rs_.solve(rhoL, uL, PL, rhoR, uR, PR, rhoSol, uSol, PSol);
    }
private:
    orc::ExactRiemann rs_;
};
