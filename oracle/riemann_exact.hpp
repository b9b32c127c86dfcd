// TEST INFRASTRUCTURE (oracle). Not part of the product; only tests/, the
// smoke check and bench.py's CPU baseline use anything under oracle/.
//
// Exact Riemann solver for an ideal gas, restated from E. F. Toro, "Riemann
// Solvers and Numerical Methods for Fluid Dynamics", 3rd ed., chapter 4
// (pressure functions f_K, Newton-Raphson iteration for p*, sampling of the
// self-similar solution at x/t = S).
//
// The reference calls this solver as the third-party header RiemannSolver.hpp
// (bwvdnbro/python_finite_volume_solver, branch master, no pinned commit:
// demonstrator/Makefile:93-94), which is not part of the reference tree. Its call
// sites are demonstrator/include/Riemann.h:9 and demonstrator/src/Riemann.cpp:84-94
// (solve(rhoL,uL,PL,rhoR,uR,PR,rho,u,P) -> -1 left / 0 vacuum / +1 right sampled).
// Riemann-level parity with that header is therefore unpinned; this restatement
// fixes the initial guess (two-rarefaction), the convergence test (relative
// change of p below `tol`) and the sampling point S = 0.
//
// The solver is a template on its arithmetic type T: double, or the oracle's
// operation-counting double (flop_count.hpp).  The constants g1..g8 are plain
// doubles, computed once per solver.
#pragma once
#include <cmath>

namespace orc {

using std::fabs;
using std::pow;
using std::sqrt;

template <typename T>
struct ExactRiemannT {
    double gamma, tol;
    int max_iter;
    double g1, g2, g3, g4, g5, g6, g7, g8;

    ExactRiemannT(double gamma_, double tol_ = 1e-10, int max_iter_ = 100)
        : gamma(gamma_), tol(tol_), max_iter(max_iter_) {
        g1 = (gamma - 1.) / (2. * gamma);
        g2 = (gamma + 1.) / (2. * gamma);
        g3 = 2. * gamma / (gamma - 1.);
        g4 = 2. / (gamma - 1.);
        g5 = 2. / (gamma + 1.);
        g6 = (gamma - 1.) / (gamma + 1.);
        g7 = (gamma - 1.) / 2.;
        g8 = gamma - 1.;
    }

    // Toro eq. (4.6)/(4.7) and their derivatives: shock branch for p > pK,
    // rarefaction branch otherwise.  (p/pK)^(-(g+1)/(2g)) is written as
    // (p/pK)^g1 / (p/pK), which needs a single pow per evaluation.
    void pfun(T p, T rhoK, T pK, T cK, T &f, T &fd) const {
        if (p <= pK) {
            T prat = p / pK;
            T q = pow(prat, g1);
            f = g4 * cK * (q - 1.);
            fd = q / (prat * rhoK * cK);
        } else {
            T ak = g5 / rhoK;
            T bk = g6 * pK;
            T qrt = sqrt(ak / (bk + p));
            f = (p - pK) * qrt;
            fd = (1. - .5 * (p - pK) / (bk + p)) * qrt;
        }
    }

    // Two-rarefaction approximation of p* (Toro eq. 4.46).
    T guess_two_rarefaction(T uL, T pL, T cL,
                                 T uR, T pR, T cR) const {
        T num = cL + cR - g7 * (uR - uL);
        T den = cL / pow(pL, g1) + cR / pow(pR, g1);
        return pow(num / den, g3);
    }

    // Newton-Raphson on f(p) = fL(p) + fR(p) + (uR - uL) from `p0`.
    // Returns the number of iterations, or -1 without convergence.
    int newton(T p0, T rhoL, T uL, T pL, T cL,
               T rhoR, T uR, T pR, T cR, T &pstar) const {
        T pfloor = 1e-12 * (pL > pR ? pL : pR);
        T p = p0 > pfloor ? p0 : pfloor;
        T du = uR - uL;
        for (int it = 1; it <= max_iter; ++it) {
            T fL, fdL, fR, fdR;
            pfun(p, rhoL, pL, cL, fL, fdL);
            pfun(p, rhoR, pR, cR, fR, fdR);
            T pnew = p - (fL + fR + du) / (fdL + fdR);
            if (!(pnew > 0.)) pnew = pfloor;
            T change = 2. * fabs(pnew - p) / (pnew + p);
            p = pnew;
            if (change <= tol) { pstar = p; return it; }
        }
        pstar = p;
        return -1;
    }

    // Solve and sample at S = 0.  Returns -1 when the left side of the contact
    // is sampled, +1 for the right side, 0 for vacuum.  `iters` receives the
    // Newton iteration count (negative on non-convergence).
    int solve(T rhoL, T uL, T pL, T rhoR, T uR, T pR,
              T &rho, T &u, T &p, int *iters = nullptr) const {
        T cL = sqrt(gamma * pL / rhoL);
        T cR = sqrt(gamma * pR / rhoR);
        if (g4 * (cL + cR) <= uR - uL) {
            rho = 0.; u = 0.; p = 0.;
            if (iters) *iters = 0;
            return 0;
        }
        T p0 = guess_two_rarefaction(uL, pL, cL, uR, pR, cR);
        T pstar;
        int it = newton(p0, rhoL, uL, pL, cL, rhoR, uR, pR, cR, pstar);
        if (iters) *iters = it;
        T fL, fdL, fR, fdR;
        pfun(pstar, rhoL, pL, cL, fL, fdL);
        pfun(pstar, rhoR, pR, cR, fR, fdR);
        T ustar = .5 * (uL + uR) + .5 * (fR - fL);
        sample(rhoL, uL, pL, cL, rhoR, uR, pR, cR, pstar, ustar, rho, u, p);
        return 0. <= ustar ? -1 : 1;
    }

    // Toro section 4.5, evaluated at S = x/t = 0.
    void sample(T rhoL, T uL, T pL, T cL,
                T rhoR, T uR, T pR, T cR,
                T pstar, T ustar, T &rho, T &u, T &p) const {
        if (0. <= ustar) {
            if (pstar <= pL) {
                T shl = uL - cL;
                if (0. <= shl) { rho = rhoL; u = uL; p = pL; }
                else {
                    T cml = cL * pow(pstar / pL, g1);
                    T stl = ustar - cml;
                    if (0. > stl) {
                        rho = rhoL * pow(pstar / pL, T(1. / gamma)); u = ustar; p = pstar;
                    } else {
                        T c = g5 * (cL + g7 * uL);
                        u = c;
                        rho = rhoL * pow(c / cL, g4);
                        p = pL * pow(c / cL, g3);
                    }
                }
            } else {
                T pml = pstar / pL;
                T sl = uL - cL * sqrt(g2 * pml + g1);
                if (0. <= sl) { rho = rhoL; u = uL; p = pL; }
                else { rho = rhoL * (pml + g6) / (pml * g6 + 1.); u = ustar; p = pstar; }
            }
        } else {
            if (pstar > pR) {
                T pmr = pstar / pR;
                T sr = uR + cR * sqrt(g2 * pmr + g1);
                if (0. >= sr) { rho = rhoR; u = uR; p = pR; }
                else { rho = rhoR * (pmr + g6) / (pmr * g6 + 1.); u = ustar; p = pstar; }
            } else {
                T shr = uR + cR;
                if (0. >= shr) { rho = rhoR; u = uR; p = pR; }
                else {
                    T cmr = cR * pow(pstar / pR, g1);
                    T str = ustar + cmr;
                    if (0. <= str) {
                        rho = rhoR * pow(pstar / pR, T(1. / gamma)); u = ustar; p = pstar;
                    } else {
                        T c = g5 * (cR - g7 * uR);
                        u = -c;
                        rho = rhoR * pow(c / cR, g4);
                        p = pR * pow(c / cR, g3);
                    }
                }
            }
        }
    }
};

using ExactRiemann = ExactRiemannT<double>;

}  // namespace orc
