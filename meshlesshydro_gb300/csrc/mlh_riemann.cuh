// Exact Riemann solver for an ideal gas on the device, one thread per face.
//
// Method: E. F. Toro, "Riemann Solvers and Numerical Methods for Fluid
// Dynamics", 3rd ed., ch. 4: Newton-Raphson on f(p) = fL(p) + fR(p) + du for
// the star pressure, two-rarefaction initial guess, sampling at x/t = 0.  The
// reference calls the third-party RiemannSolver.hpp for this step
// (demonstrator/src/Riemann.cpp:84-94), whose sources are not in its tree; this
// solver fixes the guess, the convergence test |dp| / p_mean <= tol and the
// sampling rules, the same choices as the CPU oracle.
#pragma once
#include "mlh_device.cuh"

namespace mlh {

struct RiemannConsts {
    double gamma, g1, g2, g3, g4, g5, g6, g7, inv_gamma, tol;
    int max_iter;
};

__host__ __device__ inline RiemannConsts make_riemann_consts(double gamma, double tol, int max_iter) {
    RiemannConsts c;
    c.gamma = gamma;
    c.g1 = (gamma - 1.) / (2. * gamma);
    c.g2 = (gamma + 1.) / (2. * gamma);
    c.g3 = 2. * gamma / (gamma - 1.);
    c.g4 = 2. / (gamma - 1.);
    c.g5 = 2. / (gamma + 1.);
    c.g6 = (gamma - 1.) / (gamma + 1.);
    c.g7 = (gamma - 1.) / 2.;
    c.inv_gamma = 1. / gamma;
    c.tol = tol;
    c.max_iter = max_iter;
    return c;
}

// f_K and f_K' (Toro eqs. 4.6, 4.7, 4.37); (p/pK)^(-(g+1)/(2g)) = (p/pK)^g1 / (p/pK).
__device__ __forceinline__ void pressure_fn(const RiemannConsts &c, double p, double rhoK, double pK, double cK,
                                            double &f, double &fd) {
    if (p <= pK) {
        double prat = p / pK;
        double q = pow(prat, c.g1);
        f = c.g4 * cK * (q - 1.);
        fd = q / (prat * rhoK * cK);
    } else {
        double ak = c.g5 / rhoK;
        double bk = c.g6 * pK;
        double qrt = sqrt(ak / (bk + p));
        f = (p - pK) * qrt;
        fd = (1. - .5 * (p - pK) / (bk + p)) * qrt;
    }
}

struct RiemannResult {
    double rho, u, p;
    int flag;    // -1: left of the contact sampled, +1: right, 0: vacuum
    int iters;   // Newton iterations (< 0: no convergence)
};

// Newton-Raphson from p0; returns iterations or -1.
__device__ __forceinline__ int newton_pstar(const RiemannConsts &c, double p0, double rhoL, double uL, double pL,
                                            double cL, double rhoR, double uR, double pR, double cR, double &pstar) {
    double pfloor = 1e-12 * (pL > pR ? pL : pR);
    double p = p0 > pfloor ? p0 : pfloor;
    double du = uR - uL;
    for (int it = 1; it <= c.max_iter; ++it) {
        double fL, fdL, fR, fdR;
        pressure_fn(c, p, rhoL, pL, cL, fL, fdL);
        pressure_fn(c, p, rhoR, pR, cR, fR, fdR);
        double pnew = p - (fL + fR + du) / (fdL + fdR);
        if (!(pnew > 0.)) pnew = pfloor;
        double change = 2. * fabs(pnew - p) / (pnew + p);
        p = pnew;
        if (change <= c.tol) { pstar = p; return it; }
    }
    pstar = p;
    return -1;
}

// Solve with the two-rarefaction guess (or `guess` when > 0, falling back to
// the two-rarefaction guess if Newton does not converge from it), then sample
// at S = 0 (Toro section 4.5).
__device__ inline RiemannResult riemann_exact(const RiemannConsts &c, double rhoL, double uL, double pL,
                                              double rhoR, double uR, double pR, double guess = -1.) {
    RiemannResult res;
    double cL = sqrt(c.gamma * pL / rhoL);
    double cR = sqrt(c.gamma * pR / rhoR);
    if (c.g4 * (cL + cR) <= uR - uL) {
        res.rho = 0.; res.u = 0.; res.p = 0.; res.flag = 0; res.iters = 0;
        return res;
    }
    double pstar;
    int it = -1;
    if (guess > 0.) it = newton_pstar(c, guess, rhoL, uL, pL, cL, rhoR, uR, pR, cR, pstar);
    if (it < 0) {
        double num = cL + cR - c.g7 * (uR - uL);
        double den = cL / pow(pL, c.g1) + cR / pow(pR, c.g1);
        double p0 = pow(num / den, c.g3);
        int it2 = newton_pstar(c, p0, rhoL, uL, pL, cL, rhoR, uR, pR, cR, pstar);
        it = (guess > 0. && it2 >= 0) ? it2 + c.max_iter : it2;
        if (it2 < 0) it = -1;
    }
    res.iters = it;
    double fL, fdL, fR, fdR;
    pressure_fn(c, pstar, rhoL, pL, cL, fL, fdL);
    pressure_fn(c, pstar, rhoR, pR, cR, fR, fdR);
    double ustar = .5 * (uL + uR) + .5 * (fR - fL);
    double rho, u, p;
    if (0. <= ustar) {
        if (pstar <= pL) {
            double shl = uL - cL;
            if (0. <= shl) { rho = rhoL; u = uL; p = pL; }
            else {
                double cml = cL * pow(pstar / pL, c.g1);
                double stl = ustar - cml;
                if (0. > stl) { rho = rhoL * pow(pstar / pL, c.inv_gamma); u = ustar; p = pstar; }
                else {
                    double cf = c.g5 * (cL + c.g7 * uL);
                    u = cf;
                    rho = rhoL * pow(cf / cL, c.g4);
                    p = pL * pow(cf / cL, c.g3);
                }
            }
        } else {
            double pml = pstar / pL;
            double sl = uL - cL * sqrt(c.g2 * pml + c.g1);
            if (0. <= sl) { rho = rhoL; u = uL; p = pL; }
            else { rho = rhoL * (pml + c.g6) / (pml * c.g6 + 1.); u = ustar; p = pstar; }
        }
        res.flag = -1;
    } else {
        if (pstar > pR) {
            double pmr = pstar / pR;
            double sr = uR + cR * sqrt(c.g2 * pmr + c.g1);
            if (0. >= sr) { rho = rhoR; u = uR; p = pR; }
            else { rho = rhoR * (pmr + c.g6) / (pmr * c.g6 + 1.); u = ustar; p = pstar; }
        } else {
            double shr = uR + cR;
            if (0. >= shr) { rho = rhoR; u = uR; p = pR; }
            else {
                double cmr = cR * pow(pstar / pR, c.g1);
                double str = ustar + cmr;
                if (0. <= str) { rho = rhoR * pow(pstar / pR, c.inv_gamma); u = ustar; p = pstar; }
                else {
                    double cf = c.g5 * (cR - c.g7 * uR);
                    u = -cf;
                    rho = rhoR * pow(cf / cR, c.g4);
                    p = pR * pow(cf / cR, c.g3);
                }
            }
        }
        res.flag = 1;
    }
    res.rho = rho; res.u = u; res.p = p;
    return res;
}

}  // namespace mlh
