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
    double gamma, g1, g2, g3, g4, g5, g6, g7, inv_gamma, inv_gm1, tol;
    double tol_half;   // tol / 2 (exact): 2 |dp| <= tol s  <=>  |dp| <= (tol / 2) s
    double ig5;   // 1 / g5 = (gamma + 1) / 2
    int max_iter;
    // gamma = 5/3: g1 = 1/5, g3 = 5, g4 = 3 and 1/gamma = 3 g1, so every
    // power in the solver is a fifth root or an integer power
    int root5;
};

__host__ __device__ inline RiemannConsts make_riemann_consts(double gamma, double tol, int max_iter) {
    RiemannConsts c;
    c.gamma = gamma;
    c.g1 = (gamma - 1.) / (2. * gamma);
    c.g2 = (gamma + 1.) / (2. * gamma);
    c.g3 = 2. * gamma / (gamma - 1.);
    c.g4 = 2. / (gamma - 1.);
    c.g5 = 2. / (gamma + 1.);
    c.ig5 = (gamma + 1.) / 2.;
    c.g6 = (gamma - 1.) / (gamma + 1.);
    c.g7 = (gamma - 1.) / 2.;
    c.inv_gamma = 1. / gamma;
    c.inv_gm1 = 1. / (gamma - 1.);
    c.tol = tol;
    c.tol_half = tol / 2.;
    c.max_iter = max_iter;
    c.root5 = (fabs(1. / c.g1 - 5.) < 1e-12 && fabs(c.g4 - 3.) < 1e-12) ? 1 : 0;
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
    double pstar;   // star-region pressure
    int flag;       // -1: left of the contact sampled, +1: right, 0: vacuum,
                    // 2: not solved (two-rarefaction guess above `defer_above`)
    int iters;      // Newton iterations (< 0: no convergence)
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
// at S = 0 (Toro section 4.5).  With defer_above > 0 and no guess, a problem
// whose two-rarefaction guess exceeds defer_above returns unsolved (flag 2,
// pstar = that guess) for a second pass with a better guess.
__device__ inline RiemannResult riemann_exact(const RiemannConsts &c, double rhoL, double uL, double pL,
                                              double rhoR, double uR, double pR, double guess = -1.,
                                              double defer_above = 0.) {
    RiemannResult res;
    double cL = sqrt(c.gamma * pL / rhoL);
    double cR = sqrt(c.gamma * pR / rhoR);
    if (c.g4 * (cL + cR) <= uR - uL) {
        res.rho = 0.; res.u = 0.; res.p = 0.; res.pstar = 0.; res.flag = 0; res.iters = 0;
        return res;
    }
    double pstar;
    int it = -1;
    if (guess > 0.) it = newton_pstar(c, guess, rhoL, uL, pL, cL, rhoR, uR, pR, cR, pstar);
    if (it < 0) {
        double num = cL + cR - c.g7 * (uR - uL);
        double den = cL / pow(pL, c.g1) + cR / pow(pR, c.g1);
        double p0 = pow(num / den, c.g3);
        if (defer_above > 0. && !(guess > 0.) && p0 > defer_above) {
            res.rho = 0.; res.u = 0.; res.p = 0.; res.pstar = p0; res.flag = 2; res.iters = 0;
            return res;
        }
        int it2 = newton_pstar(c, p0, rhoL, uL, pL, cL, rhoR, uR, pR, cR, pstar);
        it = (guess > 0. && it2 >= 0) ? it2 + c.max_iter : it2;
        if (it2 < 0) it = -1;
    }
    res.iters = it;
    res.pstar = pstar;
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

// ---------------------------------------------------------------- fast path

// Comparison of non-negative doubles on the integer pipe: their bit patterns
// are ordered as the values.
__device__ __forceinline__ bool nn_le(double a, double b) { return __double_as_longlong(a) <= __double_as_longlong(b); }

// x^(-1/5) to a few ulp: a single-precision seed y (relative error e below
// 3e-7) refined by one third-order step.  With r = 1 - x y^5,
// x^(-1/5) = y (1 - r)^(-1/5) = y (1 + r/5 + 3 r^2/25 + O(r^3)), and
// |r| ~ 5 e, so dropping the O(r^3) term (0.088 r^3 < 1e-18) leaves the
// roundings of y^5, r and the last two operations: within a few ulp of the
// correctly rounded value, in seven FP64 operations (two Newton steps, whose
// error contracts as 3 e^2, took twelve).  Values outside the float range go
// through pow.
__device__ __forceinline__ double rroot5(double x) {
    // 1e-30 < x < 1e30 on the bit patterns (the test is false for NaN and x <= 0)
    const long long b = __double_as_longlong(x);
    if (!(b > 0x39B4484BFEEBC2A0ll && b < 0x46293E5939A08CEAll)) return pow(x, -0.2);
    // double -> float and back on the bit patterns (integer pipe): rebias the
    // exponent (1023 - 127 = 896) and keep the top 23 mantissa bits; x and
    // the seed are positive and normal in both formats in this range
    const float xf = __int_as_float((int)((b >> 29) - (896ll << 23)));
    const float yf = exp2f(-0.2f * __log2f(xf));
    const double y = __longlong_as_double(((long long)__float_as_int(yf) + (896ll << 23)) << 29);
    const double y2 = y * y;
    const double r = fma(-x, y2 * y2 * y, 1.);
    return fma(y, r * fma(0.12, r, 0.2), y);
}
// x^(1/5) = x * (x^(-1/5))^4
__device__ __forceinline__ double root5(double x) {
    double y = rroot5(x);
    double y2 = y * y;
    return x * (y2 * y2);
}

// Two-rarefaction estimate of p* (Toro eq. 4.46), the default starting point
// of both solvers; ROOT5 takes the gamma = 5/3 powers.  Not positive when the
// states generate vacuum.
template <bool ROOT5>
__device__ __forceinline__ double two_rarefaction_guess(const RiemannConsts &k, double rhoL, double uL, double pL,
                                                        double rhoR, double uR, double pR) {
    const double cL = sqrt(k.gamma * pL / rhoL), cR = sqrt(k.gamma * pR / rhoR);
    const double num = cL + cR - k.g7 * (uR - uL);
    if (!(num > 0.)) return -1.;
    if (ROOT5) {
        const double t = fdiv(num, cL * rroot5(pL) + cR * rroot5(pR));
        const double t2 = t * t;
        return t2 * t2 * t;
    }
    return pow(num / (cL / pow(pL, k.g1) + cR / pow(pR, k.g1)), k.g3);
}

struct RiemannSide {
    double rho, u, p, c, invp, C, iak, bk, g4c;   // iak = 1 / A_K = rho / g5
};

__device__ __forceinline__ RiemannSide make_side(const RiemannConsts &k, double rho, double u, double p) {
    RiemannSide s;
    s.rho = rho; s.u = u; s.p = p;
    // one reciprocal square root for c and 1/p: with g = gamma p and
    // y = 1/sqrt(g rho), c = sqrt(g / rho) = g y and 1/p = gamma rho y^2
    // (each within a few ulp)
    const double gp = k.gamma * p;
    const double y = frsqrt(gp * rho);
    s.c = gp * y;
    s.invp = (k.gamma * rho) * (y * y);
    s.C = s.c * k.inv_gamma;     // pK / (rhoK cK) = cK / gamma: f' = (p/pK)^g1 C / p
    s.iak = rho * k.ig5;
    s.bk = k.g6 * p;
    s.g4c = k.g4 * s.c;
    return s;
}

// f_K, f_K' at p (1/p given); q = (p/pK)^g1 on the rarefaction branch
__device__ __forceinline__ void pressure_fn5(const RiemannSide &s, double p, double invp, double &f, double &fd,
                                             double &q, bool &rare) {
    if (nn_le(p, s.p)) {
        q = root5(p * s.invp);
        f = s.g4c * (q - 1.);
        fd = q * s.C * invp;
        rare = true;
    } else {
        // qrt = sqrt(A_K / (B_K + p)) and t = 1 / (B_K + p) from one
        // reciprocal square root: qrt = 1/sqrt((B_K + p) / A_K), t = qrt^2 / A_K
        const double bp = s.bk + p;
        const double qrt = frsqrt(bp * s.iak);
        // t / 2 = qrt^2 A_K^-1 / 2, halved through the operand (exact), so
        // that nothing on the iteration's dependency chain waits on it
        const double t2 = (qrt * qrt) * half_of(s.iak);
        f = (p - s.p) * qrt;
        fd = __dmul_rn(fma(-(p - s.p), t2, 1.), qrt);
        q = 0.;
        rare = false;
    }
}

// x with its sign bit flipped when f (integer pipe; exact negation)
__device__ __forceinline__ double flip_if(double x, bool f) {
    return __longlong_as_double(__double_as_longlong(x) ^ ((long long)f << 63));
}

// Same solution as riemann_exact for gamma = 5/3 with cheaper arithmetic:
// fifth roots instead of pow, integer powers for g3, g4 and 1/gamma,
// reciprocals by Newton-Raphson (frcp), f_K(p*) from the last Newton
// evaluation plus its derivative times the final (<= tol relative) step,
// which differs from re-evaluating f at p* by O(tol^2) relative, and sign
// and order tests on the integer pipe; halvings and doublings on the
// integer pipe too (half_of, twice).
// first_iters > 0: when Newton from the two-rarefaction guess has not
// converged after that many steps, return unsolved (flag 2, pstar = the
// current iterate, iters = steps run); solving again with that iterate as
// `guess` continues the same iteration with the same arithmetic.
//
// Two mirror images keep the lanes of a warp on one branch (a warp issues
// every branch that any of its lanes takes, and on this GPU an FP64
// instruction costs the same with one active lane as with 32).  The Euler
// equations are symmetric under swapping the sides and negating the
// velocities: p* is unchanged and u* and the sampled velocity change sign.
// (1) Newton solves the problem with the lower pressure on the left (A) and
// the higher on the right (B).  It performs the same operations on the same
// operands as for the unsorted problem, with the two sides' terms added in
// the other order (IEEE addition commutes, and uR - uL is unchanged), so p*
// is the same double.  In the weak-wave faces that make up most of a step,
// p* lies between pL and pR: A is a shock and B a rarefaction in nearly
// every lane, where the unsorted problem splits each side's branch of
// pressure_fn5 at random.  (2) The solution is sampled at S = 0 by the
// left-side logic only: on the left state as given when the contact moves
// right (u* >= 0), on the mirror image of the right state otherwise.  Every
// speed of the mirrored sampling is the exact negation of the right-side
// speed it stands for, and the ties at zero are resolved as the right-side
// tests resolve them, so the sampled state is the one of the two-sided
// sampling (Toro section 4.5).
// State of the gamma = 5/3 solver between its phases: the sorted sides, the
// Newton iterate and, once converged, f_K(p*) and (p*/p_K)^(1/5).
struct Solve5 {
    RiemannSide A, B;
    double du, pfloor, p, fAs, fBs, qAs, qBs;
    int iters;   // Newton steps run (a restart from p_TR counts max_iter first); -1: no convergence
    int stage;   // 0 vacuum; 1 Newton done (finish next); 2 stopped unfinished; 3 strong shock deferred
    bool mir;
};

// Newton from p0 (raised to the floor) on the sorted problem; with
// tried_guess, a start that does not converge is retried from p_TR.
// first_iters > 0 (not with tried_guess): stop unfinished after that many
// steps (stage 2, s.p the iterate).
__device__ __forceinline__ void riemann5_newton(const RiemannConsts &k, Solve5 &s, double p0, bool tried_guess,
                                                int first_iters) {
    const RiemannSide &A = s.A, &B = s.B;
    const double du = s.du, pfloor = s.pfloor;
    double p = p0;
    int iters = -1, extra = 0;
    s.fAs = 0.; s.fBs = 0.; s.qAs = -1.; s.qBs = -1.;
    for (int attempt = 0; attempt < 2 && iters < 0; ++attempt) {
        if (attempt == 1) {
            if (!tried_guess) break;
            extra = k.max_iter;
            double num = A.c + B.c - k.g7 * du;
            double den = A.c * rroot5(A.p) + B.c * rroot5(B.p);
            double t = fdiv(num, den);
            double t2 = t * t;
            p0 = t2 * t2 * t;
        }
        p = nn_le(p0, pfloor) ? pfloor : p0;
        for (int it = 1; it <= k.max_iter; ++it) {
            double invp = frcp(p);
            double fA, fdA, qA, fB, fdB, qB;
            bool rA, rB;
            pressure_fn5(A, p, invp, fA, fdA, qA, rA);
            pressure_fn5(B, p, invp, fB, fdB, qB, rB);
            double pnew = p - (fA + fB + du) * frcp(fdA + fdB);
            {   // !(pnew > 0): zero, negative or NaN (bit patterns)
                const long long pb = __double_as_longlong(pnew);
                if (pb <= 0 || pb > 0x7FF0000000000000ll) pnew = pfloor;
            }
            double dp = pnew - p;
            if (nn_le(fabs(dp), k.tol_half * (pnew + p))) {
                s.fAs = fA + fdA * dp;
                s.fBs = fB + fdB * dp;
                double rel = dp * invp;
                s.qAs = rA ? qA + qA * (k.g1 * rel) : -1.;
                s.qBs = rB ? qB + qB * (k.g1 * rel) : -1.;
                p = pnew;
                iters = it;
                break;
            }
            p = pnew;
            if (first_iters > 0 && !tried_guess && it >= first_iters) {
                s.p = p; s.iters = it; s.stage = 2;
                return;
            }
        }
    }
    s.p = p;
    s.iters = iters < 0 ? -1 : iters + extra;
    s.stage = 1;
}

// The sides, the vacuum test, the start (the given guess, or p_TR) and the
// Newton iteration of riemann_exact5, up to its optional stops.
__device__ __forceinline__ Solve5 riemann5_begin(const RiemannConsts &k, double rhoL, double uL, double pL,
                                                 double rhoR, double uR, double pR, double guess,
                                                 double defer_above, int first_iters) {
    Solve5 s;
    s.mir = dlt(pR, pL);
    const bool mir = s.mir;
    s.A = make_side(k, mir ? rhoR : rhoL, mir ? flip_if(uR, true) : uL, mir ? pR : pL);
    s.B = make_side(k, mir ? rhoL : rhoR, mir ? flip_if(uL, true) : uR, mir ? pL : pR);
    s.fAs = 0.; s.fBs = 0.; s.qAs = -1.; s.qBs = -1.; s.iters = 0; s.p = 0.;
    if (!dlt(s.B.u - s.A.u, k.g4 * (s.A.c + s.B.c))) {   // g4 (cL + cR) <= uR - uL: vacuum
        s.stage = 0;
        return s;
    }
    s.du = s.B.u - s.A.u;
    s.pfloor = 1e-12 * s.B.p;                   // 1e-12 max(pL, pR)
    double p0;
    const bool tried_guess = __double_as_longlong(guess) > 0;   // guess > 0 (-1: none)
    if (tried_guess) p0 = guess;
    else {
        double num = s.A.c + s.B.c - k.g7 * s.du;
        double den = s.A.c * rroot5(s.A.p) + s.B.c * rroot5(s.B.p);
        double t = fdiv(num, den);
        double t2 = t * t;
        p0 = t2 * t2 * t;
        // defer_above > 0 and p0 > defer_above, on the keys (see riemann_exact)
        if (ord_key(defer_above) > 0 && dlt(defer_above, p0)) {
            s.p = p0; s.stage = 3;
            return s;
        }
    }
    riemann5_newton(k, s, p0, tried_guess, first_iters);
    return s;
}

// Continue a solve stopped unfinished (stage 2) from its iterate: the same
// iteration as restarting riemann_exact5 with the iterate as the guess.
__device__ __forceinline__ void riemann5_continue(const RiemannConsts &k, Solve5 &s) {
    riemann5_newton(k, s, s.p, true, 0);
}

__device__ inline RiemannResult riemann5_finish(const RiemannConsts &k, const Solve5 &s);

__device__ inline RiemannResult riemann_exact5(const RiemannConsts &k, double rhoL, double uL, double pL,
                                               double rhoR, double uR, double pR, double guess = -1.,
                                               double defer_above = 0., int first_iters = 0) {
    const Solve5 s = riemann5_begin(k, rhoL, uL, pL, rhoR, uR, pR, guess, defer_above, first_iters);
    RiemannResult res;
    if (s.stage == 0) {
        res.rho = 0.; res.u = 0.; res.p = 0.; res.pstar = 0.; res.flag = 0; res.iters = 0;
        return res;
    }
    if (s.stage >= 2) {   // unfinished (the iterate) or deferred strong shock (p_TR)
        res.rho = 0.; res.u = 0.; res.p = 0.; res.pstar = s.p; res.flag = 2; res.iters = s.stage == 2 ? s.iters : 0;
        return res;
    }
    return riemann5_finish(k, s);
}

// u* and the sampled state of a converged (or given-up) solve.
__device__ inline RiemannResult riemann5_finish(const RiemannConsts &k, const Solve5 &s) {
    RiemannResult res;
    const RiemannSide &A = s.A, &B = s.B;
    const bool mir = s.mir;
    double fAs = s.fAs, fBs = s.fBs, qAs = s.qAs, qBs = s.qBs;
    const double p = s.p;
    const double pstar = p;
    res.pstar = pstar;
    if (s.iters < 0) {
        double invp = frcp(pstar), fdA, fdB, qA, qB;
        bool rA, rB;
        pressure_fn5(A, pstar, invp, fAs, fdA, qA, rA);
        pressure_fn5(B, pstar, invp, fBs, fdB, qB, rB);
        qAs = rA ? qA : -1.;
        qBs = rB ? qB : -1.;
    }
    res.iters = s.iters;
    // u* of the given problem (the sorted one's, negated when mirrored)
    // .5 (uA + uB) + .5 (fB - fA) = .5 ((uA + uB) + (fB - fA)): halving is
    // exact, so one rounding of the sum, halved on the integer pipe
    const double ustar = flip_if(half_of((A.u + B.u) + (fBs - fAs)), mir);
    // --- sampling at S = 0: side s of the contact, as the left side
    const bool right = dneg(ustar);               // u* < 0: the right state
    const bool useB = right != mir;               // where side s sits in the sorted problem
    const double rho_s = useB ? B.rho : A.rho, p_s = useB ? B.p : A.p, c_s = useB ? B.c : A.c;
    const double invp_s = useB ? B.invp : A.invp, q_s = useB ? qBs : qAs;
    // the side's velocity, mirrored for the right side: the sorted problem
    // holds it negated when mirrored, so the two flips combine into useB
    const double u_s = flip_if(useB ? B.u : A.u, useB);
    const double ustar_s = flip_if(ustar, right);
    double rho, u, pp;
    if (nn_le(pstar, p_s)) {                      // rarefaction on side s
        const double sh = __dsub_rn(u_s, c_s);    // head speed
        if (!dneg(sh)) { rho = rho_s; u = u_s; pp = p_s; }
        else {
            const double q = !dneg(q_s) ? q_s : root5(pstar * invp_s);
            const double st = __fma_rn(-c_s, q, ustar_s);   // tail speed
            // tail < 0 puts S = 0 in the star region (left side); the right
            // side's test, tail >= 0 there, reads tail <= 0 mirrored
            const long long kst = ord_key(st);
            if (right ? kst <= 0 : kst < 0) { rho = rho_s * (q * q * q); u = ustar_s; pp = pstar; }
            else {
                const double cf = k.g5 * __fma_rn(k.g7, u_s, c_s);
                const double r = fdiv(cf, c_s), r3 = r * r * r;
                u = cf; rho = rho_s * r3; pp = p_s * (r3 * r * r);
            }
        }
    } else {                                      // shock on side s
        const double pm = pstar * invp_s;
        const double sl = __fma_rn(-c_s, sqrt(k.g2 * pm + k.g1), u_s);   // shock speed
        if (!dneg(sl)) { rho = rho_s; u = u_s; pp = p_s; }
        else { rho = rho_s * fdiv(pm + k.g6, pm * k.g6 + 1.); u = ustar_s; pp = pstar; }
    }
    res.flag = right ? 1 : -1;
    res.rho = rho; res.u = flip_if(u, right); res.p = pp;
    return res;
}

}  // namespace mlh
