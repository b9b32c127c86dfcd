// TEST INFRASTRUCTURE (oracle).  Not part of the product: only tests/, the
// smoke check and bench.py's CPU baseline load this library, to compare against.
//
// A plain, serial CPU restatement of one MFV (meshless finite volume) step of
// the reference demonstrator, jammartin/meshlessHydro.  Every stage follows the
// reference method it names, with the same floating-point expression order, so
// that on identical inputs it reproduces the reference's numbers (bit for bit
// where the reference's own arithmetic is used; see the notes on the matrix
// inverse and on the Riemann solver).
//
// Stage order: demonstrator/src/MeshlessScheme.cpp:39-253.
//
// Differences from the reference, all deliberate:
//  * Matrix inverse: closed-form adjugate / determinant instead of LAPACK
//    dgetrf_+dgetri_ (demonstrator/src/Helper.cpp:7-18).  Agrees to rounding.
//  * Exact Riemann solver: own restatement of Toro ch. 4 (riemann_exact.hpp);
//    the reference's third-party RiemannSolver.hpp is not in its tree.
//  * Periodic images: the reference builds explicit ghost copies and searches
//    them by brute force (Particles.cpp:2113-2260, 2D only).  This restatement
//    finds the same images through the wrapped cell stencil and orders them by
//    parent index, which is the reference's ghost order (ghosts are created in
//    parent order, one image of a parent at most lies within h when every
//    periodic axis has >= 3 cells).  It extends that arithmetic per axis to 3D.
//  * In 3D with FIRST_ORDER_QUAD_POINT the reference reads an uninitialised
//    xjxi[2] in the pairwise limiter (Particles.cpp:1498-1539, 1623-1631); this
//    restatement uses z_j - z_i.
//  * Errors set bits in the returned status instead of calling exit().
//
// Threads: built with OpenMP, the per-particle loops run on several threads
// (orc_set_threads; one by default).  Every particle's sums run in the same
// order on one thread whatever the thread count, the minimum of the time step
// is taken after the loop, and the faces are solved before their mirrored
// copies are made, so the results do not depend on the number of threads.
//
// Addition without a reference counterpart (the reference uses one global
// kernelSize): per-particle smoothing lengths (hsolve) and the step mode that
// uses them (adaptive_h).  Its arithmetic is fixed operation by operation
// (explicit fma, the candidate order of the cell stencil, 32 strided partial
// sums combined pairwise at distances 16, 8, 4, 2, 1) so that a data-parallel
// implementation that sums the same way gets the same smoothing lengths bit
// for bit.
#include "mlh_oracle.h"
#ifdef ORC_COUNT_FLOPS
#include "flop_count.hpp"
#endif
#include "riemann_exact.hpp"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// threads of the per-particle loops (orc_set_threads)
int g_threads = 1;

// Arithmetic type of the step: double, or (operation-counting build,
// -DORC_COUNT_FLOPS) a double that counts the operations done on it.
#ifdef ORC_COUNT_FLOPS
using real = orc::Counted;
#else
using real = double;
#endif
using std::fabs;
using std::floor;
using std::fma;
using std::pow;
using std::sqrt;

enum Status {
    ST_OK = 0,
    ST_NEG_PRESSURE = 1 << 1,
    ST_NEG_DENSITY = 1 << 2,
    ST_NEG_MASS = 1 << 3,
    ST_NEG_ENERGY = 1 << 4,
    ST_NEWTON = 1 << 5,
    ST_VACUUM = 1 << 6,
    ST_GRID = 1 << 7,
    ST_NO_NEIGHBOUR = 1 << 8,
};

const unsigned IMG_SHIFT = 29;
const unsigned IDX_MASK = (1u << IMG_SHIFT) - 1u;

// abs() as the reference binds it.  With only <cmath>/<iostream> visible, the
// unqualified abs(double) at Particles.cpp:1416-1417, 1748-1749, 1754, 1759
// resolves to int ::abs(int): the double is truncated (x86 cvttsd2si gives
// INT_MIN for NaN and out-of-range values, and abs(INT_MIN) stays INT_MIN).
inline real ref_abs(real x, int int_abs) {
    if (!int_abs) return fabs(x);
    int t;
    if (!(x > -2147483649.0 && x < 2147483648.0)) t = INT_MIN;
    else t = (int)x;
    if (t == INT_MIN) return (real)INT_MIN;
    return (real)(t < 0 ? -t : t);
}

template <int D>
struct Sim {
    orc_config c;
    int N;
    double h;                        // kernelSize: the support radius, or its maximum with adaptive_h
    std::vector<double> hp;          // per-particle support radius (h everywhere without adaptive_h)
    std::vector<real> nEff;          // effective neighbour number of the last h solve
    long hClamped = 0, hIters = 0;
    std::vector<real> X[3], V[3], m, u, rho, P, omega;
    // gradients in the reference's call order: rho, vx, vy, (vz), P
    std::vector<real> G[5];          // [field][i*3+alpha]
    std::vector<real> Graw[5];       // unlimited copies (for tests)
    std::vector<real> B;             // inverse of E_i, D*D per particle
    // neighbour lists: real neighbours first (grid stencil order), then
    // periodic images ordered by parent index
    std::vector<int> off, noi, noiImg;
    std::vector<uint32_t> nb;
    std::vector<int> rev;              // slot of i in the neighbour's list
    std::vector<real> psi, Aij, WL, WR, vFrame, F;
    std::vector<real> mF, vF, eF;
    std::vector<int> newtonIters;
    std::vector<int> slotIters;        // Newton steps of each slot's face (copies: the face's)
    double dt = 0.;
    real lo[3], hi[3];
    int cells[3];
    real cellSize[3];
    std::vector<int> cellOf;
    std::vector<std::vector<int>> grid;
    // error bits; OR-ed from the threads of the per-particle loops
    std::atomic<unsigned> status{0};
    long riemannSolves = 0, newtonTotal = 0;

    // --- Kernel::cubicSpline, demonstrator/src/Particles.cpp:7-24, for a
    // support radius hh (the reference's kernelSize)
    real kernel(real r) const { return kernelH(r, h); }
    real kernelH(real r, double hh) const {
        double h2 = hh / 2.;
        double sigma = (D == 2) ? 10. / (7. * M_PI * h2 * h2) : 1. / (M_PI * h2 * h2 * h2);
        real q = r / h2;
        if (0. <= q && q <= 1.) return sigma * (1. - 3. / 2. * q * q * (1. - q / 2.));
        else if (1. < q && q < 2.) return sigma / 4. * pow(2. - q, 3.);
        return 0.;
    }

    // field accessor in gradient order
    const std::vector<real> &field(int f) const {
        if (f == 0) return rho;
        if (f == D + 1) return P;
        return V[f - 1];
    }
    int nfields() const { return D + 2; }

    // image coordinate of a particle coordinate along axis a, ghost rule of
    // Particles.cpp:2123-2142 (returns false when the particle has no image)
    bool image(int a, real xa, real &out) const {
        if (xa <= lo[a] + h) { out = hi[a] + (xa - lo[a]); return true; }
        else if (hi[a] - h < xa) { out = lo[a] - (hi[a] - xa); return true; }
        return false;
    }
    // coordinates of neighbour entry e (index + image bits)
    void coords(uint32_t e, real *xj) const {
        int j = (int)(e & IDX_MASK);
        for (int a = 0; a < D; ++a) {
            xj[a] = X[a][j];
            if (e & (1u << (IMG_SHIFT + a))) image(a, X[a][j], xj[a]);
        }
    }

    // --- Particles::getDomainLimits, Particles.cpp:228-267 (else-if and
    // numeric_limits<double>::min() kept)
    void domainLimits() {
        for (int a = 0; a < D; ++a) { lo[a] = std::numeric_limits<double>::max(); hi[a] = std::numeric_limits<double>::min(); }
        for (int i = 0; i < N; ++i)
            for (int a = 0; a < D; ++a) {
                if (X[a][i] < lo[a]) lo[a] = X[a][i];
                else if (X[a][i] > hi[a]) hi[a] = X[a][i];
            }
    }

    // --- Domain::createGrid, demonstrator/src/Domain.cpp:9-54
    void createGrid() {
        long total = 1;
        for (int a = 0; a < D; ++a) {
            cells[a] = (int)floor((hi[a] - lo[a]) / h);
            if (cells[a] < 1) { status |= ST_GRID; cells[a] = 1; }
            total *= cells[a];
        }
        for (int a = 0; a < D; ++a) cellSize[a] = (hi[a] - lo[a]) / (real)cells[a];
        if (c.periodic)
            for (int a = 0; a < D; ++a) if (cells[a] < 3) status |= ST_GRID;
        grid.assign(total, std::vector<int>());
    }

    // --- Particles::assignParticlesAndCells, Particles.cpp:270-322
    void assign() {
        for (auto &g : grid) g.clear();
        cellOf.assign(N, 0);
        for (int i = 0; i < N; ++i) {
            int fl[3] = {0, 0, 0};
            for (int a = 0; a < D; ++a) {
                fl[a] = (int)floor((X[a][i] - lo[a]) / cellSize[a]);
                if (fl[a] == cells[a]) fl[a] -= 1;
                if (fl[a] < 0 || fl[a] >= cells[a]) { status |= ST_GRID; fl[a] = fl[a] < 0 ? 0 : cells[a] - 1; }
            }
            int ic = fl[0] + fl[1] * cells[0] + (D == 3 ? fl[2] * cells[0] * cells[1] : 0);
            grid[ic].push_back(i);
            cellOf[i] = ic;
        }
    }

    // --- Particles::gridNNS (Particles.cpp:324-365) with the stencil of
    // Domain::getNeighborCells (Domain.cpp:83-118), plus the periodic images
    // (Particles::ghostNNS, Particles.cpp:2237-2260) found through wrapped cells.
    // squared search radius of a pair: h^2, or max(h_i^2, h_j^2) with
    // per-particle smoothing lengths (j the parent of an image)
    real pairSq(int i, int j, real hSqr) const {
        if (!c.adaptive_h) return hSqr;
        real a = hp[i] * hp[i], b = hp[j] * hp[j];
        return a > b ? a : b;
    }

    void nns() {
        const real hSqr = h * h;
        off.assign(N + 1, 0);
        noi.assign(N, 0);
        noiImg.assign(N, 0);
        std::vector<std::vector<uint32_t>> lists(N);
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {
            int ic = cellOf[i];
            int ix = ic % cells[0];
            int iy = (ic / cells[0]) % cells[1];
            int iz = D == 3 ? ic / (cells[0] * cells[1]) : 0;
            std::vector<uint32_t> own, img;   // real neighbours, periodic images
            for (int k = ix - 1; k <= ix + 1; ++k)
                for (int l = iy - 1; l <= iy + 1; ++l)
                    for (int mm = (D == 3 ? iz - 1 : 0); mm <= (D == 3 ? iz + 1 : 0); ++mm) {
                        int cc[3] = {k, l, mm};
                        unsigned wrap = 0;
                        bool skip = false;
                        for (int a = 0; a < D; ++a) {
                            if (cc[a] < 0 || cc[a] >= cells[a]) {
                                if (!c.periodic) { skip = true; break; }
                                cc[a] = cc[a] < 0 ? cc[a] + cells[a] : cc[a] - cells[a];
                                wrap |= 1u << a;
                            }
                        }
                        if (skip) continue;
                        int cell = cc[0] + cc[1] * cells[0] + (D == 3 ? cc[2] * cells[0] * cells[1] : 0);
                        for (int j : grid[cell]) {
                            if (!wrap) {
                                if (j == i) continue;
                                real dSqr = (X[0][j] - X[0][i]) * (X[0][j] - X[0][i])
                                            + (X[1][j] - X[1][i]) * (X[1][j] - X[1][i]);
                                if (D == 3) dSqr += (X[2][j] - X[2][i]) * (X[2][j] - X[2][i]);
                                if (dSqr < pairSq(i, j, hSqr)) own.push_back((uint32_t)j);
                            } else {
                                real xj[3];
                                bool ok = true;
                                for (int a = 0; a < D; ++a) {
                                    xj[a] = X[a][j];
                                    if (wrap & (1u << a)) ok = ok && image(a, X[a][j], xj[a]);
                                }
                                if (!ok) continue;
                                real dSqr = (xj[0] - X[0][i]) * (xj[0] - X[0][i])
                                            + (xj[1] - X[1][i]) * (xj[1] - X[1][i]);
                                if (D == 3) dSqr += (xj[2] - X[2][i]) * (xj[2] - X[2][i]);
                                if (dSqr < pairSq(i, j, hSqr)) img.push_back((uint32_t)j | (wrap << IMG_SHIFT));
                            }
                        }
                    }
            std::sort(img.begin(), img.end(), [](uint32_t a, uint32_t b) { return (a & IDX_MASK) < (b & IDX_MASK); });
            if (own.empty() && img.empty()) status |= ST_NO_NEIGHBOUR;
            noi[i] = (int)own.size();
            noiImg[i] = (int)img.size();
            lists[i] = own;
            lists[i].insert(lists[i].end(), img.begin(), img.end());
        }
        for (int i = 0; i < N; ++i) off[i + 1] = off[i] + (int)lists[i].size();
        nb.resize(off[N]);
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) std::copy(lists[i].begin(), lists[i].end(), nb.begin() + off[i]);
        // reverse slots: position of i in the list of its neighbour (for
        // images: the first image entry of the parent whose parent is i,
        // Particles.cpp:2514-2516)
        rev.assign(off[N], -1);
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s) {
                int j = (int)(nb[s] & IDX_MASK);
                bool isImg = (s - off[i]) >= noi[i];
                int b = isImg ? off[j] + noi[j] : off[j];
                int e = isImg ? off[j + 1] : off[j] + noi[j];
                for (int t = b; t < e; ++t)
                    if ((int)(nb[t] & IDX_MASK) == i) { rev[s] = t; break; }
            }
    }

    real dist(int i, int s) const {
        real xj[3];
        coords(nb[s], xj);
        real dSqr = (X[0][i] - xj[0]) * (X[0][i] - xj[0]) + (X[1][i] - xj[1]) * (X[1][i] - xj[1]);
        if (D == 3) dSqr += (X[2][i] - xj[2]) * (X[2][i] - xj[2]);
        return sqrt(dSqr);
    }

    // --- Particles::compDensity/compOmega, Particles.cpp:1151-1184 and the
    // image part 2262-2290
    void density() {
        omega.assign(N, 0.);
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {
            real omg = 0.;
            for (int s = off[i]; s < off[i] + noi[i]; ++s) omg += kernelH(dist(i, s), hp[i]);
            omega[i] = omg + kernelH(0., hp[i]);
            rho[i] = m[i] * omega[i];
            if (rho[i] <= 0.) status |= ST_NEG_DENSITY;
        }
        if (c.periodic) {
#pragma omp parallel for schedule(static) num_threads(g_threads)
            for (int i = 0; i < N; ++i) {
                real omg = omega[i];
                for (int s = off[i] + noi[i]; s < off[i + 1]; ++s) omg += kernelH(dist(i, s), hp[i]);
                omega[i] = omg;
                rho[i] = m[i] * omega[i];
            }
        }
    }

    // --- Particles::compPressure, Particles.cpp:1272-1288
    void pressure() {
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {
            P[i] = (c.gamma - 1.) * rho[i] * u[i];
            if (P[i] <= 0.) status |= ST_NEG_PRESSURE;
        }
    }

    static real dot(const real *a, const real *b) {
        real r = 0.;
        for (int k = 0; k < D; ++k) r += a[k] * b[k];
        return r;
    }

    // --- Particles::compGlobalTimestep, Particles.cpp:1446-1485 (real
    // neighbours only, v_sig starting at numeric_limits<double>::min())
    real globalTimestep() {
        real dt_ = std::numeric_limits<double>::max();
        std::vector<real> dtp(N);
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {
            real vSig = std::numeric_limits<double>::min();
            real ci = sqrt(c.gamma * P[i] / rho[i]);
            for (int s = off[i]; s < off[i] + noi[i]; ++s) {
                int j = (int)(nb[s] & IDX_MASK);
                real cj = sqrt(c.gamma * P[j] / rho[j]);
                real xij[3], vij[3];
                for (int a = 0; a < D; ++a) { xij[a] = X[a][i] - X[a][j]; vij[a] = V[a][i] - V[a][j]; }
                real vijxij = dot(vij, xij) / sqrt(dot(xij, xij));
                vijxij = vijxij < 0. ? vijxij : 0.;
                real vSig_i = ci + cj - vijxij;
                vSig = vSig_i > vSig ? vSig_i : vSig;
            }
            dtp[i] = c.cfl * hp[i] / vSig;
        }
        for (int i = 0; i < N; ++i) dt_ = dtp[i] < dt_ ? dtp[i] : dt_;
        return dt_;
    }

    // closed-form inverse (replaces Helper::inverseMatrix, Helper.cpp:7-18)
    static void invert(real *A) {
        if (D == 2) {
            real a = A[0], b = A[1], cc = A[2], d = A[3];
            real det = a * d - b * cc;
            real id = 1. / det;
            A[0] = d * id; A[1] = -b * id; A[2] = -cc * id; A[3] = a * id;
        } else {
            real a00 = A[0], a01 = A[1], a02 = A[2], a10 = A[3], a11 = A[4], a12 = A[5], a20 = A[6], a21 = A[7], a22 = A[8];
            real c00 = a11 * a22 - a12 * a21;
            real c01 = a12 * a20 - a10 * a22;
            real c02 = a10 * a21 - a11 * a20;
            real det = a00 * c00 + a01 * c01 + a02 * c02;
            real id = 1. / det;
            A[0] = c00 * id;
            A[1] = (a02 * a21 - a01 * a22) * id;
            A[2] = (a01 * a12 - a02 * a11) * id;
            A[3] = c01 * id;
            A[4] = (a00 * a22 - a02 * a20) * id;
            A[5] = (a02 * a10 - a00 * a12) * id;
            A[6] = c02 * id;
            A[7] = (a01 * a20 - a00 * a21) * id;
            A[8] = (a00 * a11 - a01 * a10) * id;
        }
    }

    // --- Particles::compPsijTilde, Particles.cpp:1186-1254 / 2292-2455
    void psijTilde() {
        B.assign((size_t)N * D * D, 0.);
        psi.assign((size_t)off[N] * 3, 0.);
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {
            real Bi[9] = {0};
            real xi[3];
            for (int a = 0; a < D; ++a) xi[a] = X[a][i];
            for (int s = off[i]; s < off[i + 1]; ++s) {
                real r = dist(i, s);
                real psij_xi = kernelH(r, hp[i]) / omega[i];
                real xj[3];
                coords(nb[s], xj);
                for (int al = 0; al < D; ++al)
                    for (int be = 0; be < D; ++be)
                        Bi[D * al + be] += (xj[al] - xi[al]) * (xj[be] - xi[be]) * psij_xi;
            }
            invert(Bi);
            for (int k = 0; k < D * D; ++k) B[(size_t)i * D * D + k] = Bi[k];
            for (int s = off[i]; s < off[i + 1]; ++s) {
                real r = dist(i, s);
                real psij_xi = kernelH(r, hp[i]) / omega[i];
                real xj[3];
                coords(nb[s], xj);
                for (int al = 0; al < D; ++al) {
                    real p = 0.;
                    for (int be = 0; be < D; ++be) p += Bi[D * al + be] * (xj[be] - xi[be]) * psij_xi;
                    psi[(size_t)s * 3 + al] = p;
                }
            }
        }
    }

    // --- Particles::gradient, Particles.cpp:1257-1270 / 2457-2502
    void gradients() {
        for (int f = 0; f < nfields(); ++f) {
            const std::vector<real> &fv = field(f);
            G[f].assign((size_t)N * 3, 0.);
#pragma omp parallel for schedule(static) num_threads(g_threads)
            for (int i = 0; i < N; ++i)
                for (int s = off[i]; s < off[i + 1]; ++s) {
                    int j = (int)(nb[s] & IDX_MASK);
                    for (int a = 0; a < D; ++a) G[f][(size_t)i * 3 + a] += (fv[j] - fv[i]) * psi[(size_t)s * 3 + a];
                }
            Graw[f] = G[f];
        }
    }

    // --- Particles::slopeLimiter, Particles.cpp:1313-1444
    void slopeLimiter() {
        for (int f = 0; f < nfields(); ++f) {
            const std::vector<real> &fv = field(f);
#pragma omp parallel for schedule(static) num_threads(g_threads)
            for (int i = 0; i < N; ++i) {
                real psiMaxNgb = std::numeric_limits<double>::min();
                real psiMinNgb = std::numeric_limits<double>::max();
                real psiMaxMid = std::numeric_limits<double>::min();
                real psiMinMid = std::numeric_limits<double>::max();
                real *g = &G[f][(size_t)i * 3];
                for (int s = off[i]; s < off[i + 1]; ++s) {
                    int j = (int)(nb[s] & IDX_MASK);
                    real xj[3], xij[3], xijxi[3];
                    coords(nb[s], xj);
                    for (int a = 0; a < D; ++a) {
                        if (c.first_order_quad_point) xij[a] = (X[a][i] + xj[a]) / 2.;
                        else xij[a] = X[a][i] + hp[i] / 4. * (xj[a] - X[a][i]);
                        xijxi[a] = xij[a] - X[a][i];
                    }
                    if (psiMaxNgb < fv[j]) psiMaxNgb = fv[j];
                    if (psiMinNgb > fv[j]) psiMinNgb = fv[j];
                    real fij = fv[i] + dot(g, xijxi);
                    if (psiMaxMid < fij) psiMaxMid = fij;
                    if (psiMinMid > fij) psiMinMid = fij;
                }
                real alphaMax = ref_abs((psiMaxNgb - fv[i]) / (psiMaxMid - fv[i]), c.int_abs);
                real alphaMin = ref_abs((fv[i] - psiMinNgb) / (fv[i] - psiMinMid), c.int_abs);
                if (alphaMin <= alphaMax && c.beta * alphaMin < 1.) {
                    for (int a = 0; a < D; ++a) g[a] *= alphaMin;
                } else if (alphaMax <= alphaMin && c.beta * alphaMax < 1.) {
                    for (int a = 0; a < D; ++a) g[a] *= alphaMax;
                }
            }
        }
    }

    // --- Particles::compEffectiveFace, Particles.cpp:1290-1311 / 2504-2531
    void effectiveFace() {
        Aij.assign((size_t)off[N] * 3, 0.);
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s) {
                int j = (int)(nb[s] & IDX_MASK);
                int t = rev[s];
                for (int a = 0; a < D; ++a)
                    Aij[(size_t)s * 3 + a] = 1. / omega[i] * psi[(size_t)s * 3 + a] - 1. / omega[j] * psi[(size_t)t * 3 + a];
            }
    }

    // --- Particles::pairwiseLimiter, Particles.cpp:1735-1785
    real pairwiseLimiter(real phi0, real phi_i, real phi_j, real xijxi_abs, real xjxi_abs) const {
        real phi_ = phi_i;
        real phi_ij = phi_i + xijxi_abs / xjxi_abs * (phi_j - phi_i);
        real phiMin, phiMax;
        if (phi_i < phi_j) { phiMin = phi_i; phiMax = phi_j; }
        else { phiMin = phi_j; phiMax = phi_i; }
        real delta1 = c.psi1 * ref_abs(phi_i - phi_j, c.int_abs);
        real delta2 = c.psi2 * ref_abs(phi_i - phi_j, c.int_abs);
        real phiMinus, phiPlus;
        if ((phiMax + delta1 >= 0. && phiMax >= 0.) || (phiMax + delta1 < 0. && phiMax < 0.)) phiPlus = phiMax + delta1;
        else phiPlus = phiMax / (1. + delta1 / ref_abs(phiMax, c.int_abs));
        if ((phiMin - delta1 >= 0. && phiMin >= 0.) || (phiMin - delta1 < 0. && phiMin < 0.)) phiMinus = phiMin - delta1;
        else phiMinus = phiMin / (1. + delta1 / ref_abs(phiMin, c.int_abs));
        if (phi_i < phi_j) {
            real minPhiD2 = (phi_ij + delta2 < phi0) ? phi_ij + delta2 : phi0;
            phi_ = phiMinus > minPhiD2 ? phiMinus : minPhiD2;
        } else if (phi_i > phi_j) {
            real maxPhiD2 = (phi_ij - delta2 > phi0) ? phi_ij - delta2 : phi0;
            phi_ = phiPlus < maxPhiD2 ? phiPlus : maxPhiD2;
        }
        return phi_;
    }

    // --- Particles::compRiemannStatesLR, Particles.cpp:1488-1733 (real) and
    // 2533-2683 (images: no pairwise limiter unless image_pairwise_limiter)
    void riemannStatesLR() {
        const int NV = D + 2;
        WL.assign((size_t)off[N] * NV, 0.);
        WR.assign((size_t)off[N] * NV, 0.);
        vFrame.assign((size_t)off[N] * 3, 0.);
        const std::vector<real> &rG = G[0], &vxG = G[1], &vyG = G[2], &vzG = G[3], &PG = G[D + 1];
        const real gamma = c.gamma;
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s) {
                int j = (int)(nb[s] & IDX_MASK);
                bool isImg = (s - off[i]) >= noi[i];
                real xj[3], xij[3], xijxi[3], xjxi[3], xijxj[3];
                coords(nb[s], xj);
                for (int a = 0; a < D; ++a) {
                    xjxi[a] = xj[a] - X[a][i];
                    if (c.first_order_quad_point) {
                        xij[a] = (X[a][i] + xj[a]) / 2.;
                        xijxj[a] = .5 * (X[a][i] - xj[a]);
                        xijxi[a] = .5 * (xj[a] - X[a][i]);
                    } else {
                        xij[a] = X[a][i] + hp[i] / 4. * xjxi[a];
                        xijxi[a] = xij[a] - X[a][i];
                        xijxj[a] = xij[a] - xj[a];
                    }
                }
                real *vf = &vFrame[(size_t)s * 3];
                if (!c.move_particles) { for (int a = 0; a < D; ++a) vf[a] = 0.; }
                else if (c.first_order_quad_point) { for (int a = 0; a < D; ++a) vf[a] = (V[a][i] + V[a][j]) / 2.; }
                else {
                    real dotProd = dot(xijxi, xjxi);
                    real dSqr = dot(xjxi, xjxi);
                    for (int a = 0; a < D; ++a) vf[a] = V[a][i] + (V[a][j] - V[a][i]) * dotProd / dSqr;
                }
                real *R = &WR[(size_t)s * NV], *L = &WL[(size_t)s * NV];
                R[0] = rho[i]; L[0] = rho[j];
                R[1] = P[i]; L[1] = P[j];
                for (int a = 0; a < D; ++a) { R[2 + a] = V[a][i] - vf[a]; L[2 + a] = V[a][j] - vf[a]; }
                real Rb[5], Lb[5];
                for (int nu = 0; nu < NV; ++nu) { Rb[nu] = R[nu]; Lb[nu] = L[nu]; }
                const real *gi, *gj;
                size_t I = (size_t)i * 3, J = (size_t)j * 3;
                R[0] += dot(&rG[I], xijxi); L[0] += dot(&rG[J], xijxj);
                R[1] += dot(&PG[I], xijxi); L[1] += dot(&PG[J], xijxj);
                R[2] += dot(&vxG[I], xijxi); L[2] += dot(&vxG[J], xijxj);
                R[3] += dot(&vyG[I], xijxi); L[3] += dot(&vyG[J], xijxj);
                if (D == 3) { R[4] += dot(&vzG[I], xijxi); L[4] += dot(&vzG[J], xijxj); }
                (void)gi; (void)gj;
                if (c.pairwise_limiter && (!isImg || c.image_pairwise_limiter)) {
                    real xijxi_abs = 0., xijxj_abs = 0., xjxi_abs = 0.;
                    for (int a = 0; a < D; ++a) {
                        xijxi_abs += xijxi[a] * xijxi[a];
                        xijxj_abs += xijxj[a] * xijxj[a];
                        xjxi_abs += xjxi[a] * xjxi[a];
                    }
                    xijxi_abs = sqrt(xijxi_abs);
                    xijxj_abs = sqrt(xijxj_abs);
                    xjxi_abs = sqrt(xjxi_abs);
                    for (int nu = 0; nu < NV; ++nu) {
                        R[nu] = pairwiseLimiter(R[nu], Rb[nu], Lb[nu], xijxi_abs, xjxi_abs);
                        L[nu] = pairwiseLimiter(L[nu], Lb[nu], Rb[nu], xijxj_abs, xjxi_abs);
                    }
                }
                real viDiv = vxG[I + 0] + vyG[I + 1];
                real vjDiv = vxG[J + 0] + vyG[J + 1];
                if (D == 3) { viDiv += vzG[I + 2]; vjDiv += vzG[J + 2]; }
                real vxi = V[0][i], vyi = V[1][i], vxj = V[0][j], vyj = V[1][j];
                R[0] -= dt / 2. * (rho[i] * viDiv + (vxi - vf[0]) * rG[I + 0] + (vyi - vf[1]) * rG[I + 1]);
                L[0] -= dt / 2. * (rho[j] * vjDiv + (vxj - vf[0]) * rG[J + 0] + (vyj - vf[1]) * rG[J + 1]);
                R[1] -= dt / 2. * (gamma * P[i] * viDiv + (vxi - vf[0]) * PG[I + 0] + (vyi - vf[1]) * PG[I + 1]);
                L[1] -= dt / 2. * (gamma * P[j] * vjDiv + (vxj - vf[0]) * PG[J + 0] + (vyj - vf[1]) * PG[J + 1]);
                R[2] -= dt / 2. * (PG[I + 0] / rho[i] + (vxi - vf[0]) * vxG[I + 0] + (vyi - vf[1]) * vxG[I + 1]);
                L[2] -= dt / 2. * (PG[J + 0] / rho[j] + (vxj - vf[0]) * vxG[J + 0] + (vyj - vf[1]) * vxG[J + 1]);
                R[3] -= dt / 2. * (PG[I + 1] / rho[i] + (vxi - vf[0]) * vyG[I + 0] + (vyi - vf[1]) * vyG[I + 1]);
                L[3] -= dt / 2. * (PG[J + 1] / rho[j] + (vxj - vf[0]) * vyG[J + 0] + (vyj - vf[1]) * vyG[J + 1]);
                if (D == 3) {
                    real vzi = V[2][i], vzj = V[2][j];
                    R[0] -= dt / 2. * (vzi - vf[2]) * rG[I + 2];
                    L[0] -= dt / 2. * (vzj - vf[2]) * rG[J + 2];
                    R[1] -= dt / 2. * (vzi - vf[2]) * PG[I + 2];
                    L[1] -= dt / 2. * (vzj - vf[2]) * PG[J + 2];
                    // Particles.cpp:1717,1719 use vz[i] on the j side
                    R[2] -= dt / 2. * (vzi - vf[2]) * vxG[I + 2];
                    L[2] -= dt / 2. * (vzi - vf[2]) * vxG[J + 2];
                    R[3] -= dt / 2. * (vzi - vf[2]) * vyG[I + 2];
                    L[3] -= dt / 2. * (vzi - vf[2]) * vyG[J + 2];
                    R[4] -= dt / 2. * (PG[I + 2] / rho[i] + (vxi - vf[0]) * vzG[I + 0] + (vyi - vf[1]) * vzG[I + 1] + (vzi - vf[2]) * vzG[I + 2]);
                    L[4] -= dt / 2. * (PG[J + 2] / rho[j] + (vxj - vf[0]) * vzG[J + 0] + (vyj - vf[1]) * vzG[J + 1] + (vzj - vf[2]) * vzG[J + 2]);
                }
            }
    }

    // --- Helper::rotationMatrix2D/3D, demonstrator/src/Helper.cpp:39-77
    static void rot2(const real *a, const real *b, real *L) {
        L[0] = a[0] * b[0] + a[1] * b[1];
        L[1] = -(a[0] * b[1] - a[1] * b[0]);
        L[2] = -L[1];
        L[3] = L[0];
    }
    static void rot3(const real *a, const real *b, real *L) {
        real v[3];
        v[0] = a[1] * b[2] - a[2] * b[1];
        v[1] = a[2] * b[0] - a[0] * b[2];
        v[2] = a[0] * b[1] - a[1] * b[0];
        real cosAB = dot(a, b);
        real n = 1. / (1. + cosAB);
        L[0] = 1. - n * (v[2] * v[2] + v[1] * v[1]);
        L[1] = -v[2] + n * v[0] * v[1];
        L[2] = v[1] + n * v[0] * v[2];
        L[3] = v[2] + n * v[0] * v[1];
        L[4] = 1. - n * (v[2] * v[2] + v[0] * v[0]);
        L[5] = -v[0] + n * v[1] * v[2];
        L[6] = -v[1] + n * v[0] * v[2];
        L[7] = v[0] + n * v[1] * v[2];
        L[8] = 1. - n * (v[1] * v[1] + v[0] * v[0]);
    }

    // --- Riemann::Riemann + Riemann::exact + rotateAndProjectFluxes2D/3D,
    // demonstrator/src/Riemann.cpp:7-229.  wi = state of the list owner i
    // (the reference's WijR, which the constructor receives as WL), wj = state
    // of neighbour j; i is the LEFT state of the 1D problem.
    // returns the Newton iterations (-1: no convergence)
    int riemann(real *wi, real *wj, const real *vfr, const real *A, real *Fo, const orc::ExactRiemannT<real> &rs) {
        const real unitX[3] = {1., 0., 0.};
        real AN = sqrt(dot(A, A));
        real hatA[3];
        for (int a = 0; a < D; ++a) hatA[a] = 1. / AN * A[a];
        real Lam[9];
        if (D == 2) {
            rot2(hatA, unitX, Lam);
            real bR[2] = {wj[2], wj[3]}, bL[2] = {wi[2], wi[3]};
            wj[2] = Lam[0] * bR[0] + Lam[1] * bR[1];
            wj[3] = Lam[2] * bR[0] + Lam[3] * bR[1];
            wi[2] = Lam[0] * bL[0] + Lam[1] * bL[1];
            wi[3] = Lam[2] * bL[0] + Lam[3] * bL[1];
        } else {
            rot3(hatA, unitX, Lam);
            real bR[3] = {wj[2], wj[3], wj[4]}, bL[3] = {wi[2], wi[3], wi[4]};
            wj[2] = Lam[0] * bR[0] + Lam[1] * bR[1] + Lam[2] * bR[2];
            wj[3] = Lam[3] * bR[0] + Lam[4] * bR[1] + Lam[5] * bR[2];
            wj[4] = Lam[6] * bR[0] + Lam[7] * bR[1] + Lam[8] * bR[2];
            wi[2] = Lam[0] * bL[0] + Lam[1] * bL[1] + Lam[2] * bL[2];
            wi[3] = Lam[3] * bL[0] + Lam[4] * bL[1] + Lam[5] * bL[2];
            wi[4] = Lam[6] * bL[0] + Lam[7] * bL[1] + Lam[8] * bL[2];
        }
        real rhoSol, vSol[3] = {0., 0., 0.}, PSol;
        int iters = 0;
        int flag = rs.solve(wi[0], wi[2], wi[1], wj[0], wj[2], wj[1], rhoSol, vSol[0], PSol, &iters);
        if (iters < 0) status |= ST_NEWTON;
        if (flag == 1) { for (int a = 1; a < D; ++a) vSol[a] = wj[2 + a]; }
        else if (flag == -1) { for (int a = 1; a < D; ++a) vSol[a] = wi[2 + a]; }
        else status |= ST_VACUUM;
        const real gamma = c.gamma;
        real LI[9];
        if (D == 2) {
            rot2(unitX, hatA, LI);
            real b[2] = {vSol[0], vSol[1]};
            vSol[0] = LI[0] * b[0] + LI[1] * b[1];
            vSol[1] = LI[2] * b[0] + LI[3] * b[1];
            Fo[0] = A[0] * rhoSol * vSol[0] + A[1] * rhoSol * vSol[1];
            real vLab[2] = {vSol[0] + vfr[0], vSol[1] + vfr[1]};
            if (c.meshless_finite_mass) { vSol[0] = 0.; vSol[1] = 0.; }
            Fo[2] = A[0] * (rhoSol * vLab[0] * vSol[0] + PSol) + A[1] * rhoSol * vLab[0] * vSol[1];
            Fo[3] = A[0] * rhoSol * vLab[1] * vSol[0] + A[1] * (rhoSol * vLab[1] * vSol[1] + PSol);
            Fo[1] = A[0] * (vSol[0] * (PSol / (gamma - 1.) + rhoSol * .5 * dot(vLab, vLab)) + PSol * vLab[0])
                  + A[1] * (vSol[1] * (PSol / (gamma - 1.) + rhoSol * .5 * dot(vLab, vLab)) + PSol * vLab[1]);
        } else {
            rot3(unitX, hatA, LI);
            real b[3] = {vSol[0], vSol[1], vSol[2]};
            vSol[0] = LI[0] * b[0] + LI[1] * b[1] + LI[2] * b[2];
            vSol[1] = LI[3] * b[0] + LI[4] * b[1] + LI[5] * b[2];
            vSol[2] = LI[6] * b[0] + LI[7] * b[1] + LI[8] * b[2];
            Fo[0] = A[0] * rhoSol * vSol[0] + A[1] * rhoSol * vSol[1] + A[2] * rhoSol * vSol[2];
            real vLab[3] = {vSol[0] + vfr[0], vSol[1] + vfr[1], vSol[2] + vfr[2]};
            if (c.meshless_finite_mass) { vSol[0] = 0.; vSol[1] = 0.; vSol[2] = 0.; }
            Fo[2] = A[0] * (rhoSol * vLab[0] * vSol[0] + PSol) + A[1] * rhoSol * vLab[0] * vSol[1] + A[2] * rhoSol * vLab[0] * vSol[2];
            Fo[3] = A[0] * rhoSol * vLab[1] * vSol[0] + A[1] * (rhoSol * vLab[1] * vSol[1] + PSol) + A[2] * rhoSol * vLab[1] * vSol[2];
            Fo[4] = A[0] * rhoSol * vLab[2] * vSol[0] + A[1] * rhoSol * vLab[2] * vSol[1] + A[2] * (rhoSol * vLab[2] * vSol[2] + PSol);
            Fo[1] = A[0] * (vSol[0] * (PSol / (gamma - 1.) + rhoSol * .5 * dot(vLab, vLab)) + PSol * vLab[0])
                  + A[1] * (vSol[1] * (PSol / (gamma - 1.) + rhoSol * .5 * dot(vLab, vLab)) + PSol * vLab[1])
                  + A[2] * (vSol[2] * (PSol / (gamma - 1.) + rhoSol * .5 * dot(vLab, vLab)) + PSol * vLab[2]);
        }
        return iters;
    }

    // --- Particles::solveRiemannProblems, Particles.cpp:1787-1911: the face is
    // solved from the side of the lower (parent) index; the other side copies
    // -F (ENFORCE_FLUX_SYM).
    // (Faces first, then the copies, so that the faces can be solved in any
    // order; the iteration list keeps the reference's face order.)
    void solveRiemannProblems() {
        const int NV = D + 2;
        F.assign((size_t)off[N] * NV, 0.);
        slotIters.assign(off[N], 0);
        orc::ExactRiemannT<real> rs(c.gamma, c.riemann_tol, c.riemann_max_iter);
#pragma omp parallel for schedule(dynamic, 256) num_threads(g_threads)
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s) {
                int j = (int)(nb[s] & IDX_MASK);
                real *R = &WR[(size_t)s * NV], *L = &WL[(size_t)s * NV];
                if (R[1] < 0. || L[1] < 0.) status |= ST_NEG_PRESSURE;
                if (j >= i) {
                    real wi[5], wj[5];
                    for (int d = 0; d < NV; ++d) { wi[d] = R[d]; wj[d] = L[d]; }
                    slotIters[s] = riemann(wi, wj, &vFrame[(size_t)s * 3], &Aij[(size_t)s * 3], &F[(size_t)s * NV], rs);
                }
            }
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s) {
                int j = (int)(nb[s] & IDX_MASK);
                if (j < i) {
                    int t = rev[s];
                    for (int d = 0; d < NV; ++d) F[(size_t)s * NV + d] = -F[(size_t)t * NV + d];
                    slotIters[s] = slotIters[t];
                }
            }
        newtonIters.clear();
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s)
                if ((int)(nb[s] & IDX_MASK) >= i) {
                    const int it = slotIters[s];
                    ++riemannSolves;
                    if (it >= 0) newtonTotal += it;
                    newtonIters.push_back(it);
                }
    }

    // --- Particles::collectFluxes, Particles.cpp:1913-2011
    void collectFluxes() {
        const int NV = D + 2;
        mF.assign(N, 0.); eF.assign(N, 0.); vF.assign((size_t)N * 3, 0.);
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s) {
                const real *f = &F[(size_t)s * NV];
                mF[i] += f[0];
                vF[(size_t)i * 3 + 0] += f[2];
                vF[(size_t)i * 3 + 1] += f[3];
                if (D == 3) vF[(size_t)i * 3 + 2] += f[4];
                eF[i] += f[1];
            }
    }

    // --- Particles::checkFluxSymmetry, Particles.cpp:2888-2976 (DEBUG_LVL >= 1,
    // called after solveRiemannProblems, MeshlessScheme.cpp:210-217): for every
    // interaction i -> j the reverse interaction is searched in j's list from
    // its start (real neighbours among the real ones, images among the
    // images), and F_ij + F_ji of every component is compared with
    // FLUX_SYM_TOL = 1e-20.  Returns the number of interactions that fail (the
    // reference logs them).
    long checkFluxSymmetry() const {
        const int NV = D + 2;
        const real tol = 1e-20;
        long bad = 0;
        for (int i = 0; i < N; ++i)
            for (int s = off[i]; s < off[i + 1]; ++s) {
                const int j = (int)(nb[s] & IDX_MASK);
                const bool isImg = (s - off[i]) >= noi[i];
                const int b = isImg ? off[j] + noi[j] : off[j];
                const int e = isImg ? off[j + 1] : off[j] + noi[j];
                int t = b;
                for (; t < e; ++t)
                    if ((int)(nb[t] & IDX_MASK) == i) break;
                if (t == e) { ++bad; continue; }
                bool notSym = false;
                for (int d = 0; d < NV; ++d)
                    if (F[(size_t)t * NV + d] + F[(size_t)s * NV + d] > tol) notSym = true;
                if (notSym) ++bad;
            }
        return bad;
    }

    // --- Particles::updateStateAndPosition, Particles.cpp:2013-2110
    void update() {
#pragma omp parallel for schedule(static) num_threads(g_threads)
        for (int i = 0; i < N; ++i) {
            real vxi = V[0][i], vyi = V[1][i], vzi = D == 3 ? V[2][i] : 0.;
            real Q[4];
            if (D == 3) Q[0] = m[i] * (u[i] + .5 * (vxi * vxi + vyi * vyi + vzi * vzi));
            else Q[0] = m[i] * (u[i] + .5 * (vxi * vxi + vyi * vyi));
            Q[1] = m[i] * vxi;
            Q[2] = m[i] * vyi;
            if (D == 3) Q[3] = m[i] * vzi;
            if (!c.meshless_finite_mass) m[i] -= dt * mF[i];
            if (m[i] <= 0.) status |= ST_NEG_MASS;
            for (int a = 0; a < D; ++a) {
                Q[1 + a] -= dt * vF[(size_t)i * 3 + a];
                V[a][i] = Q[1 + a] / m[i];
            }
            Q[0] -= dt * eF[i];
            if (D == 3) u[i] = Q[0] / m[i] - .5 * (V[0][i] * V[0][i] + V[1][i] * V[1][i] + V[2][i] * V[2][i]);
            else u[i] = Q[0] / m[i] - .5 * (V[0][i] * V[0][i] + V[1][i] * V[1][i]);
            if (u[i] <= 0.) status |= ST_NEG_ENERGY;
            if (c.move_particles) {
                real vo[3] = {vxi, vyi, vzi};
                for (int a = 0; a < D; ++a) X[a][i] += vo[a] * dt;
                if (c.periodic)
                    for (int a = 0; a < D; ++a) {
                        if (X[a][i] < lo[a]) X[a][i] = hi[a] - (lo[a] - X[a][i]);
                        else if (hi[a] <= X[a][i]) X[a][i] = lo[a] + (X[a][i] - hi[a]);
                    }
            }
        }
    }

    // --- Per-particle smoothing lengths (no reference counterpart).  For each
    // particle the support radius x in (0, h] at which the effective
    // neighbour number N(x) = V_D x^D (W(0, x) + sum_j W(r_ij, x)) equals
    // n_ngb (V_D the volume of the unit ball).  With the cubic spline of
    // support x, N(x) = K_D (1 + S(x)), S(x) = sum_j f(2 r_ij / x), f the
    // spline's shape (f(0) = 1) and K_D = 32/3 in 3D, 40/7 in 2D.  S is
    // increasing in x; dS/dx = G(x) / x with G = sum_j -f'(q) q.  Bracketed
    // Newton from the previous h_i (or h); the candidates are the particles
    // of the 3^D cell stencil within h (images by the ghost rule), in stencil
    // order; a particle with N(h) < n_ngb keeps h (counted as clamped).
    static void shape(real r, real ihh2, real &f, real &g) {
        real q = r * ihh2;
        if (q <= 1.) {
            real q2 = q * q;
            f = fma(q2, fma(0.75, q, -1.5), 1.);
            g = q2 * fma(-2.25, q, 3.);
        } else if (q < 2.) {
            real t = 2. - q, t2 = t * t;
            f = 0.25 * t2 * t;
            g = 0.75 * t2 * q;
        } else {
            f = 0.;
            g = 0.;
        }
    }

    void hsolve(real n_ngb) {
        const real KD = D == 3 ? 32. / 3. : 40. / 7.;
        const real St = n_ngb / KD - 1.;
        const real tolS = 1e-12 * St;
        const real hSqr = h * h;
        hp.resize(N, h);
        nEff.assign(N, 0.);
        long clampedSum = 0, itersSum = 0;
#pragma omp parallel for schedule(dynamic, 64) num_threads(g_threads) reduction(+ : clampedSum, itersSum)
        for (int i = 0; i < N; ++i) {
            std::vector<real> r;
            int ic = cellOf[i];
            int ix = ic % cells[0];
            int iy = (ic / cells[0]) % cells[1];
            int iz = D == 3 ? ic / (cells[0] * cells[1]) : 0;
            for (int k = ix - 1; k <= ix + 1; ++k)
                for (int l = iy - 1; l <= iy + 1; ++l)
                    for (int mm = (D == 3 ? iz - 1 : 0); mm <= (D == 3 ? iz + 1 : 0); ++mm) {
                        int cc[3] = {k, l, mm};
                        unsigned wrap = 0;
                        bool skip = false;
                        for (int a = 0; a < D; ++a)
                            if (cc[a] < 0 || cc[a] >= cells[a]) {
                                if (!c.periodic) { skip = true; break; }
                                cc[a] = cc[a] < 0 ? cc[a] + cells[a] : cc[a] - cells[a];
                                wrap |= 1u << a;
                            }
                        if (skip) continue;
                        int cell = cc[0] + cc[1] * cells[0] + (D == 3 ? cc[2] * cells[0] * cells[1] : 0);
                        for (int j : grid[cell]) {
                            if (!wrap && j == i) continue;
                            real xj[3];
                            bool ok = true;
                            for (int a = 0; a < D; ++a) {
                                xj[a] = X[a][j];
                                if (wrap & (1u << a)) ok = ok && image(a, X[a][j], xj[a]);
                            }
                            if (!ok) continue;
                            real dSqr = (xj[0] - X[0][i]) * (xj[0] - X[0][i]) + (xj[1] - X[1][i]) * (xj[1] - X[1][i]);
                            if (D == 3) dSqr += (xj[2] - X[2][i]) * (xj[2] - X[2][i]);
                            if (dSqr < hSqr) r.push_back(sqrt(dSqr));
                        }
                    }
            real x = hp[i];
            if (!(x > 0. && x <= h)) x = h;
            real lo_ = 0., hi_ = h, S = 0.;
            bool upper = false;
            for (int it = 0;; ++it) {
                // 32 strided partial sums, then pairwise at distance 16 .. 1
                real sf[32], sg[32];
                for (int l = 0; l < 32; ++l) { sf[l] = 0.; sg[l] = 0.; }
                const real ihh2 = 1. / (0.5 * x);
                for (size_t t = 0; t < r.size(); ++t) {
                    real f, g;
                    shape(r[t], ihh2, f, g);
                    sf[t % 32] += f;
                    sg[t % 32] += g;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    real tf[32], tg[32];
                    for (int l = 0; l < 32; ++l) { tf[l] = sf[l] + sf[l ^ o]; tg[l] = sg[l] + sg[l ^ o]; }
                    for (int l = 0; l < 32; ++l) { sf[l] = tf[l]; sg[l] = tg[l]; }
                }
                S = sf[0];
                const real G = sg[0];
                ++itersSum;
                const real F = S - St;
                if (fabs(F) <= tolS) break;
                if (F < 0. && x >= h) { ++clampedSum; break; }
                if (it + 1 >= 50) break;
                if (F > 0.) { hi_ = x; upper = true; }
                else lo_ = x;
                real xn = G > 0. ? x - F * x / G : 0.5 * (lo_ + hi_);
                if (!(xn > lo_ && xn < hi_)) xn = (!upper && xn >= hi_) ? h : 0.5 * (lo_ + hi_);
                if (xn == x) break;
                x = xn;
            }
            hp[i] = (double)x;
            nEff[i] = KD * (S + 1.);
        }
        hClamped = clampedSum;
        hIters = itersSum;
    }

    // grid of the current positions: the periodic box, or the bounding box
    void binning() {
        if (c.periodic) {
            for (int a = 0; a < D; ++a) { lo[a] = c.box_lo[a]; hi[a] = c.box_hi[a]; }
        } else {
            domainLimits();
        }
        createGrid();
        assign();
    }

    // operation counts per stage, summed over the steps (counting build)
#ifdef ORC_COUNT_FLOPS
    orc::FlopCounts stageFlops[ORC_NSTAGES] = {};
#endif
    template <typename F>
    void stage(int k, F run) {
#ifdef ORC_COUNT_FLOPS
        const orc::FlopCounts b = orc::flop_counts();
        run();
        const orc::FlopCounts &a = orc::flop_counts();
        orc::FlopCounts &t = stageFlops[k];
        t.add += a.add - b.add; t.mul += a.mul - b.mul; t.div += a.div - b.div;
        t.sqrt += a.sqrt - b.sqrt; t.pow += a.pow - b.pow; t.fma += a.fma - b.fma;
#else
        (void)k;
        run();
#endif
    }

    // DEBUG_LVL of the reference's build: >= 1 adds checkFluxSymmetry after
    // the Riemann solves (its count in fluxAsymmetric)
    int debugLvl = 0;
    long fluxAsymmetric = 0;

    // MeshlessScheme::run loop body, MeshlessScheme.cpp:39-253 (no dumps)
    int step() {
        status = 0;
        riemannSolves = 0; newtonTotal = 0;
        stage(ORC_STAGE_BINNING, [&] { binning(); });
        if (c.adaptive_h) stage(ORC_STAGE_HSOLVE, [&] { hsolve(c.n_ngb); });
        stage(ORC_STAGE_NNS, [&] { nns(); });
        stage(ORC_STAGE_DENSITY, [&] { density(); });
        stage(ORC_STAGE_PRESSURE, [&] { pressure(); });
        stage(ORC_STAGE_TIMESTEP, [&] { dt = c.adaptive_timestep ? (double)globalTimestep() : c.time_step; });
        stage(ORC_STAGE_PSI, [&] { psijTilde(); });
        stage(ORC_STAGE_GRADIENTS, [&] { gradients(); });
        if (c.slope_limiting) stage(ORC_STAGE_LIMITER, [&] { slopeLimiter(); });
        stage(ORC_STAGE_FACE, [&] { effectiveFace(); });
        stage(ORC_STAGE_STATES, [&] { riemannStatesLR(); });
        stage(ORC_STAGE_RIEMANN, [&] { solveRiemannProblems(); });
        if (debugLvl >= 1) fluxAsymmetric = checkFluxSymmetry();
        stage(ORC_STAGE_COLLECT, [&] { collectFluxes(); });
        stage(ORC_STAGE_UPDATE, [&] { update(); });
        return (int)status;
    }
};

struct Handle {
    int dim;
    void *sim;
};

template <int D>
Sim<D> *make(const orc_config *cfg, int n, const double *x, const double *y, const double *z,
             const double *vx, const double *vy, const double *vz, const double *m, const double *u) {
    Sim<D> *s = new Sim<D>();
    s->c = *cfg;
    s->N = n;
    s->h = cfg->kernel_size;
    s->hp.assign(n, cfg->kernel_size);
    const double *xs[3] = {x, y, z}, *vs[3] = {vx, vy, vz};
    for (int a = 0; a < 3; ++a) {
        s->X[a].assign(n, 0.);
        s->V[a].assign(n, 0.);
        if (a < D) {
            std::copy(xs[a], xs[a] + n, s->X[a].begin());
            std::copy(vs[a], vs[a] + n, s->V[a].begin());
        }
    }
    s->m.assign(m, m + n);
    s->u.assign(u, u + n);
    s->rho.assign(n, 0.);
    s->P.assign(n, 0.);
    return s;
}

template <int D>
long sizeOf(Sim<D> *s, const std::string &nm) {
    long N = s->N, S = s->off.empty() ? 0 : s->off[N];
    if (nm == "x" || nm == "y" || nm == "z" || nm == "vx" || nm == "vy" || nm == "vz" || nm == "m" || nm == "u" ||
        nm == "rho" || nm == "P" || nm == "omega" || nm == "noi" || nm == "noi_img" || nm == "mF" || nm == "eF" ||
        nm == "h" || nm == "n_eff")
        return N;
    if (nm == "off") return N + 1;
    if (nm == "nnl" || nm == "rev" || nm == "slot_iters") return S;
    if (nm == "vF") return N * 3;
    if (nm.compare(0, 4, "grad") == 0) return N * 3;
    if (nm == "B") return N * D * D;
    if (nm == "psi" || nm == "Aij" || nm == "vFrame") return S * 3;
    if (nm == "WL" || nm == "WR" || nm == "F") return S * (D + 2);
    if (nm == "dt" || nm == "grid" || nm == "stats") return nm == "grid" ? 9 : (nm == "stats" ? 2 : 1);
    if (nm == "newton_iters") return (long)s->newtonIters.size();
    return -1;
}

template <int D>
int getArr(Sim<D> *s, const std::string &nm, void *out) {
    double *o = (double *)out;
    int *oi = (int *)out;
    auto cp = [&](const auto &v) { for (size_t k = 0; k < v.size(); ++k) o[k] = (double)v[k]; return 0; };
    auto cpi = [&](const std::vector<int> &v) { std::copy(v.begin(), v.end(), oi); return 0; };
    if (nm == "x") return cp(s->X[0]);
    if (nm == "y") return cp(s->X[1]);
    if (nm == "z") return cp(s->X[2]);
    if (nm == "vx") return cp(s->V[0]);
    if (nm == "vy") return cp(s->V[1]);
    if (nm == "vz") return cp(s->V[2]);
    if (nm == "m") return cp(s->m);
    if (nm == "u") return cp(s->u);
    if (nm == "rho") return cp(s->rho);
    if (nm == "P") return cp(s->P);
    if (nm == "omega") return cp(s->omega);
    if (nm == "h") return cp(s->hp);
    if (nm == "n_eff") { if (s->nEff.size() != (size_t)s->N) return -1; return cp(s->nEff); }
    if (nm == "mF") return cp(s->mF);
    if (nm == "eF") return cp(s->eF);
    if (nm == "vF") return cp(s->vF);
    if (nm == "B") return cp(s->B);
    if (nm == "psi") return cp(s->psi);
    if (nm == "Aij") return cp(s->Aij);
    if (nm == "vFrame") return cp(s->vFrame);
    if (nm == "WL") return cp(s->WL);
    if (nm == "WR") return cp(s->WR);
    if (nm == "F") return cp(s->F);
    if (nm == "noi") return cpi(s->noi);
    if (nm == "noi_img") return cpi(s->noiImg);
    if (nm == "off") return cpi(s->off);
    if (nm == "rev") return cpi(s->rev);
    if (nm == "newton_iters") return cpi(s->newtonIters);
    if (nm == "slot_iters") { if (s->slotIters.size() != s->nb.size()) return -1; return cpi(s->slotIters); }
    if (nm == "nnl") { std::copy(s->nb.begin(), s->nb.end(), (uint32_t *)out); return 0; }
    if (nm == "dt") { o[0] = s->dt; return 0; }
    if (nm == "stats") { o[0] = (double)s->riemannSolves; o[1] = (double)s->newtonTotal; return 0; }
    if (nm == "grid") {
        for (int a = 0; a < 3; ++a) {
            o[a] = a < D ? (double)s->lo[a] : 0.;
            o[3 + a] = a < D ? (double)s->hi[a] : 0.;
            o[6 + a] = a < D ? s->cells[a] : 0;
        }
        return 0;
    }
    // gradients: "grad_<f>" limited, "gradraw_<f>" unlimited; f in
    // rho, vx, vy, vz, P
    static const char *names[5] = {"rho", "vx", "vy", "vz", "P"};
    for (int k = 0; k < 5; ++k) {
        int f = k;
        if (D == 2) { if (k == 3) continue; if (k == 4) f = 3; }
        if (nm == std::string("grad_") + names[k]) return cp(s->G[f]);
        if (nm == std::string("gradraw_") + names[k]) return cp(s->Graw[f]);
    }
    return -1;
}

template <int D>
long smoothing(Sim<D> *s, double n_ngb, double *h_out, double *neff_out) {
    s->status = 0;
    s->binning();
    s->hsolve(n_ngb);
    if (h_out) std::copy(s->hp.begin(), s->hp.end(), h_out);
    if (neff_out) for (int k = 0; k < s->N; ++k) neff_out[k] = (double)s->nEff[k];
    return s->hClamped;
}

// Riemann::Riemann + Riemann::exact for independent faces (the step's
// riemann() on a simulation without particles).
template <int D>
int riemannFaces(int n, const double *Wi, const double *Wj, const double *vFrame, const double *Aij, double gamma,
                 int mfm, double *F, int *iters) {
    orc_config cfg;
    std::memset(&cfg, 0, sizeof(cfg));
    cfg.dim = D;
    cfg.gamma = gamma;
    cfg.meshless_finite_mass = mfm;
    cfg.riemann_tol = 1e-10;
    cfg.riemann_max_iter = 100;
    Sim<D> s;
    s.c = cfg;
    s.N = 0;
    orc::ExactRiemannT<real> rs(gamma, cfg.riemann_tol, cfg.riemann_max_iter);
    const int NV = D + 2;
    for (int f = 0; f < n; ++f) {
        real wi[5], wj[5], vf[3], A[3], Fo[5];
        for (int k = 0; k < NV; ++k) { wi[k] = Wi[(size_t)f * NV + k]; wj[k] = Wj[(size_t)f * NV + k]; }
        for (int k = 0; k < D; ++k) { vf[k] = vFrame[(size_t)f * D + k]; A[k] = Aij[(size_t)f * D + k]; }
        if (wi[1] < 0. || wj[1] < 0.) s.status |= ST_NEG_PRESSURE;
        const int it = s.riemann(wi, wj, vf, A, Fo, rs);
        for (int k = 0; k < NV; ++k) F[(size_t)f * NV + k] = (double)Fo[k];
        if (iters) iters[f] = it;
    }
    return (int)s.status;
}

}  // namespace

extern "C" {

void *orc_create(const orc_config *cfg, int n, const double *x, const double *y, const double *z,
                 const double *vx, const double *vy, const double *vz, const double *m, const double *u) {
    Handle *hnd = new Handle();
    hnd->dim = cfg->dim;
    if (cfg->dim == 2) hnd->sim = make<2>(cfg, n, x, y, z, vx, vy, vz, m, u);
    else hnd->sim = make<3>(cfg, n, x, y, z, vx, vy, vz, m, u);
    return hnd;
}

int orc_step(void *ctx) {
    Handle *hnd = (Handle *)ctx;
    if (hnd->dim == 2) return ((Sim<2> *)hnd->sim)->step();
    return ((Sim<3> *)hnd->sim)->step();
}

long orc_size(void *ctx, const char *name) {
    Handle *hnd = (Handle *)ctx;
    if (hnd->dim == 2) return sizeOf((Sim<2> *)hnd->sim, name);
    return sizeOf((Sim<3> *)hnd->sim, name);
}

int orc_get(void *ctx, const char *name, void *out) {
    Handle *hnd = (Handle *)ctx;
    if (hnd->dim == 2) return getArr((Sim<2> *)hnd->sim, name, out);
    return getArr((Sim<3> *)hnd->sim, name, out);
}

// Exact Riemann solves of n independent states: star pressure and Newton
// iterations, from the two-rarefaction guess or from guess[k] when given
// (for checking learned initial guesses).
int orc_riemann_batch(int n, const double *rhoL, const double *uL, const double *pL, const double *rhoR,
                      const double *uR, const double *pR, double gamma, const double *guess, double *pstar,
                      int *iters) {
    orc::ExactRiemann rs(gamma, 1e-10, 100);
    for (int k = 0; k < n; ++k) {
        double cL = std::sqrt(gamma * pL[k] / rhoL[k]), cR = std::sqrt(gamma * pR[k] / rhoR[k]);
        double p0 = guess ? guess[k] : rs.guess_two_rarefaction(uL[k], pL[k], cL, uR[k], pR[k], cR);
        double ps = 0.;
        int it = rs.newton(p0, rhoL[k], uL[k], pL[k], cL, rhoR[k], uR[k], pR[k], cR, ps);
        pstar[k] = ps;
        if (iters) iters[k] = it;
    }
    return 0;
}

long orc_smoothing_lengths(void *ctx, double n_ngb, double *h_out, double *neff_out) {
    Handle *hnd = (Handle *)ctx;
    if (hnd->dim == 2) return smoothing((Sim<2> *)hnd->sim, n_ngb, h_out, neff_out);
    return smoothing((Sim<3> *)hnd->sim, n_ngb, h_out, neff_out);
}

int orc_riemann_fluxes(int dim, int n, const double *Wi, const double *Wj, const double *vFrame, const double *Aij,
                       double gamma, int mfm, double *F, int *iters) {
    if (dim == 2) return riemannFaces<2>(n, Wi, Wj, vFrame, Aij, gamma, mfm, F, iters);
    return riemannFaces<3>(n, Wi, Wj, vFrame, Aij, gamma, mfm, F, iters);
}

int orc_set_debug_level(void *ctx, int lvl) {
    Handle *hnd = (Handle *)ctx;
    if (hnd->dim == 2) ((Sim<2> *)hnd->sim)->debugLvl = lvl;
    else ((Sim<3> *)hnd->sim)->debugLvl = lvl;
    return 0;
}

long orc_flux_asymmetric(void *ctx) {
    Handle *hnd = (Handle *)ctx;
    if (hnd->dim == 2) return ((Sim<2> *)hnd->sim)->fluxAsymmetric;
    return ((Sim<3> *)hnd->sim)->fluxAsymmetric;
}

int orc_set_threads(int n) {
#ifdef _OPENMP
    if (n < 1) n = omp_get_num_procs();
    g_threads = n;
    return n;
#else
    (void)n;
    return 1;
#endif
}

int orc_flop_counts(void *ctx, unsigned long long *out) {
#ifdef ORC_COUNT_FLOPS
    Handle *hnd = (Handle *)ctx;
    const orc::FlopCounts *t = hnd->dim == 2 ? ((Sim<2> *)hnd->sim)->stageFlops : ((Sim<3> *)hnd->sim)->stageFlops;
    for (int k = 0; k < ORC_NSTAGES; ++k) {
        const unsigned long long v[6] = {t[k].add, t[k].mul, t[k].div, t[k].sqrt, t[k].pow, t[k].fma};
        for (int q = 0; q < 6; ++q) out[6 * k + q] = v[q];
    }
    return ORC_NSTAGES;
#else
    (void)ctx; (void)out;
    return -1;
#endif
}

void orc_destroy(void *ctx) {
    Handle *hnd = (Handle *)ctx;
    if (hnd->dim == 2) delete (Sim<2> *)hnd->sim;
    else delete (Sim<3> *)hnd->sim;
    delete hnd;
}

}  // extern "C"
