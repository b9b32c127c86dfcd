// Device-side definitions shared by the MFV kernels (sm_103a).
//
// Physics and arithmetic follow the reference demonstrator
// (jammartin/meshlessHydro, demonstrator/src/Particles.cpp, Riemann.cpp,
// Helper.cpp); each function cites the lines it restates.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mlh {

constexpr unsigned IMG_SHIFT = 29;
constexpr unsigned IDX_MASK = (1u << IMG_SHIFT) - 1u;
constexpr double DBL_MIN_ = 2.2250738585072014e-308;   // numeric_limits<double>::min()
constexpr double DBL_MAX_ = 1.7976931348623157e+308;   // numeric_limits<double>::max()
constexpr float FLT_MAX_ = 3.40282347e+38f;
constexpr float FLT_INF_ = __builtin_huge_valf();

// status bits (mirror MLH_ERR_* of include/mlh.h)
enum : unsigned {
    ST_NGB_OVERFLOW = 1u << 0,
    ST_NEG_PRESSURE = 1u << 1,
    ST_NEG_DENSITY = 1u << 2,
    ST_NEG_MASS = 1u << 3,
    ST_NEG_ENERGY = 1u << 4,
    ST_NEWTON = 1u << 5,
    ST_VACUUM = 1u << 6,
    ST_GRID = 1u << 7,
    ST_NO_NEIGHBOUR = 1u << 8,
    ST_ASYMMETRIC = 1u << 9,
    ST_NAN = 1u << 10,
    ST_TIMEOUT = 1u << 11,
    ST_CAPACITY = 1u << 23,   // a fixed-size device buffer was too small
};

// Uniform search grid of one simulation (Domain::createGrid,
// demonstrator/src/Domain.cpp:9-54); its cells are numbered from cell_base in
// the concatenated cell array of all simulations of a context.
struct GridInfo {
    double lo[3], hi[3], cs[3];
    // ghost bands of the periodic box: a coordinate x has an image when
    // x <= band_lo = lo + h or band_hi = hi - h < x (Particles.cpp:2123-2142)
    double band_lo[3], band_hi[3];
    float Lf[3];           // box lengths hi - lo in single precision (pre-filter)
    int cells[3];
    int ncells;
    int cell_base;
};

// One simulation of a context (a context holds one, or an ensemble of
// independent simulations stored back to back): its kernel size and the
// quantities derived from it, its periodic box and its particle range.
struct Member {
    double h, hsq, h2, ih2, sigma, w0, cfl_h;
    double box_lo[3], box_hi[3];
    float hsq_f;           // conservative single-precision bound for the pre-filter
    int first, count;
};

// Everything a kernel needs to know about the run, passed by value.
struct Params {
    int n, dim, periodic, adaptive, slope, pairwise, mfm, move, foqp, int_abs, img_pw, rmaxit;
    int K;                 // neighbour slots per particle
    int ncells_cap;
    int faces_cap;         // capacity of the face arrays
    double h, hsq, h2, sigma, w0, gamma, cfl_h, beta, psi1, psi2, rtol, time_step;
    double box_lo[3], box_hi[3];
    float hsq_f;           // conservative single-precision bound for the pre-filter
    // per-particle smoothing lengths (adaptive_h): the step's support radius
    // of particle i is hp[i] <= the member's kernelSize, which stays the
    // search radius (grid cells, periodic-image band)
    int adaptive_h;
    double cfl;            // CFL (cfl_h = CFL * kernelSize without adaptive_h)
    int face_split;        // faces unfinished after one Newton step go to a second pass
    double sngb_t;         // target of S = sum_j f(2 r_ij / h_i): n_ngb / K_D - 1
    const double *hp;
    const float *hpf;      // hp rounded up to single precision (pre-filter)
};

// Per-particle records (array of structures: one particle's values sit in
// one or two 64-byte sectors for the random-access neighbour loops).
struct Prim {       // positions, primitive state of this step
    double x, y, z, rho, vx, vy, vz, P;
};
struct Grad {       // limited gradients: rho, vx, vy, vz, P (x,y,z each), div v
    double g[16];
    // particle part of the half-step prediction of each field, in the order
    // rho, P, vx, vy, vz: rho div v + v.grad rho, gamma P div v + v.grad P,
    // (grad P)_a / rho + v.grad v_a (the face subtracts v_frame.grad f)
    double t[8];
};
struct Geo {        // E_i^{-1}, 1/omega_i, omega_i, sound speed, 1/rho_i
    double B[9];
    double V, omega, c, irho;
};
struct FaceRef {    // canonical face: owner i, slot index, reverse slot (images)
    int i, slot, rslot, pad;
};
// Face-frame state of one deferred face between the two passes of the
// learned-guess face pipeline: R[5], L[5], A[3], v_frame[3], A/|A| [3], p_TR
struct FaceState {
    double v[20];
};
// A queue of faces for a second face pass: their face-frame states, face ids
// and the number of faces offered (entries at or beyond cap were not stored).
struct FaceQueue {
    FaceState *st;
    int *face;
    int *count;
    int cap;
};
// Where the plain face kernel records network training pairs.
struct Harvest {
    float4 *x;
    float *t;
    int *count;
    int stride, cap;
    int strong;   // record the strong shocks only (compacted), not every stride-th face
};

// Kernel::cubicSpline, demonstrator/src/Particles.cpp:7-24, for a support
// radius h: ih2 = 2 / h and sigma computed with the reference's expression
// (kernel_sigma); q = r / (h/2) is taken as r * (2/h) (within an ulp of the
// quotient) and pow(2-q, 3.) is written as a product.  The two pieces run as
// the same five operations with selected operands, so that a warp whose
// lanes fall on both sides of q = 1 issues them once:
//   q <= 1:     sigma   * fma(-(1.5 q) q, t, 1),  t = fma(-0.5, q, 1) = 1 - q/2
//   1 < q < 2:  sigma/4 * fma((t t) t, 1, 0),     t = fma(-1, q, 2) = 2 - q
// (fma(z, 1, 0) = z for z >= 0, and sigma/4 is exact), each the value of the
// reference's expression for its piece.  sigma4 = sigma / 4 is passed in
// (computed once per particle, not per neighbour).
__device__ __forceinline__ double kernelW2(double r, double ih2, double sigma, double sigma4) {
    // r >= 0, so q >= 0 and the range tests compare bit patterns (integer
    // pipe): q <= 1 and q < 2
    const double q = __dmul_rn(r, ih2);
    const long long qb = __double_as_longlong(q);
    const bool inner = qb <= 0x3FF0000000000000ll;
    const double t = __fma_rn(inner ? -0.5 : -1., q, inner ? 1. : 2.);
    const double y = __dmul_rn(inner ? 1.5 : t, inner ? q : t);
    const double z = __dmul_rn(y, inner ? q : t);
    const double zs = __longlong_as_double(__double_as_longlong(z) ^ (inner ? (long long)0x8000000000000000ull : 0ll));
    const double w = __fma_rn(zs, inner ? t : 1., inner ? 1. : 0.);
    const double W = __dmul_rn(inner ? sigma : sigma4, w);
    return qb < 0x4000000000000000ll ? W : 0.;
}
// Particles.cpp:10-15 (the value of the kernel at r = 0 is sigma)
template <int D>
__device__ __forceinline__ double kernel_sigma(double h2) {
    constexpr double PI = 3.14159265358979323846;
    return D == 2 ? 10. / (7. * PI * h2 * h2) : 1. / (PI * h2 * h2 * h2);
}

// abs() as bound by the reference's limiter code (fabs, or int abs(int) with
// x86 conversion semantics: NaN / out of range -> INT_MIN, abs(INT_MIN) = INT_MIN).
__device__ __forceinline__ double ref_abs(double x, int int_abs) {
    if (!int_abs) return fabs(x);
    if (!(x > -2147483649.0 && x < 2147483648.0)) return -2147483648.0;
    int t = (int)x;
    if (t == (int)0x80000000) return -2147483648.0;
    return (double)(t < 0 ? -t : t);
}

// Order-preserving integer keys of doubles.  On GB300 an FP64 compare or
// min/max occupies the scarce FP64 pipe like an FMA; comparing these keys on
// the integer pipe instead gives the same answer for non-NaN operands:
// ord_key(a) < ord_key(b) exactly when a < b, with -0 and +0 on the same key
// 0 (so ord_key(x) >= 0 exactly when x >= 0).  The map is its own inverse on
// keys (key_double), except that -0 comes back as +0.
__device__ __forceinline__ long long ord_key(double x) {
    const long long s = __double_as_longlong(x);
    return s >= 0 ? s : (long long)(0x8000000000000000ull - (unsigned long long)s);
}
__device__ __forceinline__ double key_double(long long k) {
    return __longlong_as_double(k >= 0 ? k : (long long)(0x8000000000000000ull - (unsigned long long)k));
}
__device__ __forceinline__ bool dlt(double a, double b) { return ord_key(a) < ord_key(b); }

// x * 2^-K (K = 1, 2) on the integer pipe, the IEEE product bit for bit: a
// normal result takes K off the exponent; a subnormal one is the significand
// (with its implicit bit) shifted right and rounded to nearest even; zero,
// infinity and NaN stay as they are.  (A DMUL by 0.5 occupies the scarce FP64
// pipe like an FMA.)  Straight-line selects, no branches: a branch would
// split the caller's basic blocks and with them the compiler's fusing of
// neighbouring multiplies and adds, which then could differ between the
// kernels that inline the same code.
template <int K>
__device__ __forceinline__ double scale_down(double x) {
    static_assert(K == 1 || K == 2, "scale_down: K = 1 or 2");
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long sign = b & 0x8000000000000000ull, mag = b ^ sign;
    const unsigned long long E = mag >> 52;
    const unsigned long long rn = mag - ((unsigned long long)K << 52);   // normal result (E > K)
    // subnormal result (E <= K): shift 1..K, kept in range on the other paths
    const unsigned long long sig = E ? ((mag & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull) : mag;
    const unsigned sh0 = (unsigned)K - (E ? (unsigned)E - 1u : 0u);
    const unsigned sh = E <= (unsigned long long)K ? sh0 : 1u;
    const unsigned long long q = sig >> sh, rem = sig & ((1ull << sh) - 1ull), hv = 1ull << (sh - 1u);
    const unsigned long long rs = q + (unsigned long long)((rem > hv) | ((rem == hv) & ((q & 1ull) != 0)));
    unsigned long long r = E > (unsigned long long)K ? rn : rs;
    r = E == 0x7FFull ? mag : r;
    return __longlong_as_double((long long)(r | sign));
}
__device__ __forceinline__ double half_of(double x) { return scale_down<1>(x); }
// 2 x on the integer pipe, the IEEE product bit for bit (overflow to
// infinity); straight-line selects as in scale_down
__device__ __forceinline__ double twice(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long sign = b & 0x8000000000000000ull, mag = b ^ sign;
    unsigned long long r = mag < 0x0010000000000000ull ? mag << 1 : mag + 0x0010000000000000ull;
    r = mag >= 0x7FE0000000000000ull ? 0x7FF0000000000000ull : r;   // overflow
    r = mag >= 0x7FF0000000000000ull ? mag : r;                      // infinity, NaN
    return __longlong_as_double((long long)(r | sign));
}
__device__ __forceinline__ bool dneg(double x) { return ord_key(x) < 0; }   // x < 0

// Ghost image coordinate, Particles.cpp:2123-2142: a coordinate in the
// lower band (x <= lo + h) is mirrored to hi + (x - lo), one in the upper
// band (hi - h < x) to lo - (hi - x) = lo + (x - hi) (the same double: RN
// rounding is symmetric).  The band limits are precomputed in GridInfo and
// compared as order-preserving integer keys (ord_key), so neither
// test nor mirror takes FP64 compares; the mirror is two additions with
// selected operands.
__device__ __forceinline__ bool in_band(double xa, const GridInfo &g, int a) {
    const long long k = ord_key(xa);
    return k <= ord_key(g.band_lo[a]) || ord_key(g.band_hi[a]) < k;
}
__device__ __forceinline__ double image_coord(double xa, const GridInfo &g, int a) {
    const bool low = ord_key(xa) <= ord_key(g.band_lo[a]);
    return __dadd_rn(low ? g.hi[a] : g.lo[a], __dsub_rn(xa, low ? g.lo[a] : g.hi[a]));
}

// Reciprocal and reciprocal square root from the hardware estimates of PTX
// rcp.approx.ftz.f64 / rsqrt.approx.ftz.f64 (relative error e of the estimate
// a few times 2^-23), each refined by one third-order step:
//   1/x       = r (1 - e)^-1   = r (1 + e + e^2 + ...),         e = 1 - x r
//   1/sqrt(x) = y (1 - e)^-1/2 = y (1 + e/2 + 3 e^2/8 + ...),   e = 1 - x y^2
// whose dropped terms (e^3, 5 e^3 / 16) are below 2^-60: the result is within
// about an ulp of the correctly rounded one (the probe mlh_probe_fast_math
// measures it against exact values).  Three and five FP64 operations in a
// dependent chain of the same length, against four and six for two
// Newton-Raphson steps: these sit on the Riemann iteration's dependency
// chain, and the face pass waits on that chain as well as on the pipe.
// Cheaper on the FP64 pipe than IEEE division, which also guards subnormal,
// zero and infinite operands: these are for normal, finite, nonzero operands
// only.
__device__ __forceinline__ double frcp(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double e = fma(-x, r, 1.);
    return fma(r, fma(e, e, e), r);
}
__device__ __forceinline__ double fdiv(double a, double b) { return a * frcp(b); }
__device__ __forceinline__ double frsqrt(double x) {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-(x * y), y, 1.);
    return fma(y, e * fma(0.375, e, 0.5), y);
}

template <int D>
__device__ __forceinline__ double dotD(const double *a, const double *b) {
    double r = 0.;
#pragma unroll
    for (int k = 0; k < D; ++k) r += a[k] * b[k];
    return r;
}

// base + a . b as one chain of fused multiply-adds starting from base
template <int D>
__device__ __forceinline__ double fma_dotD(const double *a, const double *b, double base) {
    double r = base;
#pragma unroll
    for (int k = 0; k < D; ++k) r = fma(a[k], b[k], r);
    return r;
}

__device__ __forceinline__ void flag(unsigned *status, unsigned bits) {
    atomicOr(status, bits);
}

}  // namespace mlh
