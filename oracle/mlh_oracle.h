/* TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * C interface of the CPU restatement of the reference's MFV timestep
 * (jammartin/meshlessHydro, demonstrator/src/MeshlessScheme.cpp:39-253 and the
 * Particles stage methods it calls).  Only tests/, the smoke check and
 * bench.py's CPU baseline load this library, to compare against.
 */
#ifndef MLH_ORACLE_H
#define MLH_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* Same field meaning as mlh_config in include/mlh.h (the compile-time
 * switches of demonstrator/include/parameter.h:9-74 and the config.info keys
 * of demonstrator/config.info:1-33), declared separately so that the oracle
 * and the product share no code. */
typedef struct orc_config {
    int dim;
    int periodic;
    int adaptive_timestep;
    int slope_limiting;
    int pairwise_limiter;
    int meshless_finite_mass;
    int move_particles;
    int first_order_quad_point;
    int int_abs;
    int image_pairwise_limiter;
    int riemann_max_iter;
    int max_neighbours;
    double box_lo[3];
    double box_hi[3];
    double kernel_size;
    double gamma;
    double cfl;
    double time_step;
    double beta;
    double psi1;
    double psi2;
    double riemann_tol;
    double n_ngb;       /* target effective neighbour number of the h solve */
    int adaptive_h;     /* per-particle smoothing lengths in the step */
} orc_config;

void *orc_create(const orc_config *cfg, int n,
                 const double *x, const double *y, const double *z,
                 const double *vx, const double *vy, const double *vz,
                 const double *m, const double *u);
/* One MFV step.  Returns 0, or a nonzero status (see the .cpp). */
int orc_step(void *ctx);
/* Number of elements of a named array (after the last step), -1 if unknown. */
long orc_size(void *ctx, const char *name);
/* Copy a named array into `out` (doubles, or int32 for integer arrays). */
int orc_get(void *ctx, const char *name, void *out);
void orc_destroy(void *ctx);
/* Riemann::Riemann + Riemann::exact of n independent faces: Wi (left, particle
 * i) and Wj (right) [rho, P, v..] (dim + 2 each), vFrame, Aij (dim each); F
 * (dim + 2: mass, energy, momentum), iters (may be NULL). */
int orc_riemann_fluxes(int dim, int n, const double *Wi, const double *Wj, const double *vFrame, const double *Aij,
                       double gamma, int mfm, double *F, int *iters);
/* Per-particle smoothing lengths on the current positions (see the .cpp):
 * h_out, neff_out: n doubles each (may be NULL).  Returns the number of
 * particles clamped at kernel_size. */
long orc_smoothing_lengths(void *ctx, double n_ngb, double *h_out, double *neff_out);
int orc_riemann_batch(int n, const double *rhoL, const double *uL, const double *pL, const double *rhoR,
                      const double *uR, const double *pR, double gamma, const double *guess, double *pstar,
                      int *iters);

/* Stages of one step, in the reference's order (MeshlessScheme.cpp:39-253). */
enum {
    ORC_STAGE_BINNING = 0,   /* domain limits, grid, cell assignment */
    ORC_STAGE_HSOLVE,        /* per-particle smoothing lengths (adaptive_h) */
    ORC_STAGE_NNS,           /* gridNNS + ghostNNS */
    ORC_STAGE_DENSITY,       /* compDensity (omega, rho) */
    ORC_STAGE_PRESSURE,      /* compPressure */
    ORC_STAGE_TIMESTEP,      /* compGlobalTimestep */
    ORC_STAGE_PSI,           /* compPsijTilde */
    ORC_STAGE_GRADIENTS,     /* gradient x (dim + 2) */
    ORC_STAGE_LIMITER,       /* slopeLimiter */
    ORC_STAGE_FACE,          /* compEffectiveFace */
    ORC_STAGE_STATES,        /* compRiemannStatesLR + pairwiseLimiter */
    ORC_STAGE_RIEMANN,       /* solveRiemannProblems (Riemann::exact) */
    ORC_STAGE_COLLECT,       /* collectFluxes */
    ORC_STAGE_UPDATE,        /* updateStateAndPosition */
    ORC_NSTAGES
};

/* DEBUG_LVL of the reference's build (0 or 1): 1 adds the reference's
 * checkFluxSymmetry after the Riemann solves of every step
 * (demonstrator/src/MeshlessScheme.cpp:210-217, Particles.cpp:2888-2976);
 * orc_flux_asymmetric gives the count of interactions it found asymmetric
 * in the last step. */
int orc_set_debug_level(void *ctx, int lvl);
long orc_flux_asymmetric(void *ctx);

/* Threads of the per-particle loops (results do not depend on them); n < 1:
 * one per processor.  Returns the count in effect (1 in a build without
 * OpenMP).  The default is 1: the serial restatement of the reference. */
int orc_set_threads(int n);

/* Operation-counting build only (liborc_count.so, -DORC_COUNT_FLOPS):
 * operation counts of each stage summed over the steps of this context,
 * out[6 * stage + k] for k = add, mul, div, sqrt, pow, fma.  Returns
 * ORC_NSTAGES, or -1 in the plain build. */
int orc_flop_counts(void *ctx, unsigned long long *out);

#ifdef __cplusplus
}
#endif
#endif
