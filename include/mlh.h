/*
 * meshlesshydro-gb300: C ABI of the GB300 (sm_103a) MFV timestep.
 *
 * This is the boundary that replaces the body of one step of the reference's
 * MeshlessScheme::run (jammartin/meshlessHydro, demonstrator/src/
 * MeshlessScheme.cpp:39-253) and the Particles stage methods it calls.  All
 * functions take plain pointers and sizes, return an int status (0 = OK,
 * otherwise MLH_ERR_* bits), and never exit().  One context owns the device
 * memory and one CUDA stream; calls on one context must be serialised.
 */
#ifndef MLH_H
#define MLH_H

#ifdef __cplusplus
extern "C" {
#endif

#define MLH_ABI_VERSION 4

/* Status bits.  The reference exits instead (demonstrator/src/Particles.cpp:
 * 348-352 exit(1) neighbour overflow, :2249-2253 exit(3), :1878-1881 exit(6)
 * negative ghost-face pressure) or only warns. */
enum mlh_status_bits {
    MLH_OK = 0,
    MLH_ERR_NGB_OVERFLOW = 1 << 0,   /* a particle has more neighbours than slots */
    MLH_ERR_NEG_PRESSURE = 1 << 1,   /* P <= 0 or a face state with P < 0 */
    MLH_ERR_NEG_DENSITY = 1 << 2,
    MLH_ERR_NEG_MASS = 1 << 3,
    MLH_ERR_NEG_ENERGY = 1 << 4,
    MLH_ERR_NEWTON = 1 << 5,         /* Riemann Newton iteration did not converge */
    MLH_ERR_VACUUM = 1 << 6,         /* vacuum generated in a Riemann problem */
    MLH_ERR_GRID = 1 << 7,           /* particle outside the grid / < 3 periodic cells */
    MLH_ERR_NO_NEIGHBOUR = 1 << 8,
    MLH_ERR_ASYMMETRIC = 1 << 9,     /* a neighbour pair found from one side only */
    MLH_ERR_NAN = 1 << 10,
    MLH_ERR_TIMEOUT = 1 << 11,       /* a bounded device wait gave up */
    MLH_ERR_INVALID = 1 << 20,       /* bad argument */
    MLH_ERR_CUDA = 1 << 21,          /* CUDA runtime error (message: mlh_last_error) */
    MLH_ERR_NO_DEVICE = 1 << 22,
    MLH_ERR_CAPACITY = 1 << 23       /* a size above a fixed maximum */
};

/* Run-time form of the reference's settings: the compile-time switches of
 * demonstrator/include/parameter.h:9-74 and the config.info keys read in
 * demonstrator/src/main.cpp:55-85. */
typedef struct mlh_config {
    int dim;                    /* DIM: 2 or 3 */
    int periodic;               /* PERIODIC_BOUNDARIES */
    int adaptive_timestep;      /* ADAPTIVE_TIMESTEP */
    int slope_limiting;         /* SLOPE_LIMITING */
    int pairwise_limiter;       /* PAIRWISE_LIMITER */
    int meshless_finite_mass;   /* MESHLESS_FINITE_MASS */
    int move_particles;         /* MOVE_PARTICLES */
    int first_order_quad_point; /* FIRST_ORDER_QUAD_POINT */
    int int_abs;                /* limiters use int abs(int), the binding of the reference's unqualified
                                   abs(double) when no <math.h>/<stdlib.h> is seen */
    int image_pairwise_limiter; /* pairwise limiter also on periodic-image faces */
    int riemann_max_iter;       /* Newton iteration cap */
    int max_neighbours;         /* slots per particle; 0 = automatic */
    double box_lo[3];           /* periodicBoxLimits lowerX/Y/Z */
    double box_hi[3];           /* periodicBoxLimits upperX/Y/Z */
    double kernel_size;         /* kernelSize (support radius h) */
    double gamma;               /* gamma */
    double cfl;                 /* CFL */
    double time_step;           /* timeStep: dt when !adaptive_timestep */
    double beta;                /* BETA */
    double psi1;                /* PSI_1 */
    double psi2;                /* PSI_2 */
    double riemann_tol;         /* relative Newton tolerance on p* */
    /* Per-particle smoothing lengths (no counterpart in the reference, which
     * uses one global kernelSize).  With adaptive_h set, every step first
     * solves h_i <= kernel_size (see mlh_smoothing_lengths) and the step uses
     * them: neighbours are the pairs with r_ij < max(h_i, h_j), particle i's
     * kernel sums (omega, E_i, psi) use W(r, h_i), its dt uses CFL * h_i.
     * kernel_size stays the search radius (cell size, image band). */
    double n_ngb;               /* target effective neighbour number */
    int adaptive_h;
} mlh_config;

/* Caller-owned host arrays (structure of arrays, float64), the fields of the
 * reference's Particles class (demonstrator/include/Particles.h:33-38) that
 * InitialDistribution fills (demonstrator/src/InitialDistribution.cpp:32-59).
 * z and vz are ignored in 2D and may be NULL there. */
typedef struct mlh_particles_view {
    int n;
    double *x, *y, *z;
    double *vx, *vy, *vz;
    double *m, *u;
} mlh_particles_view;

typedef struct mlh_step_stats {
    int steps;                       /* steps completed by this call */
    unsigned int status;             /* accumulated MLH_ERR_* bits */
    double dt;                       /* dt of the last step */
    double time;                     /* simulation time after the call */
    long long pair_interactions;     /* directed neighbour slots, summed over steps */
    long long faces;                 /* Riemann problems solved, summed */
    long long newton_iterations;     /* summed over faces and steps */
    double device_ms;                /* device time of the call (CUDA events) */
    long long newton_fallbacks;      /* faces whose learned p* guess did not
                                        converge and restarted from the
                                        two-rarefaction guess (0 without one) */
    long long learned_faces;         /* faces solved from the learned guess
                                        (strong shocks; 0 without one) */
} mlh_step_stats;

/* One simulation of an ensemble: its particle count (members are stored back
 * to back in the particle view, in member order), kernelSize and periodic box. */
typedef struct mlh_member {
    int n;
    double kernel_size;
    double box_lo[3];
    double box_hi[3];
} mlh_member;

typedef struct mlh_ctx mlh_ctx;

int mlh_abi_version(void);
const char *mlh_last_error(void);

/* Particles(N) + InitialDistribution::getAllParticles + MeshlessScheme ctor
 * (demonstrator/src/MeshlessScheme.cpp:8-19): copies the initial state to the
 * device and allocates all per-particle and per-interaction buffers.
 * MLH_ERR_INVALID for an empty or incomplete view; MLH_ERR_CAPACITY for more
 * than 2^29 - 1 particles (29-bit neighbour indices) or a face table above
 * 2^31 - 1 faces (n x neighbour slots / 2 + n: 32-bit face ids). */
int mlh_create(const mlh_config *cfg, const mlh_particles_view *init, mlh_ctx **out);
void mlh_destroy(mlh_ctx *ctx);

/* An ensemble of independent simulations of uneven sizes advanced together:
 * every stage of a step runs once for all members (one launch per kernel),
 * each member with its own kernelSize, box, grid and dt.  The settings of
 * `cfg` other than kernel_size and the box apply to every member.  No
 * counterpart in the reference (which runs one simulation per process);
 * mlh_step then advances all members by one step each. */
int mlh_ensemble_create(const mlh_config *cfg, int nmembers, const mlh_member *members,
                        const mlh_particles_view *all, mlh_ctx **out);
/* dt of the last step and simulation time of every member (host arrays of
 * nmembers doubles, either may be NULL). */
int mlh_member_times(mlh_ctx *ctx, double *dt, double *time, int nmembers);
/* Launch shapes of the step's main kernels. */
typedef struct mlh_tuning {
    int face_threads;        /* threads per block, Riemann face kernel */
    int face_blocks_per_sm;  /* blocks per SM of its grid-stride loop */
    int grad_threads;        /* threads per block, gradient/limiter kernel */
    int nns_warps_per_sm;    /* warps per SM of the neighbour search */
    int face_split;          /* faces Newton has not finished after one step:
                              * 1 go to a second, dense pass over a queue;
                              * 2 are continued inside the block by its first
                              * threads; 0: one pass (the plain gamma = 5/3
                              * step only) */
    int link_overlap;        /* 1: the face links run on a second stream beside
                              * the time step and the gradients; 2: inside the
                              * gradients kernel, each particle's links before
                              * its neighbour passes; 0: in order on the
                              * step's stream */
    int persistent_binning;  /* 1: the binning (bounds, grid, cell assignment,
                              * counts, scan, cell lists) as one persistent
                              * cooperative kernel whose phases wait on one
                              * another at bounded grid barriers (a wait that
                              * runs out sets MLH_ERR_TIMEOUT and the step
                              * leaves the state untouched); 0: one launch per
                              * phase */
    int fp32_filters;        /* single-precision filters that decide where the
                              * FP64 arithmetic runs, with the same bits as
                              * without them; bit 0 (1): the slope limiter
                              * (Particles::slopeLimiter) evaluates the
                              * face-point values f_ij only at the neighbours
                              * where a bounded estimate can reach an extremum;
                              * bit 1 (2): the time step (compGlobalTimestep)
                              * evaluates v_sig only for the particles whose
                              * bounded dt can be the minimum; 0: FP64 at every
                              * neighbour */
    int learned_guess;       /* with star-pressure weights set
                              * (mlh_set_pstar_weights): 1 runs the learned face
                              * pipeline, 0 the plain one (the weights stay
                              * set); the autotuner keeps the faster, so that
                              * the network runs only where it pays */
} mlh_tuning;

/* Autotuner: times the face-pass structures over candidate grids, then
 * candidate launch shapes of the face, gradient and neighbour kernels, then
 * whole steps with the face links in order, overlapped on a second stream
 * or inside the gradients kernel, with and without the persistent binning
 * and with and without the slope limiter's single-precision filter, over
 * `trial_steps` steps each (from a saved copy of the state, which is
 * restored afterwards), keeps the fastest in the context and reports them in
 * *out (may be NULL).  With star-pressure weights set it runs that search
 * for the learned face pipeline and for the plain one (`learned_guess`) and
 * keeps the faster.  Needs one state-sized temporary. */
int mlh_autotune(mlh_ctx *ctx, int trial_steps, mlh_tuning *out);
/* Set the launch shapes directly (for example those an autotuned context of
 * the same workload reported).  Threads per block: 64, 128 or 256; blocks
 * per SM 1..32; warps per SM 8..256; face_split and link_overlap 0, 1 or 2;
 * persistent_binning and learned_guess 0 or 1; fp32_filters 0..3.
 * MLH_ERR_INVALID otherwise. */
int mlh_set_tuning(mlh_ctx *ctx, const mlh_tuning *tuning);

/* Per-particle smoothing lengths of the current state (no counterpart in the
 * reference, which uses one global kernelSize): for every particle i the
 * support radius h_i in (0, H], H the simulation's kernel_size, at which the
 * effective neighbour number
 *     N_i(h) = V_D h^D (W(0, h) + sum_j W(|x_j - x_i|, h))
 * (V_D = pi in 2D, 4 pi / 3 in 3D; W the cubic spline of support h; images
 * by the periodic ghost rule) equals n_ngb, by a bracketed Newton iteration
 * over the particles within H, started from the context's current h_i.
 * A particle with N_i(H) < n_ngb keeps H and is counted in *clamped.  The
 * result is stored in the context (the start of the next solve, and the
 * smoothing lengths of adaptive_h steps) and copied to the host arrays h_out
 * and n_eff_out (N doubles each, either may be NULL).  n_ngb must exceed a
 * particle's own count, 32/3 in 3D and 40/7 in 2D (MLH_ERR_INVALID). */
int mlh_smoothing_lengths(mlh_ctx *ctx, double n_ngb, double *h_out, double *n_eff_out, long long *clamped);

/* Graph mode: mlh_step captures one step into a CUDA graph (once, and again
 * after a capacity change) and replays it; kernel timing bypasses it. */
int mlh_set_graph_mode(mlh_ctx *ctx, int enable);

/* Host <-> device copies of the state (x, v, m, u). */
int mlh_set_fields(mlh_ctx *ctx, const mlh_particles_view *src);
int mlh_get_fields(mlh_ctx *ctx, mlh_particles_view *dst);

/* `nsteps` MFV steps (MeshlessScheme.cpp:39-253: bin, neighbour search,
 * density, pressure, dt, gradients, limiter, faces, reconstruction, Riemann,
 * flux gather, kick/drift).  `dt_max` > 0 clamps dt (the dump-time clamp of
 * MeshlessScheme.cpp:98-101); pass 0 for none.  stats may be NULL. */
int mlh_step(mlh_ctx *ctx, int nsteps, double dt_max, mlh_step_stats *stats);

/* The first stages of a step on the current state, without advancing it:
 * grid, smoothing lengths (adaptive_h), neighbour search, density, pressure,
 * dt (clamped to dt_max > 0) and the limited gradients
 * (demonstrator/src/MeshlessScheme.cpp:39-144).  Afterwards the stage arrays
 * ("rho", "P", "omega", "noi", "nnl", "grad_*", "dt", "h", ...) describe the
 * current state: what the reference writes in Particles::dump2file
 * (demonstrator/src/Particles.cpp:2978-3076), which it calls after these
 * stages and before the Riemann solve of the same step.  mlh_step recomputes
 * them. */
int mlh_prepare(mlh_ctx *ctx, double dt_max);

/* Riemann::Riemann + Riemann::exact (demonstrator/include/Riemann.h:19-26,
 * demonstrator/src/Riemann.cpp:7-229) for n independent faces on the GPU, the
 * same device code as the step's face kernel.  Per face (host arrays, face
 * after face): Wi, the state of particle i, which is the LEFT state of the
 * solve (the reference passes it as the constructor's WL, Particles.cpp:1852),
 * and Wj, the neighbour's (RIGHT) state, each [rho, P, v_x, v_y(, v_z)]
 * (dim + 2 doubles, velocities in the frame of vFrame); vFrame and Aij (dim
 * doubles each).  Writes F (dim + 2 doubles per face: mass, energy, momentum,
 * the order of the reference's Fij) and, if iters is not NULL, the Newton
 * iterations per face (-1: no convergence).  meshless_finite_mass: the
 * MESHLESS_FINITE_MASS variant (no mass flux through the face frame).  Newton
 * tolerance 1e-10 relative, at most 100 iterations.  Returns MLH_ERR_* bits
 * (MLH_ERR_NEWTON, MLH_ERR_VACUUM, MLH_ERR_NEG_PRESSURE) accumulated over the
 * faces. */
int mlh_riemann_fluxes(int dim, int n, const double *Wi, const double *Wj, const double *vFrame, const double *Aij,
                       double gamma, int meshless_finite_mass, double *F, int *iters);

/* Copy a named per-step array of the last step to host memory, for parity
 * checks (the arrays the reference keeps as Particles members, and the
 * smoothing lengths "h", "n_eff" (N) and "h_stats" (2: solve iterations,
 * clamped particles) of the last solve):
 *   int32 : "off" (N+1), "noi", "noi_img" (N), "nnl" (uint32 index|image bits,
 *           real neighbours first in the reference's order, then images by
 *           parent index), "face_of" (per slot)
 *   double: "omega", "rho", "P" (N); "grad_rho", "grad_vx", "grad_vy",
 *           "grad_vz", "grad_P" (N*3, limited); "B" (N*dim*dim); "dt" (1);
 *           "grid" (9: lo[3], hi[3], cells[3]); "F" (per slot, dim+2, the
 *           flux of each interaction as the reference's Fij); "mF", "eF" (N),
 *           "vF" (N*3).
 * `count` receives the number of elements; `out` may be NULL to query it. */
int mlh_stage_array(mlh_ctx *ctx, const char *name, void *out, long long capacity, long long *count);

/* Per-kernel device times: when enabled, every launch of the step is
 * bracketed by CUDA events on the context's stream.  mlh_kernel_times fills
 * up to `max` entries (name, launches, total ms) and returns the count. */
int mlh_set_kernel_timing(mlh_ctx *ctx, int enable);
int mlh_kernel_times(mlh_ctx *ctx, const char **names, long long *launches, double *total_ms, int max);
void mlh_reset_kernel_times(mlh_ctx *ctx);

/* FP64 fused multiply-add throughput of the current device (TFLOP/s, an FMA
 * counts as two operations), measured for about `seconds`: the denominator
 * of the FP64 roofline.  No counterpart in the reference (it has no GPU
 * code); used by bench.py. */
int mlh_probe_fp64_tflops(double seconds, double *tflops);
/* The same, also giving the effective SM clock (MHz) of the fastest launch:
 * SM clock cycles over global-timer time of one thread's loop.  The probe's
 * TFLOP/s over (sm_mhz * SMs * 4 FP64 operations per cycle, the rate of two
 * fused multiply-adds per SM and cycle) is the share of the per-cycle FP64
 * peak it reaches. */
int mlh_probe_fp64_clock(double seconds, double *tflops, double *sm_mhz);

/* ---- Test hooks: not part of the step's interface.  They expose device
 * arithmetic and the FP64 pipe's behaviour to the test suite
 * (tests/test_gpu_fastmath.py, tests/test_gpu_fp64_lanes.py); no counterpart
 * in the reference. */

/* TEST HOOK.  The reciprocal, quotient and reciprocal square root the kernels
 * use in place of IEEE division (Newton-Raphson from the hardware estimates),
 * for n host values: rcp = 1/x, quot = y/x, rsqrt = 1/sqrt(x); for checking
 * their error against exact values. */
int mlh_probe_fast_math(int n, const double *x, const double *y, double *rcp, double *quot, double *rsqrt);

/* TEST HOOK.  The kernels' exact scalings by powers of two on the integer
 * pipe, for n host values: half = x/2, quarter = x/4, twice = 2x; for checking
 * them bit for bit against IEEE products (subnormal results included). */
int mlh_probe_scale2(int n, const double *x, double *half, double *quarter, double *twice);

/* TEST HOOK.  The grid barriers of the persistent binning wait for
 * `extra_arrivals` more blocks than the launch holds (nonzero: every wait runs
 * out, which no correct launch can make happen) and give up after
 * `spin_limit` polls (0: the default, about half a second).  For testing the
 * timeout path; 0, 0 restores the defaults. */
int mlh_test_binning_barrier(mlh_ctx *ctx, unsigned extra_arrivals, unsigned spin_limit);

/* TEST HOOK.  Device time (ms, best of three launches) of the FMA chains of
 * mlh_probe_fp64_tflops run by only the first active_lanes (1..32) lanes of
 * every warp, iters (1..2^20) steps: how the FP64 pipe charges a partially
 * active warp instruction. */
int mlh_probe_fp64_lanes(int active_lanes, int iters, double *ms);

/* ---- End of the test hooks. */

/* Learned initial guess for the Riemann star pressure (no counterpart in the
 * reference): a 4-64-64-64-1 SiLU MLP, 8705 float parameters laid out as
 * W1[64][4], b1[64], W2[64][64], b2[64], W3[64][64], b3[64], W4[64], b4,
 * evaluated on the tensor cores in BF16 with FP32 accumulation.  Input per
 * face (4 floats), from the face-frame states sorted by pressure (side A the
 * lower, B the higher; the mirror image negates both normal velocities, so
 * du = uB - uA is that of the unsorted problem): log(rhoB/rhoA), du/cA,
 * log(pB/pA), log(cB/cA), with c = sqrt(gamma p / rho); output y, one float
 * per row.  The
 * step reads y as log(p* / p_TR), p_TR the two-rarefaction guess of the face
 * (Toro eq. 4.46).  All arrays are host arrays. */
int mlh_pstar_infer(const float *weights, const float *x, int n, float *y);
/* Mean squared error over n samples and its gradient (8705 floats). */
int mlh_pstar_grad(const float *weights, const float *x, const float *t, int n, float *loss, float *grad);
/* Adam training on the GPU (epochs over shuffled mini-batches, the learning
 * rate decayed from lr to lr / 100 along a half cosine), in place on
 * `weights`; loss_history (epochs floats, may be NULL) gets the mean batch loss. */
int mlh_pstar_train(const float *x, const float *t, long long n, int epochs, int batch, float lr, unsigned seed,
                    float *weights, float *loss_history);

/* Use the network (weights: 8705 floats) for the initial guess of the
 * Riemann problems of the context's steps: p_TR * exp(y) where |y| > 0.01,
 * p_TR (the two-rarefaction guess) elsewhere; NULL returns to p_TR
 * everywhere.  Newton still iterates to riemann_tol and restarts from p_TR
 * when it does not converge from the network's guess
 * (mlh_step_stats.newton_fallbacks counts those faces). */
int mlh_set_pstar_weights(mlh_ctx *ctx, const float *weights);
/* One mlh_step(ctx, 1, 0, NULL) that also records the network inputs (4
 * floats) and targets log(p* / p_TR) of every `stride`-th face into x, t
 * (host, capacity rows); *count receives the number of rows. */
int mlh_pstar_harvest(mlh_ctx *ctx, int stride, float *x, float *t, long long capacity, long long *count);
/* The same, recording every face that the learned step hands to the network
 * (two-rarefaction guess above 2 min(pL, pR): strong shocks).  *count
 * receives the number of such faces (rows beyond capacity are dropped). */
int mlh_pstar_harvest_strong(mlh_ctx *ctx, float *x, float *t, long long capacity, long long *count);

/* Largest particle count mlh_grid_bounds_noalloc accepts (29-bit indices). */
#define MLH_NOALLOC_MAX_PARTICLES ((1 << 29) - 1)

/* Search grid of one step computed without allocating any memory: for
 * callers that cannot call cudaMalloc (frameworks that own all device memory
 * through their own pool, loops that must not allocate after start-up).  No
 * counterpart in the reference:
 * it computes what Particles::getDomainLimits + Domain::createGrid compute at
 * the start of a non-periodic step (the box itself when `periodic`), as
 * mlh_step does, from caller-owned device arrays x, y (, z) of n particles.
 * Writes 9 doubles to the device buffer grid_out: lo[3], hi[3], cells[3]
 * (unused axes 0).  box_lo/box_hi are host arrays, read only when periodic.
 * stream: a cudaStream_t, or NULL for the default stream; the call waits for
 * it to finish.
 * Scratch: a fixed 16 KiB static device array that every GPU loading the
 * library keeps until exit; its device address is looked up on the first
 * call on each device, so make that first call before any stream capture.
 * Every call shares the same scratch: calls that overlap on the GPU (from
 * several host threads or streams at once) race and must be serialised by
 * the caller.  n > MLH_NOALLOC_MAX_PARTICLES returns MLH_ERR_CAPACITY
 * (message in mlh_last_error()). */
int mlh_grid_bounds_noalloc(int dim, int periodic, int n, const double *x, const double *y, const double *z,
                            const double *box_lo, const double *box_hi, double kernel_size, double *grid_out,
                            void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MLH_H */
