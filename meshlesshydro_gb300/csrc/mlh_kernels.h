// Host-visible interface of the step kernels (mlh_kernels.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mlh_device.cuh"

namespace mlh {

enum KernelTimerId { KT_GRID = 0, KT_NNS, KT_DT, KT_GRAD, KT_LINK, KT_FACES, KT_UPDATE, KT_HSOLVE, KT_COUNT };

// Launch shapes chosen by the autotuner (mlh_autotune).
struct Tuning {
    int face_threads = 128;        // threads per block of k_faces
    int face_blocks_per_sm = 8;    // grid of the grid-stride face loop
    int grad_threads = 128;        // threads per block of k_gradients
    int nns_warps_per_sm = 64;     // warps (= particles in flight) of k_neighbours
    int face_split = 1;            // plain gamma = 5/3 step: 1 second Newton pass over a queue, 2 in-block, 0 none
    int link_overlap = 1;          // face links on the second stream beside the time step and gradients
    int persistent_binning = 0;    // the binning as one persistent cooperative kernel (k_binning)
    int fp32_filters = 3;          // bits: 1 slope-limiter extrema, 2 time step (FP64 only where a single-precision bound reaches the result)
    int learned_guess = 1;         // with weights set: 1 the learned face pipeline, 0 the plain one
};

// bits of Tuning::fp32_filters
constexpr int MLH_FILTER_SLOPE = 1, MLH_FILTER_TIMESTEP = 2;

// Device pointers and settings of one step.
struct StepArgs {
    Tuning tune;
    Params p;
    cudaStream_t stream;
    // second stream for the face links, with the events of its fork and join
    // (null: everything on `stream`)
    cudaStream_t stream2;
    cudaEvent_t ev_fork, ev_join;
    int face_blocks;
    int sm_count;
    int root5;              // gamma = 5/3 fast path of the Riemann solver
    size_t faces_cap;
    double dt_max;
    // state (structure of arrays)
    double *x, *y, *z, *vx, *vy, *vz, *m, *u;
    float4 *posf;
    // velocity and sound speed in single precision (written with the
    // density); the time step's bounds: per particle a lower bound on dt,
    // per simulation the least upper bound (float bits)
    float4 *velf;
    float *dtlo;
    unsigned *dtcap;
    // simulations (members) of the context
    int nmembers;
    int bpm;                   // bounding-box blocks per member
    const Member *members;
    const int *memberOf;       // per particle; nullptr when nmembers == 1
    // grids, one per member
    GridInfo *grids;
    int *cellTotal;
    double *boundsPart;
    int *cell, *cellCount, *cellStart, *cellFill, *cellList;
    // neighbours
    uint32_t *nbr;
    double *rr, *ww, *psi;
    int *noi, *noiImg, *faceCnt, *faceOff, *faceOf;
    FaceRef *faces;
    // per particle
    Prim *prim;
    Geo *geo;
    Grad *grad, *gradRaw;
    double *Fface, *fluxSums;
    // scalars
    unsigned *status;
    unsigned long long *dtbits, *newtonSum;
    double *dt, *simTime;
    int *stepsDone;
    int *scanTiles, *scanTotal;
    // learned p* guess: queue of the faces handed to the network (face ids,
    // their face-frame states, network inputs and outputs), packed weights
    int learned;
    FaceState *fstate;      // queue A: strong shocks (learned) or the plain second pass
    FaceState *fstate2;     // queue B: the learned step's second Newton pass
    int *queueFace2;
    int *queueCount2;
    int qcap, qcap2;
    float4 *feat;
    float *yguess;
    int *queueFace;
    int *queueCount;
    const void *mlp_packed;
    Harvest harvest;
    // per-particle smoothing lengths: h (also p.hp), effective neighbour
    // number (may be null), counters [iterations, clamped particles]
    double *hp, *neff;
    float *hpf;   // hp rounded up to single precision, written beside it
    unsigned long long *hstat;
    // end the step after the gradients and the limiter (mlh_prepare)
    int stop_after_gradients;
    // the time step as its own kernel (k_timestep) instead of inside the
    // gradients' first neighbour pass
    int separate_dt;
    // persistent binning: its grid-barrier words (2 unsigned), its block
    // count (resident blocks, 0: unavailable), extra arrivals the barriers
    // wait for (a test hook: nonzero makes every wait run out) and the polls
    // before a wait gives up
    unsigned *bar;
    int bin_blocks;
    unsigned bar_extra, bar_spin;
    // optional per-kernel timer callback (phase 0 = before, 1 = after)
    void (*timer)(void *, int, int);
    void *timer_ctx;
};

// blocks of the bounding-box reduction of a single simulation; its scratch
// holds 6 doubles per block
constexpr int BOUNDS_BLOCKS = 304;

void step(StepArgs &a);
// blocks of the persistent binning kernel resident at once (0: none)
int binning_blocks(int dim, int sm_count);
// binning and the smoothing-length solve alone, on the current positions
void smoothing_lengths(StepArgs &a);
// Particles::getDomainLimits + Domain::createGrid alone: per-block partial
// minima/maxima in `partials` (nmembers * bpm * 6 doubles), one GridInfo per
// member in `grids`, the concatenated cell count in `cellTotal`.
void launch_grid_bounds(const double *x, const double *y, const double *z, const Params &p,
                        const Member *members, int nmembers, int bpm, double *partials, GridInfo *grids,
                        int *cellTotal, unsigned *status, cudaStream_t s);
void pack_posf(const double *x, const double *y, const double *z, int n, int dim, float4 *posf, cudaStream_t s);
void exclusive_scan(const int *in, int n, int *out, int *tile_buf, int *total, cudaStream_t s);
const char *kernel_timer_name(int id);
// Riemann problems of n independent faces (device arrays; see k_riemann_batch)
void riemann_batch(int dim, int n, double gamma, double rtol, int max_iter, int mfm, const double *Wi,
                   const double *Wj, const double *vFrame, const double *Aij, double *F, int *iters,
                   unsigned *status, cudaStream_t s);
void set_last_error(const char *msg);
// MLP inference over the faces of a step: n read on the device (min with cap)
void pstar_infer_dev(const float4 *x, const int *n_dev, int cap, const void *packed, float *y, int sm_count,
                     cudaStream_t s);

}  // namespace mlh
