// MFV timestep kernels for GB300 (sm_103a), FP64 state.
//
// One step = the stage sequence of the reference's MeshlessScheme::run
// (jammartin/meshlessHydro, demonstrator/src/MeshlessScheme.cpp:39-253):
//   bounds + grid        Particles::getDomainLimits / Domain::createGrid
//   bin                  Particles::assignParticlesAndCells
//   neighbour search     Particles::gridNNS + ghostNNS (images via wrapped cells)
//   density, pressure    Particles::compDensity / compPressure
//   dt                   Particles::compGlobalTimestep
//   E^-1, gradients,     Particles::compPsijTilde / gradient / slopeLimiter
//   limiter
//   faces                compEffectiveFace + compRiemannStatesLR +
//                        solveRiemannProblems (one thread per canonical face)
//   gather + kick/drift  collectFluxes + updateStateAndPosition
//
// Determinism: no floating-point atomics.  Every per-particle sum runs over the
// neighbour list in the reference's order; each face flux is computed once,
// from the side of the lower particle index, and gathered with sign.
#include "mlh_device.cuh"
#include "mlh_riemann.cuh"
#include "mlh_kernels.h"
#include "mlh_mlp.cuh"

#include <cfloat>

namespace mlh {

// ------------------------------------------------------------------ helpers

__device__ __forceinline__ double atomic_min_pos_double(unsigned long long *addr, double v) {
    // positive doubles order like their bit patterns
    return (double)atomicMin(addr, (unsigned long long)__double_as_longlong(v));
}

template <typename T>
__device__ __forceinline__ T warp_reduce_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ------------------------------------------------------------------ scan

// Exclusive scan of int counts in three launches (tile reduce, scan of tile
// sums in one block, tile scan).  Tile = 1024 threads x 4 items.
constexpr int SCAN_T = 1024, SCAN_I = 4, SCAN_TILE = SCAN_T * SCAN_I;

__device__ __forceinline__ int block_exclusive_scan(int v, int *smem, int &total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem[w] = x;
    __syncthreads();
    if (w == 0) {
        int s = (lane < (int)(blockDim.x >> 5)) ? smem[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        smem[lane] = s;
    }
    __syncthreads();
    int base = w > 0 ? smem[w - 1] : 0;
    total = smem[(blockDim.x >> 5) - 1];
    __syncthreads();
    return base + x - v;
}

__global__ void k_scan_reduce(const int *__restrict__ in, int n, int *__restrict__ tile_sums) {
    __shared__ int smem[32];
    long long base = (long long)blockIdx.x * SCAN_TILE;
    int s = 0;
    for (int k = 0; k < SCAN_I; ++k) {
        long long idx = base + (long long)k * SCAN_T + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    s = warp_reduce_sum(s);
    if ((threadIdx.x & 31) == 0) smem[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int v = threadIdx.x < (blockDim.x >> 5) ? smem[threadIdx.x] : 0;
        v = warp_reduce_sum(v);
        if (threadIdx.x == 0) tile_sums[blockIdx.x] = v;
    }
}

__global__ void k_scan_tiles(int *__restrict__ tile_sums, int ntiles, int *__restrict__ total_out) {
    __shared__ int smem[32];
    int carry = 0;
    for (int b = 0; b < ntiles; b += SCAN_T) {
        int idx = b + threadIdx.x;
        int v = idx < ntiles ? tile_sums[idx] : 0;
        int tot;
        int ex = block_exclusive_scan(v, smem, tot);
        if (idx < ntiles) tile_sums[idx] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) *total_out = carry;
}

__global__ void k_scan_apply(const int *__restrict__ in, int n, const int *__restrict__ tile_offsets,
                             int *__restrict__ out, const int *__restrict__ total, int write_total_at_n) {
    __shared__ int smem[32];
    long long base = (long long)blockIdx.x * SCAN_TILE;
    long long idx0 = base + (long long)threadIdx.x * SCAN_I;
    int v[SCAN_I];
    int loc = 0;
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) {
        long long idx = idx0 + k;
        v[k] = idx < n ? in[idx] : 0;
        loc += v[k];
    }
    int tot;
    int ex = block_exclusive_scan(loc, smem, tot) + tile_offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_I; ++k) {
        long long idx = idx0 + k;
        if (idx < n) out[idx] = ex;
        ex += v[k];
    }
    if (write_total_at_n && blockIdx.x == 0 && threadIdx.x == 0) out[n] = *total;
}

void exclusive_scan(const int *in, int n, int *out, int *tile_buf, int *total, cudaStream_t s) {
    int ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (ntiles < 1) ntiles = 1;
    k_scan_reduce<<<ntiles, SCAN_T, 0, s>>>(in, n, tile_buf);
    k_scan_tiles<<<1, SCAN_T, 0, s>>>(tile_buf, ntiles, total);
    k_scan_apply<<<ntiles, SCAN_T, 0, s>>>(in, n, tile_buf, out, total, 1);
}

// ------------------------------------------------------------------ bounds + grid

// Particles::getDomainLimits (Particles.cpp:228-267): lo = min over all
// particles; because of `else if` and numeric_limits<double>::min(), hi = the
// max over i >= 1 of the x_i that are not below the running minimum of
// x_0..x_{i-1}, or DBL_MIN.  The partial pass computes min over all i and max
// over i >= 1 of each simulation's range (blocks_per_member blocks each); the
// final pass falls back to the sequential rule whenever x_0 is above every
// other particle (the only case where the two differ).
constexpr int BOUNDS_T = 256;

// the partial minima and maxima of virtual block vb (block vb % bpm of member
// vb / bpm), for a block of BOUNDS_T threads
template <int D>
__device__ __forceinline__ void bounds_partial_block(int vb, const double *__restrict__ x,
                                                     const double *__restrict__ y, const double *__restrict__ z,
                                                     const Params &p, const Member *__restrict__ members, int bpm,
                                                     double *__restrict__ part) {
    __shared__ double smin[3][BOUNDS_T / 32], smax[3][BOUNDS_T / 32];
    const int mi = vb / bpm, sub = vb % bpm;
    const Member mb = members[mi];
    const double *X[3] = {x, y, z};
    double mn[3], mx[3];
    for (int a = 0; a < 3; ++a) { mn[a] = DBL_MAX_; mx[a] = -DBL_MAX_; }
    if (!p.periodic) {
        const int end = mb.first + mb.count;
        for (int i = mb.first + sub * blockDim.x + threadIdx.x; i < end; i += bpm * blockDim.x) {
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double v = X[a][i];
                mn[a] = fmin(mn[a], v);
                if (i >= mb.first + 1) mx[a] = fmax(mx[a], v);
            }
        }
    }
#pragma unroll
    for (int a = 0; a < D; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[a] = fmin(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = fmax(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
        if ((threadIdx.x & 31) == 0) { smin[a][threadIdx.x >> 5] = mn[a]; smax[a][threadIdx.x >> 5] = mx[a]; }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int a = 0; a < D; ++a) {
            double a0 = DBL_MAX_, a1 = -DBL_MAX_;
            for (int w = 0; w < BOUNDS_T / 32; ++w) { a0 = fmin(a0, smin[a][w]); a1 = fmax(a1, smax[a][w]); }
            part[(vb * 3 + a) * 2 + 0] = a0;
            part[(vb * 3 + a) * 2 + 1] = a1;
        }
    }
    __syncthreads();   // the shared partials are reused by the next virtual block
}

template <int D>
__global__ void k_bounds_partial(const double *__restrict__ x, const double *__restrict__ y,
                                 const double *__restrict__ z, Params p, const Member *__restrict__ members,
                                 int bpm, double *__restrict__ part) {
    bounds_partial_block<D>(blockIdx.x, x, y, z, p, members, bpm, part);
}

// Final pass + Domain::createGrid (Domain.cpp:9-54) for every simulation,
// then the cell numbering of the concatenated grids.  For periodic runs the
// bounds are the configured box.
template <int D>
__device__ __forceinline__ void bounds_final_block(const double *__restrict__ x, const double *__restrict__ y,
                                                   const double *__restrict__ z, const double *__restrict__ part,
                                                   int bpm, const Params &p, const Member *__restrict__ members,
                                                   int nmembers, GridInfo *__restrict__ grids,
                                                   int *__restrict__ cellTotal, unsigned *__restrict__ status) {
    const double *X[3] = {x, y, z};
    for (int mi = threadIdx.x; mi < nmembers; mi += blockDim.x) {
        const Member mb = members[mi];
        GridInfo g;
        for (int a = 0; a < 3; ++a) { g.lo[a] = 0.; g.hi[a] = 0.; g.cs[a] = 1.; g.cells[a] = 1; }
        for (int a = 0; a < D; ++a) {
            if (p.periodic) { g.lo[a] = mb.box_lo[a]; g.hi[a] = mb.box_hi[a]; continue; }
            double mn = DBL_MAX_, mx1 = -DBL_MAX_;
            for (int b = mi * bpm; b < (mi + 1) * bpm; ++b) {
                mn = fmin(mn, part[(b * 3 + a) * 2]);
                mx1 = fmax(mx1, part[(b * 3 + a) * 2 + 1]);
            }
            const double x0 = X[a][mb.first];
            double hi;
            if (mb.count < 2 || !(mx1 >= x0)) {
                // sequential rule of the reference
                double lo_s = DBL_MAX_, hi_s = DBL_MIN_;
                for (int i = mb.first; i < mb.first + mb.count; ++i) {
                    double v = X[a][i];
                    if (v < lo_s) lo_s = v;
                    else if (v > hi_s) hi_s = v;
                }
                hi = hi_s;
            } else {
                hi = mx1 > DBL_MIN_ ? mx1 : DBL_MIN_;
            }
            g.lo[a] = mn;
            g.hi[a] = hi;
        }
        // the product saturates at ncells_cap + 1 (each factor is below 2^31,
        // so the product of the saturated value and one factor fits in 64 bits)
        long long total = 1;
        for (int a = 0; a < D; ++a) {
            double c = floor((g.hi[a] - g.lo[a]) / mb.h);
            int ci = (c >= 1. && c < 2147483647.) ? (int)c : 1;
            if (!(c >= 1.)) flag(status, ST_GRID);
            if (c >= 2147483647.) { flag(status, ST_CAPACITY); ci = 1; }
            if (p.periodic && ci < 3) flag(status, ST_GRID);
            g.cells[a] = ci;
            total *= ci;
            if (total > p.ncells_cap) total = (long long)p.ncells_cap + 1;
        }
        for (int a = 0; a < D; ++a) g.cs[a] = (g.hi[a] - g.lo[a]) / (double)g.cells[a];
        for (int a = 0; a < 3; ++a) {
            g.band_lo[a] = g.lo[a] + mb.h;
            g.band_hi[a] = g.hi[a] - mb.h;
            g.Lf[a] = (float)(g.hi[a] - g.lo[a]);
        }
        if (total > p.ncells_cap) { flag(status, ST_CAPACITY); total = 1; }
        g.ncells = (int)total;
        g.cell_base = 0;
        grids[mi] = g;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long base = 0;
        for (int mi = 0; mi < nmembers; ++mi) {
            int nc = grids[mi].ncells;
            if (base + nc > p.ncells_cap) { flag(status, ST_CAPACITY); nc = 0; grids[mi].ncells = 0; }
            grids[mi].cell_base = (int)base;
            base += nc;
        }
        *cellTotal = (int)base;
    }
}

template <int D>
__global__ void k_bounds_final(const double *__restrict__ x, const double *__restrict__ y,
                               const double *__restrict__ z, const double *__restrict__ part, int bpm, Params p,
                               const Member *__restrict__ members, int nmembers, GridInfo *__restrict__ grids,
                               int *__restrict__ cellTotal, unsigned *__restrict__ status) {
    bounds_final_block<D>(x, y, z, part, bpm, p, members, nmembers, grids, cellTotal, status);
}

// Particles::assignParticlesAndCells (Particles.cpp:270-322).
template <int D>
__device__ __forceinline__ void assign_one(int i, const double *__restrict__ x, const double *__restrict__ y,
                                           const double *__restrict__ z, const int *__restrict__ memberOf,
                                           const GridInfo *__restrict__ grids, int *__restrict__ cell,
                                           int *__restrict__ cellCount, unsigned *__restrict__ status) {
    const double *X[3] = {x, y, z};
    {
        const GridInfo g = grids[memberOf ? memberOf[i] : 0];
        int fl[3] = {0, 0, 0};
        bool bad = false;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double f = floor((X[a][i] - g.lo[a]) / g.cs[a]);
            int fi = (f > -1e9 && f < 1e9) ? (int)f : -1;
            if (fi == g.cells[a]) fi -= 1;
            if (fi < 0 || fi >= g.cells[a]) { bad = true; fi = fi < 0 ? 0 : g.cells[a] - 1; }
            fl[a] = fi;
        }
        if (bad) flag(status, ST_GRID);
        int c = fl[0] + fl[1] * g.cells[0] + (D == 3 ? fl[2] * g.cells[0] * g.cells[1] : 0);
        if (c >= g.ncells) { c = g.ncells > 0 ? g.ncells - 1 : 0; flag(status, ST_GRID); }
        c += g.cell_base;
        cell[i] = c;
        atomicAdd(&cellCount[c], 1);
    }
}

template <int D>
__global__ void k_assign(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                         int n, const int *__restrict__ memberOf, const GridInfo *__restrict__ grids,
                         int *__restrict__ cell, int *__restrict__ cellCount, unsigned *__restrict__ status) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        assign_one<D>(i, x, y, z, memberOf, grids, cell, cellCount, status);
}

// True when the binning of this step is not valid: a bounded wait gave up
// (ST_TIMEOUT), a particle fell outside the grid (ST_GRID: outside the box,
// a NaN coordinate, or fewer than 3 cells on a periodic axis) or the cells
// exceed their buffers (ST_CAPACITY, the step is repeated with more).  The
// kernels that read the binning then skip their work: the step completes
// nothing and reports the bits, and a NaN particle, which the grid clamps
// into one cell, cannot make a cell of every particle whose sort and search
// are quadratic in its size.  The value is the same for every thread of a
// launch (the bits are set by earlier kernels or before a grid barrier).
__device__ __forceinline__ bool step_aborted(const unsigned *status) {
    return (*(volatile const unsigned *)status & (ST_TIMEOUT | ST_GRID | ST_CAPACITY)) != 0u;
}

__global__ void k_fill_cells(const int *__restrict__ cell, int n, const int *__restrict__ cellStart,
                             int *__restrict__ cellFill, int *__restrict__ cellList,
                             const unsigned *__restrict__ status) {
    if (step_aborted(status)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int c = cell[i];
        int pos = atomicAdd(&cellFill[c], 1);
        cellList[cellStart[c] + pos] = i;
    }
}

// Members of a cell in ascending particle index: the order in which
// assignParticlesAndCells pushes them (Particles.cpp:319).
__device__ __forceinline__ void sort_cell(int c, const int *__restrict__ cellStart, int *__restrict__ cellList) {
    int b = cellStart[c], e = cellStart[c + 1];
    for (int k = b + 1; k < e; ++k) {
        int v = cellList[k];
        int t = k - 1;
        while (t >= b && cellList[t] > v) { cellList[t + 1] = cellList[t]; --t; }
        cellList[t + 1] = v;
    }
}

__global__ void k_sort_cells(const int *__restrict__ cellTotal, const int *__restrict__ cellStart,
                             int *__restrict__ cellList, const unsigned *__restrict__ status) {
    if (step_aborted(status)) return;
    const int nc = *cellTotal;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x)
        sort_cell(c, cellStart, cellList);
}

// ------------------------------------------------------------------ persistent binning

// The binning of a step (bounds, grid, assignment, cell counts, their scan,
// cell lists, in-cell order) as one persistent kernel: a cooperative launch of
// at most the blocks the GPU holds at once, its phases separated by grid
// barriers.  Results are those of the launch-per-phase sequence (integer and
// min/max work, the cell lists sorted).
//
// Grid barrier: arrivals counted in bar.count, phases in bar.gen; the last
// block to arrive resets the count and opens the next phase.  Every wait is
// bounded: after bar.spin_limit polls (each followed by a short sleep) the
// block sets ST_TIMEOUT and leaves the kernel, and so does every other block
// (a block that left does not arrive again, so the others run out too).  The
// step's later kernels that read the binning skip their work when ST_TIMEOUT
// is set, so that a step which timed out leaves the state untouched.
struct GridBar {
    unsigned *count;
    unsigned *gen;
    unsigned expected;     // blocks that arrive at each barrier
    unsigned spin_limit;   // polls before giving up
};

__device__ __forceinline__ bool grid_sync(const GridBar &b, unsigned *status) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int good = 1;
        __threadfence();
        const unsigned g = *(volatile unsigned *)b.gen;
        const unsigned prev = atomicAdd(b.count, 1u);
        if (prev + 1 == b.expected) {
            atomicExch(b.count, 0u);
            __threadfence();
            atomicAdd(b.gen, 1u);
        } else {
            unsigned polls = 0;
            while (*(volatile unsigned *)b.gen == g) {
                if (++polls > b.spin_limit) {
                    good = 0;
                    flag(status, ST_TIMEOUT);
                    break;
                }
                __nanosleep(256);
            }
        }
        __threadfence();
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

constexpr int PB_T = 256;                    // threads per block of k_binning
constexpr int PB_ITEMS = SCAN_TILE / PB_T;   // scan items per thread (a tile of SCAN_TILE counts)

template <int D>
__global__ void __launch_bounds__(PB_T) k_binning(const double *__restrict__ x, const double *__restrict__ y,
                                                  const double *__restrict__ z, Params p,
                                                  const Member *__restrict__ members, const int *__restrict__ memberOf,
                                                  int nmembers, int bpm, double *__restrict__ part,
                                                  GridInfo *__restrict__ grids, int *__restrict__ cellTotal,
                                                  int *__restrict__ cell, int *__restrict__ cellCount,
                                                  int *__restrict__ cellStart, int *__restrict__ cellFill,
                                                  int *__restrict__ cellList, int *__restrict__ tileSums,
                                                  int *__restrict__ scanTotal, unsigned *__restrict__ status,
                                                  GridBar bar) {
    __shared__ int smem[32];
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nthr = gridDim.x * blockDim.x;
    const int ncap = p.ncells_cap;
    const int ntiles = (ncap + SCAN_TILE - 1) / SCAN_TILE;
    // 1: partial bounds of every member; clear the cell counters
    for (int vb = blockIdx.x; vb < nmembers * bpm; vb += gridDim.x)
        bounds_partial_block<D>(vb, x, y, z, p, members, bpm, part);
    for (int k = tid; k <= ncap; k += nthr) { cellCount[k] = 0; cellFill[k] = 0; }
    if (!grid_sync(bar, status)) return;
    // 2: final bounds and Domain::createGrid (one block)
    if (blockIdx.x == 0) bounds_final_block<D>(x, y, z, part, bpm, p, members, nmembers, grids, cellTotal, status);
    if (!grid_sync(bar, status)) return;
    // 3: Particles::assignParticlesAndCells and the cell counts
    for (int i = tid; i < p.n; i += nthr) assign_one<D>(i, x, y, z, memberOf, grids, cell, cellCount, status);
    if (!grid_sync(bar, status)) return;
    // the same decision in every block: the bits were set before the barrier
    if (step_aborted(status)) return;
    // 4: exclusive scan of the counts: tile sums, their scan, the tiles
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long b0 = (long long)t * SCAN_TILE + (long long)threadIdx.x * PB_ITEMS;
        int sum = 0;
#pragma unroll 4
        for (int k = 0; k < PB_ITEMS; ++k) sum += b0 + k < ncap ? cellCount[b0 + k] : 0;
        int tot;
        (void)block_exclusive_scan(sum, smem, tot);
        if (threadIdx.x == 0) tileSums[t] = tot;
    }
    if (!grid_sync(bar, status)) return;
    if (blockIdx.x == 0) {
        int carry = 0;
        for (int b = 0; b < ntiles; b += PB_T) {
            const int idx = b + threadIdx.x;
            const int v = idx < ntiles ? tileSums[idx] : 0;
            int tot;
            const int ex = block_exclusive_scan(v, smem, tot);
            if (idx < ntiles) tileSums[idx] = carry + ex;
            carry += tot;
        }
        if (threadIdx.x == 0) { *scanTotal = carry; cellStart[ncap] = carry; }
    }
    if (!grid_sync(bar, status)) return;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const long long b0 = (long long)t * SCAN_TILE + (long long)threadIdx.x * PB_ITEMS;
        int sum = 0;
#pragma unroll 4
        for (int k = 0; k < PB_ITEMS; ++k) sum += b0 + k < ncap ? cellCount[b0 + k] : 0;
        int tot;
        int ex = block_exclusive_scan(sum, smem, tot) + tileSums[t];
#pragma unroll 4
        for (int k = 0; k < PB_ITEMS; ++k) {
            if (b0 + k < ncap) {
                const int v = cellCount[b0 + k];
                cellStart[b0 + k] = ex;
                ex += v;
            }
        }
    }
    if (!grid_sync(bar, status)) return;
    // 5: cell lists, then the reference's in-cell order
    for (int i = tid; i < p.n; i += nthr) {
        const int c = cell[i];
        const int pos = atomicAdd(&cellFill[c], 1);
        cellList[cellStart[c] + pos] = i;
    }
    if (!grid_sync(bar, status)) return;
    const int nc = *cellTotal;
    for (int c = tid; c < nc; c += nthr) sort_cell(c, cellStart, cellList);
}

// ------------------------------------------------------------------ neighbour search

// Particles::gridNNS (Particles.cpp:324-365) over the 3^D stencil of
// Domain::getNeighborCells (Domain.cpp:83-118, x outer, z inner), and the
// periodic images of Particles::ghostNNS (Particles.cpp:2237-2260) through
// wrapped stencil cells, appended after the real neighbours in parent order.
// Then Particles::compDensity/compOmega (Particles.cpp:1151-1184, 2262-2290)
// and compPressure (:1272-1288) for the particle.
//
// One warp per cell: the particles of a cell share the candidate sequence
// (the stencil cells of their cell, in order), so the warp stages it in
// shared memory once, 128 candidates at a time (index with image bits, and
// the single-precision position with the image shift applied), and filters
// every chunk for a batch of up to NNS_PB particles of the cell against the
// staged copy: a single-precision distance test against a bound slightly
// above h^2, survivors compacted with a ballot into the particle's shared
// list in stencil order.  Then, particle by particle, phase 2: the lanes take
// the survivors 32 at a time and apply the reference's FP64 test exactly (d^2
// = (dx*dx + dy*dy) + dz*dz < h*h, no fused multiply-add), compute r and
// W(r), and append real neighbours (in order) to the slot list and images to
// a shared list, which is then placed behind the real neighbours sorted by
// parent index.  The single-precision test only decides which candidates
// phase 2 sees; it passes every neighbour (its error is far below the bound's
// margin), so the lists are those of the FP64 test alone.
constexpr int NNS_WARPS = 8;
constexpr int NNS_PB = 12;    // particles of a cell filtered per staged chunk
constexpr int NNS_CH = 128;   // candidates per staged chunk
// blocks of the neighbour search resident per SM: 3 caps it at 80 registers
// and gives 24 warps per SM
#ifndef MLH_NNS_MINB
#define MLH_NNS_MINB 3
#endif

struct NnsCells {
    int excl[27], start[27];
    unsigned wrap[27];
    float shift[27][3];   // image shift of a wrapped axis (-L or +L, single precision), else 0
};

// shared memory of k_neighbours: NNS_WARPS NnsCells, then per warp the
// staged chunk (NNS_CH float4 positions and entries), NNS_PB candidate lists
// (K + 32 uint32 each), four NNS_PB int arrays (candidate counts, offsets in
// the batch's sequence, real and image neighbour counts), image r and W (K
// doubles each) and image entries (K uint32), each rounded up to 16 bytes
__host__ __device__ constexpr size_t nns_cells_bytes() {
    return (sizeof(NnsCells) * NNS_WARPS + 15) / 16 * 16;
}
__host__ __device__ constexpr size_t nns_r16(size_t b) { return (b + 15) / 16 * 16; }
// (with per-particle smoothing lengths also the staged chunk's h_j, NNS_CH
// floats, at the end: without them the area of 8 warps stays within a third
// of the SM's shared memory at K = 64, for 3 blocks per SM)
__host__ __device__ constexpr size_t nns_warp_bytes(int K, bool adaptive = false) {
    return (size_t)NNS_CH * 4 + (size_t)NNS_CH * 16 + nns_r16((size_t)NNS_PB * (K + 32) * 4) +
           nns_r16((size_t)4 * NNS_PB * 4) + (size_t)K * 16 + nns_r16((size_t)K * 4) +
           (adaptive ? (size_t)NNS_CH * 4 : 0);
}

// The 3^D stencil cells of local cell ic in the reference's order
// (Domain::getNeighborCells, demonstrator/src/Domain.cpp:83-118; lane k
// holds cell k), written to the warp's NnsCells: the offset of each cell's
// members in the concatenated sequence, the start of its member list, its
// wrapped axes and image shift.  Returns the length of the sequence.
template <int D>
__device__ __forceinline__ int nns_stencil(const Params &p, const GridInfo &g, int ic,
                                           const int *__restrict__ cellStart, NnsCells *cs) {
    constexpr int NC = D == 3 ? 27 : 9;
    const int lane = threadIdx.x & 31;
    const int ix = ic % g.cells[0];
    const int iy = (ic / g.cells[0]) % g.cells[1];
    const int iz = D == 3 ? ic / (g.cells[0] * g.cells[1]) : 0;
    int cnt = 0, start = 0;
    unsigned wrap = 0;
    float sh[3] = {0.f, 0.f, 0.f};
    if (lane < NC) {
        int off[3] = {D == 3 ? lane / 9 - 1 : lane / 3 - 1, D == 3 ? (lane / 3) % 3 - 1 : lane % 3 - 1,
                      D == 3 ? lane % 3 - 1 : 0};
        int cc[3] = {ix + off[0], iy + off[1], iz + off[2]};
        bool skip = false;
#pragma unroll
        for (int a = 0; a < D; ++a) {
            if (cc[a] < 0 || cc[a] >= g.cells[a]) {
                if (!p.periodic) skip = true;
                cc[a] = cc[a] < 0 ? cc[a] + g.cells[a] : cc[a] - g.cells[a];
                wrap |= 1u << a;
                sh[a] = off[a] < 0 ? -g.Lf[a] : g.Lf[a];
            }
        }
        if (!skip) {
            int c = g.cell_base + cc[0] + cc[1] * g.cells[0] + (D == 3 ? cc[2] * g.cells[0] * g.cells[1] : 0);
            start = cellStart[c];
            cnt = cellStart[c + 1] - start;
        }
    }
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const int total = __shfl_sync(0xffffffffu, incl, 31);
    if (lane < NC) {
        cs->excl[lane] = incl - cnt;
        cs->start[lane] = start;
        cs->wrap[lane] = wrap;
        cs->shift[lane][0] = sh[0]; cs->shift[lane][1] = sh[1]; cs->shift[lane][2] = sh[2];
    }
    __syncwarp();
    return total;
}

// Stencil cell of position t of the concatenated sequence: the last cell
// whose range starts at or before t (empty cells share their offset with the
// next one), by binary search over the non-decreasing offsets.
template <int D>
__device__ __forceinline__ int nns_cell_of(const NnsCells *cs, int t) {
    constexpr int NC = D == 3 ? 27 : 9;
    int k = 0;
#pragma unroll
    for (int step = 16; step > 0; step >>= 1) {
        const int kk = k + step;
        if (kk < NC && cs->excl[kk] <= t) k = kk;
    }
    return k;
}

template <int D>
__global__ void __launch_bounds__(NNS_WARPS * 32, MLH_NNS_MINB) k_neighbours(
    Params p, const Member *__restrict__ members, const int *__restrict__ memberOf,
    const GridInfo *__restrict__ grids, const double *__restrict__ x, const double *__restrict__ y,
    const double *__restrict__ z, const float4 *__restrict__ posf, const double *__restrict__ vx,
    const double *__restrict__ vy, const double *__restrict__ vz, const double *__restrict__ m,
    const double *__restrict__ u, const int *__restrict__ cellTotal, const int *__restrict__ cellStart,
    const int *__restrict__ cellList, uint32_t *__restrict__ nbr, double *__restrict__ rr,
    double *__restrict__ ww, int *__restrict__ noi, int *__restrict__ noiImg, int *__restrict__ faceCnt,
    Prim *__restrict__ prim, Geo *__restrict__ geo, float4 *__restrict__ velf, unsigned *__restrict__ status) {
    const int K = p.K;
    const int CAP = K + 32;
    extern __shared__ __align__(16) unsigned char nns_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    // per-warp shared areas; every sub-array starts on a 16-byte boundary
    // whatever K is (see nns_warp_bytes)
    NnsCells *cs = reinterpret_cast<NnsCells *>(nns_smem) + warp;
    unsigned char *wbase = nns_smem + nns_cells_bytes() + (size_t)warp * nns_warp_bytes(K, p.adaptive_h);
    float4 *stP = reinterpret_cast<float4 *>(wbase);                                  // staged positions
    uint32_t *stE = reinterpret_cast<uint32_t *>(wbase + (size_t)NNS_CH * 16);        // staged entries
    uint32_t *candq = stE + NNS_CH;                                                   // NNS_PB lists of CAP
    int *ncq = reinterpret_cast<int *>(wbase + (size_t)NNS_CH * 20 + nns_r16((size_t)NNS_PB * CAP * 4));
    int *offq = ncq + NNS_PB, *nrq = offq + NNS_PB, *niq = nrq + NNS_PB;
    double *imgR = reinterpret_cast<double *>(reinterpret_cast<unsigned char *>(ncq) + nns_r16((size_t)4 * NNS_PB * 4));
    double *imgW = imgR + K;
    uint32_t *imgE = reinterpret_cast<uint32_t *>(imgW + K);
    float *stH = reinterpret_cast<float *>(reinterpret_cast<unsigned char *>(imgE) + nns_r16((size_t)K * 4));   // staged h_j

    const double *X[3] = {x, y, z};
    // a binning that gave up a bounded wait left no valid cells
    if (step_aborted(status)) return;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    // omega, density, pressure, 1/omega and sound speed of particle bi (per
    // lane): omega sums the stored W of the real neighbours in list order,
    // then W(0), then the images (Particles::compDensity, Particles.cpp:
    // 1151-1184, and its image part :2262-2290, in that order)
    int bi = -1, bnr = 0, bni = 0, iter = 0;
    double bw0 = 0.;
    auto finish = [&]() {
        if (bi < 0) return;
        const double *wb = ww + (size_t)bi * K;
        double bomega = 0.;
        for (int s = 0; s < bnr; ++s) bomega += wb[s];
        bomega += bw0;
        for (int s = bnr; s < bnr + bni; ++s) bomega += wb[s];
        const double rho = m[bi] * bomega;
        const double P = (p.gamma - 1.) * rho * u[bi];
        // rho <= 0 and P <= 0 as sign tests on the bit patterns (a NaN with
        // the sign bit set also counts)
        unsigned st = 0;
        if (__double_as_longlong(rho) <= 0) st |= ST_NEG_DENSITY;
        if (__double_as_longlong(P) <= 0) st |= ST_NEG_PRESSURE;
        if (st) flag(status, st);
        Prim pr;
        pr.x = x[bi]; pr.y = y[bi]; pr.z = D == 3 ? z[bi] : 0.;
        pr.rho = rho; pr.P = P;
        pr.vx = vx[bi]; pr.vy = vy[bi]; pr.vz = D == 3 ? vz[bi] : 0.;
        prim[bi] = pr;
        geo[bi].omega = bomega;
        geo[bi].V = frcp(bomega);
        const double irho = frcp(rho);   // also the face kernel's 1/rho_i
        geo[bi].irho = irho;
        const double cs = sqrt(p.gamma * P * irho);
        geo[bi].c = cs;
        // velocity and sound speed in single precision, for the time step's
        // filter (k_gradients)
        velf[bi] = make_float4(__double2float_rn(pr.vx), __double2float_rn(pr.vy), __double2float_rn(pr.vz),
                               __double2float_rn(cs));
    };
    const int ncells = *cellTotal;
    for (int c = gw; c < ncells; c += nw) {
        const int c0 = cellStart[c], ncell = cellStart[c + 1] - c0;
        if (ncell <= 0) continue;
        const int mi = memberOf ? memberOf[cellList[c0]] : 0;   // a cell holds one member's particles
        const GridInfo g = grids[mi];
        const Member mb = members[mi];
        const int total = nns_stencil<D>(p, g, c - g.cell_base, cellStart, cs);
        for (int b0 = 0; b0 < ncell; b0 += NNS_PB) {
            const int nb = ncell - b0 < NNS_PB ? ncell - b0 : NNS_PB;
            // --- phase 1 for the batch: particle q of the batch on lane q
            int myI = -1;
            float4 myF = make_float4(0.f, 0.f, 0.f, 0.f);
            float myHf = 0.f;
            if (lane < nb) {
                myI = cellList[c0 + b0 + lane];
                myF = posf[myI];
                if (p.adaptive_h) myHf = p.hpf[myI];
            }
            if (lane < NNS_PB) ncq[lane] = 0;
            __syncwarp();
            for (int ch = 0; ch < total; ch += NNS_CH) {
                const int cl = total - ch < NNS_CH ? total - ch : NNS_CH;
                // stage candidates [ch, ch + cl) of the sequence
                for (int t = lane; t < cl; t += 32) {
                    const int k = nns_cell_of<D>(cs, ch + t);
                    const int j = cellList[cs->start[k] + (ch + t - cs->excl[k])];
                    const unsigned wr = cs->wrap[k];
                    float4 fj = posf[j];
                    if (wr) {
                        fj.x += cs->shift[k][0];
                        fj.y += cs->shift[k][1];
                        if (D == 3) fj.z += cs->shift[k][2];
                    }
                    stP[t] = fj;
                    stE[t] = (uint32_t)j | (wr << IMG_SHIFT);
                    if (p.adaptive_h) stH[t] = p.hpf[j];
                }
                __syncwarp();
                for (int q = 0; q < nb; ++q) {
                    const uint32_t iq = (uint32_t)__shfl_sync(0xffffffffu, myI, q);
                    const float fx = __shfl_sync(0xffffffffu, myF.x, q);
                    const float fy = __shfl_sync(0xffffffffu, myF.y, q);
                    const float fz = __shfl_sync(0xffffffffu, myF.z, q);
                    const float hq = __shfl_sync(0xffffffffu, myHf, q);
                    uint32_t *cq = candq + (size_t)q * CAP;
                    int nq = ncq[q];
                    for (int t0 = 0; t0 < cl; t0 += 32) {
                        const int t = t0 + lane;
                        bool pass = false;
                        uint32_t ent = 0;
                        if (t < cl) {
                            ent = stE[t];
                            if (ent != iq) {   // the particle itself (its images are candidates)
                                const float4 fj = stP[t];
                                const float dx = fj.x - fx, dy = fj.y - fy, dz = fj.z - fz;
                                const float d2f = dx * dx + dy * dy + (D == 3 ? dz * dz : 0.f);
                                // with per-particle smoothing lengths the pair needs
                                // r < max(h_i, h_j): the same bound margin on the
                                // rounded-up single-precision h
                                float lim = mb.hsq_f;
                                if (p.adaptive_h) {
                                    const float m = fmaxf(hq, stH[t]);
                                    lim = m * m * 1.001f;
                                }
                                pass = d2f <= lim;
                            }
                        }
                        const unsigned bal = __ballot_sync(0xffffffffu, pass);
                        if (pass) {
                            const int pos = nq + __popc(bal & lt_mask);
                            if (pos < CAP) cq[pos] = ent;
                        }
                        nq += __popc(bal);
                    }
                    __syncwarp();
                    if (lane == 0) ncq[q] = nq;
                    __syncwarp();
                }
            }
            // --- phase 2: exact FP64 test, r, W, over the candidate lists of
            // the batch walked as one sequence, 32 candidates at a time (about
            // 20 candidates per particle in 2D would leave a third of the lanes
            // idle per particle).  With per-particle smoothing lengths the pair
            // test is r^2 < max(h_i^2, h_j^2) and W uses h_i.  Particle q's
            // position and kernel parameters live on lane q.  Real neighbours
            // go to the front of the particle's slot row in candidate order,
            // images to its back (slot K-1-t for the t-th), from where the
            // per-particle step below sorts them behind the real ones.
            {
                const int myN = lane < nb ? (ncq[lane] < CAP ? ncq[lane] : CAP) : 0;
                int myOff = myN;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, myOff, o);
                    if (lane >= o) myOff += t;
                }
                const int seq = __shfl_sync(0xffffffffu, myOff, 31);
                myOff -= myN;
                if (lane < NNS_PB) { offq[lane] = myOff; nrq[lane] = 0; niq[lane] = 0; }
                double myX[3] = {0., 0., 0.};
                double myHsq = mb.hsq, myIh2 = mb.ih2, mySig = mb.sigma, mySig4 = 0.;
                if (lane < nb) {
#pragma unroll
                    for (int a = 0; a < D; ++a) myX[a] = X[a][myI];
                    if (p.adaptive_h) {
                        const double hi_ = p.hp[myI];
                        const double h2_i = hi_ / 2.;
                        myHsq = __dmul_rn(hi_, hi_);
                        myIh2 = 1. / h2_i;
                        mySig = kernel_sigma<D>(h2_i);
                    }
                }
                mySig4 = 0.25 * mySig;   // the outer piece's factor, once per particle (exact)
                __syncwarp();
                for (int t0 = 0; t0 < seq; t0 += 32) {
                    const int gi = t0 + lane;
                    const bool valid = gi < seq;
                    // the particle of position gi: the last one whose list starts at
                    // or before it (an empty list shares its offset with the next)
                    int q = 0;
#pragma unroll
                    for (int l = 1; l < NNS_PB; ++l)
                        if (l < nb && offq[l] <= gi) q = l;
                    const int i = __shfl_sync(0xffffffffu, myI, q);
                    double xi[3] = {0., 0., 0.};
#pragma unroll
                    for (int a = 0; a < D; ++a) xi[a] = __shfl_sync(0xffffffffu, myX[a], q);
                    const double hsq_i = __shfl_sync(0xffffffffu, myHsq, q);
                    const double ih2_i = __shfl_sync(0xffffffffu, myIh2, q);
                    const double sigma_i = __shfl_sync(0xffffffffu, mySig, q);
                    const double sigma4_i = __shfl_sync(0xffffffffu, mySig4, q);
                    bool pass = false, img = false;
                    uint32_t e = 0;
                    double r = 0., w = 0.;
                    if (valid) {
                        e = candq[(size_t)q * CAP + (gi - offq[q])];
                        const int j = (int)(e & IDX_MASK);
                        const unsigned wr = e >> IMG_SHIFT;
                        img = wr != 0;
                        double xj[3];
                        bool ok = true;
#pragma unroll
                        for (int a = 0; a < D; ++a) {
                            xj[a] = X[a][j];
                            if (wr & (1u << a)) {
                                if (in_band(xj[a], g, a)) xj[a] = image_coord(xj[a], g, a);
                                else ok = false;
                            }
                        }
                        if (ok) {
                            double ex = __dsub_rn(xj[0], xi[0]), ey = __dsub_rn(xj[1], xi[1]);
                            double d2 = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
                            if (D == 3) { double ez = __dsub_rn(xj[2], xi[2]); d2 = __dadd_rn(d2, __dmul_rn(ez, ez)); }
                            // d2, h^2 >= 0: compared as bit patterns on the integer pipe
                            double lim = mb.hsq;
                            if (p.adaptive_h) {
                                const double hj = p.hp[j];
                                const double hsq_j = __dmul_rn(hj, hj);
                                lim = __double_as_longlong(hsq_i) < __double_as_longlong(hsq_j) ? hsq_j : hsq_i;
                            }
                            pass = __double_as_longlong(d2) < __double_as_longlong(lim);
                            if (pass) {
                                r = sqrt(d2);
                                w = kernelW2(r, ih2_i, sigma_i, sigma4_i);
                            }
                        }
                    }
                    // lanes of the same particle, and their ranks among its passes
                    const unsigned grp = __match_any_sync(0xffffffffu, valid ? q : -1);
                    const unsigned balR = __ballot_sync(0xffffffffu, pass && !img) & grp;
                    const unsigned balI = __ballot_sync(0xffffffffu, pass && img) & grp;
                    const int nr0 = nrq[q], ni0 = niq[q];
                    const size_t base = (size_t)i * K;
                    if (pass && !img) {
                        const int pos = nr0 + __popc(balR & lt_mask);
                        if (pos < K) { nbr[base + pos] = e; rr[base + pos] = r; ww[base + pos] = w; }
                    }
                    if (pass && img) {
                        const int pos = ni0 + __popc(balI & lt_mask);
                        if (pos < K) { nbr[base + K - 1 - pos] = e; rr[base + K - 1 - pos] = r; ww[base + K - 1 - pos] = w; }
                    }
                    __syncwarp();
                    if (valid && (grp & lt_mask) == 0) {   // first lane of each particle's group
                        nrq[q] = nr0 + __popc(balR);
                        niq[q] = ni0 + __popc(balI);
                    }
                    __syncwarp();
                }
            }
            for (int q = 0; q < nb; ++q) {
                const int i = __shfl_sync(0xffffffffu, myI, q);
                bool overflow = ncq[q] > CAP;
                int nr = nrq[q], ni = niq[q], fc = 0;
                const size_t base = (size_t)i * K;
                double w0_i = mb.w0;
                if (p.adaptive_h) w0_i = kernel_sigma<D>(p.hp[i] / 2.);
                if (nr + ni > K || overflow) {
                    overflow = true;
                    if (nr > K) nr = K;
                    if (ni > K - nr) ni = K - nr;
                }
                // images from the back of the row, in candidate order
                for (int t = lane; t < ni; t += 32) {
                    imgE[t] = nbr[base + K - 1 - t];
                    imgR[t] = rr[base + K - 1 - t];
                    imgW[t] = ww[base + K - 1 - t];
                }
                __syncwarp();
                // --- images behind the real neighbours, ordered by parent index
                for (int t = lane; t < ni; t += 32) {
                    const uint32_t e = imgE[t];
                    const uint32_t id = e & IDX_MASK;
                    int rank = 0;
                    for (int u = 0; u < ni; ++u) rank += (imgE[u] & IDX_MASK) < id;
                    nbr[base + nr + rank] = e;
                    rr[base + nr + rank] = imgR[t];
                    ww[base + nr + rank] = imgW[t];
                }
                __syncwarp();
                // canonical faces among the stored slots (neighbour or parent > i);
                // counted from the final list so that it matches k_link exactly
                for (int t = lane; t < nr + ni; t += 32) fc += (int)(nbr[base + t] & IDX_MASK) > i;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) fc += __shfl_xor_sync(0xffffffffu, fc, o);
                if (lane == 0) {
                    if (overflow) flag(status, ST_NGB_OVERFLOW);
                    if (nr + ni == 0) flag(status, ST_NO_NEIGHBOUR);
                    noi[i] = nr;
                    noiImg[i] = ni;
                    faceCnt[i] = fc;
                }
                // the floating-point tail of every 32 particles of this warp runs
                // once on all 32 lanes (lane k keeps the k-th particle); the stored
                // slots are visible to every lane after the __syncwarp above
                if (lane == (iter & 31)) { bi = i; bnr = nr; bni = ni; bw0 = w0_i; }
                if ((iter & 31) == 31) { finish(); bi = -1; }
                ++iter;
                __syncwarp();
            }   // particles of the batch
        }   // batches of the cell
    }
    finish();
}

// ------------------------------------------------------------------ smoothing lengths

// Per-particle smoothing lengths (no counterpart in the reference, which uses
// one global kernelSize).  For particle i the support radius x in (0, H],
// H the member's kernelSize (the search radius), at which the effective
// neighbour number N(x) = V_D x^D (W(0, x) + sum_j W(r_ij, x)) equals n_ngb.
// With the cubic spline of support x, N(x) = K_D (1 + S(x)) where
// S(x) = sum_j f(2 r_ij / x) (f the spline's shape, f(0) = 1; K_D = 32/3 in
// 3D, 40/7 in 2D); S increases with x and dS/dx = G(x) / x with
// G = sum_j -f'(q) q.  The candidates within H of each particle (the
// neighbour search's stencil, pre-filter and exact test, images by the ghost
// rule) are kept in shared memory in stencil order.  Every Newton iteration
// sums f and g over them in 32 lane-strided partial sums combined by an xor
// butterfly, and the iteration is bracketed (bisection when Newton leaves the
// bracket).  The start is the previous h_i (H at first); a particle with
// N(H) < n_ngb keeps H and is counted in hstat[1]; hstat[0] counts
// iterations.  The CPU restatement performs the same operations in the same
// order and gets the same bits.
//
// One warp per cell, as the neighbour search: the cell's candidate sequence
// is staged in shared memory once and filtered for a batch of up to HS_PB of
// its particles; the warp then computes their candidate distances and runs
// their Newton iterations side by side: per iteration, the sums of each
// unfinished particle of the batch (all lanes, the order above), then the
// scalar updates of all of them at once, particle q on lane q, so that the
// divisions and tests of an update are issued once per batch instead of once
// per particle.
constexpr int HSOLVE_MAXIT = 50;
constexpr int HS_PB = 8;
// the reduce-scatter of the solve's sums maps the 2 HS_PB = 16 sums onto
// the 32 lanes (sum k on lanes 2k and 2k + 1)
static_assert(HS_PB == 8, "k_hsolve reduces exactly 16 sums per batch");

// staged chunk (NNS_CH entries and positions), HS_PB candidate lists (K + 32
// uint32) and their counts, HS_PB distance lists (K + 32 doubles) and their
// counts, each rounded up to 16 bytes
__host__ __device__ constexpr size_t hsolve_warp_bytes(int K) {
    return (size_t)NNS_CH * 20 + nns_r16((size_t)HS_PB * (K + 32) * 4) + nns_r16((size_t)HS_PB * 4) +
           (size_t)HS_PB * (K + 32) * 8 + nns_r16((size_t)HS_PB * 4);
}

// Shape of the cubic spline and its scaled derivative for the smoothing-length
// solve: q = r / (h/2) (given as r times 1 / (h/2)), f(q) with f(0) = 1 and
// g(q) = -f'(q) q; for q <= 1, f = fma(q^2, fma(0.75, q, -1.5), 1) and
// g = q^2 fma(-2.25, q, 3); for 1 < q < 2, with t = 2 - q, f = (t^2/4) t and
// g = (3 t^2/4) q; 0 beyond.  Every operation is an explicitly rounded
// intrinsic so that the CPU restatement, which performs the same operations,
// gets the same bits.  Both pieces run as the same operations with selected
// operands (f = (t^2/4) t as fma(t^2/4, t, 0), the same rounded product), so
// a warp whose candidates fall on both sides of q = 1 issues them once.
__device__ __forceinline__ void hsolve_shape_sel(double r, double ihh2, double &f, double &g) {
    const double q = __dmul_rn(r, ihh2);
    const long long qb = __double_as_longlong(q);   // q >= 0: q <= 1 and q < 2 on the bits
    const bool inner = qb <= 0x3FF0000000000000ll, in = qb < 0x4000000000000000ll;
    const double t = __dsub_rn(2., q);
    const double a = inner ? q : t;
    const double a2 = __dmul_rn(a, a);
    const double u = __fma_rn(0.75, q, -1.5);
    const double v = __fma_rn(-2.25, q, 3.);
    // a2 / 4 (exact) on the integer pipe
    const double f_ = __fma_rn(inner ? a2 : scale_down<2>(a2), inner ? u : t, inner ? 1. : 0.);
    const double g_ = __dmul_rn(inner ? a2 : __dmul_rn(0.75, a2), inner ? v : q);
    f = in ? f_ : 0.;
    g = in ? g_ : 0.;
}

template <int D>
__global__ void __launch_bounds__(NNS_WARPS * 32) k_hsolve(
    Params p, const Member *__restrict__ members, const int *__restrict__ memberOf,
    const GridInfo *__restrict__ grids, const double *__restrict__ x, const double *__restrict__ y,
    const double *__restrict__ z, const float4 *__restrict__ posf, const int *__restrict__ cellTotal,
    const int *__restrict__ cellStart, const int *__restrict__ cellList, double *__restrict__ hp,
    float *__restrict__ hpf, double *__restrict__ neff, unsigned long long *__restrict__ hstat,
    unsigned *__restrict__ status) {
    const int K = p.K;
    const int CAP = K + 32;
    extern __shared__ __align__(16) unsigned char hs_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    NnsCells *cs = reinterpret_cast<NnsCells *>(hs_smem) + warp;
    unsigned char *wbase = hs_smem + nns_cells_bytes() + (size_t)warp * hsolve_warp_bytes(K);
    float4 *stP = reinterpret_cast<float4 *>(wbase);
    uint32_t *stE = reinterpret_cast<uint32_t *>(wbase + (size_t)NNS_CH * 16);
    uint32_t *candq = stE + NNS_CH;                                                   // HS_PB lists of CAP
    unsigned char *nb0 = wbase + (size_t)NNS_CH * 20 + nns_r16((size_t)HS_PB * CAP * 4);
    int *ncq = reinterpret_cast<int *>(nb0);
    double *rlq = reinterpret_cast<double *>(nb0 + nns_r16((size_t)HS_PB * 4));       // HS_PB lists of CAP
    int *nrq = reinterpret_cast<int *>(reinterpret_cast<unsigned char *>(rlq) + (size_t)HS_PB * CAP * 8);
    constexpr double KD = D == 3 ? 32. / 3. : 40. / 7.;
    const double St = p.sngb_t;
    const double tolS = __dmul_rn(1e-12, St);
    const double *X[3] = {x, y, z};
    if (step_aborted(status)) return;   // no valid cells
    unsigned long long iters = 0, clamped = 0;   // per lane, for its particles
    bool overflow_any = false;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int ncells = *cellTotal;
    for (int c = gw; c < ncells; c += nw) {
        const int c0 = cellStart[c], ncell = cellStart[c + 1] - c0;
        if (ncell <= 0) continue;
        const int mi = memberOf ? memberOf[cellList[c0]] : 0;
        const GridInfo g = grids[mi];
        const Member mb = members[mi];
        const double H = mb.h;
        const int total = nns_stencil<D>(p, g, c - g.cell_base, cellStart, cs);
        for (int b0 = 0; b0 < ncell; b0 += HS_PB) {
            const int nb = ncell - b0 < HS_PB ? ncell - b0 : HS_PB;
            int myI = -1;
            float4 myF = make_float4(0.f, 0.f, 0.f, 0.f);
            if (lane < nb) { myI = cellList[c0 + b0 + lane]; myF = posf[myI]; }
            if (lane < HS_PB) ncq[lane] = 0;
            __syncwarp();
            // --- candidates of the batch: staged chunks, single-precision filter
            for (int ch = 0; ch < total; ch += NNS_CH) {
                const int cl = total - ch < NNS_CH ? total - ch : NNS_CH;
                for (int t = lane; t < cl; t += 32) {
                    const int k = nns_cell_of<D>(cs, ch + t);
                    const int j = cellList[cs->start[k] + (ch + t - cs->excl[k])];
                    const unsigned wr = cs->wrap[k];
                    float4 fj = posf[j];
                    if (wr) {
                        fj.x += cs->shift[k][0];
                        fj.y += cs->shift[k][1];
                        if (D == 3) fj.z += cs->shift[k][2];
                    }
                    stP[t] = fj;
                    stE[t] = (uint32_t)j | (wr << IMG_SHIFT);
                }
                __syncwarp();
                for (int q = 0; q < nb; ++q) {
                    const uint32_t iq = (uint32_t)__shfl_sync(0xffffffffu, myI, q);
                    const float fx = __shfl_sync(0xffffffffu, myF.x, q);
                    const float fy = __shfl_sync(0xffffffffu, myF.y, q);
                    const float fz = __shfl_sync(0xffffffffu, myF.z, q);
                    uint32_t *cq = candq + (size_t)q * CAP;
                    int nq = ncq[q];
                    for (int t0 = 0; t0 < cl; t0 += 32) {
                        const int t = t0 + lane;
                        bool pass = false;
                        uint32_t ent = 0;
                        if (t < cl) {
                            ent = stE[t];
                            if (ent != iq) {
                                const float4 fj = stP[t];
                                const float dx = fj.x - fx, dy = fj.y - fy, dz = fj.z - fz;
                                pass = dx * dx + dy * dy + (D == 3 ? dz * dz : 0.f) <= mb.hsq_f;
                            }
                        }
                        const unsigned bal = __ballot_sync(0xffffffffu, pass);
                        if (pass) {
                            const int pos = nq + __popc(bal & lt_mask);
                            if (pos < CAP) cq[pos] = ent;
                        }
                        nq += __popc(bal);
                    }
                    __syncwarp();
                    if (lane == 0) ncq[q] = nq;
                    __syncwarp();
                }
            }
            // --- exact FP64 distances of the candidates within H, in order
            for (int q = 0; q < nb; ++q) {
                const int i = __shfl_sync(0xffffffffu, myI, q);
                const int ncand = ncq[q];
                int nr = 0;
                if (ncand <= CAP) {
                    const uint32_t *cand = candq + (size_t)q * CAP;
                    double *rl = rlq + (size_t)q * CAP;
                    double xi[3] = {0., 0., 0.};
#pragma unroll
                    for (int a = 0; a < D; ++a) xi[a] = X[a][i];
                    for (int t0 = 0; t0 < ncand; t0 += 32) {
                        const int t = t0 + lane;
                        bool pass = false;
                        double r = 0.;
                        if (t < ncand) {
                            const uint32_t e = cand[t];
                            const int j = (int)(e & IDX_MASK);
                            const unsigned wr = e >> IMG_SHIFT;
                            double xj[3];
                            bool ok = true;
#pragma unroll
                            for (int a = 0; a < D; ++a) {
                                xj[a] = X[a][j];
                                if (wr & (1u << a)) {
                                    if (in_band(xj[a], g, a)) xj[a] = image_coord(xj[a], g, a);
                                    else ok = false;
                                }
                            }
                            if (ok) {
                                double ex = __dsub_rn(xj[0], xi[0]), ey = __dsub_rn(xj[1], xi[1]);
                                double d2 = __dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey));
                                if (D == 3) { double ez = __dsub_rn(xj[2], xi[2]); d2 = __dadd_rn(d2, __dmul_rn(ez, ez)); }
                                pass = __double_as_longlong(d2) < __double_as_longlong(mb.hsq);   // d2 < H^2, both >= 0
                                if (pass) r = __dsqrt_rn(d2);
                            }
                        }
                        const unsigned bal = __ballot_sync(0xffffffffu, pass);
                        if (pass) rl[nr + __popc(bal & lt_mask)] = r;
                        nr += __popc(bal);
                    }
                } else {
                    nr = -1;   // overflow: the host grows the slots and repeats
                }
                if (lane == 0) nrq[q] = nr;
                __syncwarp();
            }
            // --- bracketed Newton on S(x) = St, particle q's state on lane q
            const int mynr = lane < nb ? nrq[lane] : -1;
            if (lane < nb && mynr < 0) overflow_any = true;
            bool done = !(lane < nb) || mynr < 0;
            double xh = H, lo = 0., hi = H, S = 0., sfq = 0., sgq = 0.;
            bool upper = false;
            int it = 0;
            if (!done) {
                xh = hp[myI];
                if (!(xh > 0. && xh <= H)) xh = H;
            }
            for (;;) {
                const unsigned act = __ballot_sync(0xffffffffu, !done);
                if (!act) break;
                const double ihh2 = __ddiv_rn(1., __dmul_rn(0.5, xh));
                // 32 lane-strided partial sums of f and g per unfinished
                // particle: v[2q], v[2q + 1]
                double v[2 * HS_PB];
#pragma unroll
                for (int q = 0; q < HS_PB; ++q) {
                    v[2 * q] = 0.;
                    v[2 * q + 1] = 0.;
                    if (act & (1u << q)) {
                        const double ihq = __shfl_sync(0xffffffffu, ihh2, q);
                        const int nrq_ = __shfl_sync(0xffffffffu, mynr, q);
                        const double *rl = rlq + (size_t)q * CAP;
                        for (int t = lane; t < nrq_; t += 32) {
                            double f, gg;
                            hsolve_shape_sel(rl[t], ihq, f, gg);
                            v[2 * q] = __dadd_rn(v[2 * q], f);
                            v[2 * q + 1] = __dadd_rn(v[2 * q + 1], gg);
                        }
                    }
                }
                // reduce-scatter of the 16 partial sums: at distance d = 16,
                // 8, 4, 2 each lane keeps half of its values and adds its
                // partner's (own + partner, the pairs of an xor butterfly, so
                // every sum has the butterfly's tree and bits), then d = 1;
                // sum k ends on lanes 2k and 2k + 1
#pragma unroll
                for (int d = 16, m = HS_PB; d > 1; d >>= 1, m >>= 1) {
                    const bool upper = (lane & d) != 0;
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        if (j < m) {
                            const double send = upper ? v[j] : v[j + m];
                            const double keep = upper ? v[j + m] : v[j];
                            v[j] = __dadd_rn(keep, __shfl_xor_sync(0xffffffffu, send, d));
                        }
                    }
                }
                v[0] = __dadd_rn(v[0], __shfl_xor_sync(0xffffffffu, v[0], 1));
                // particle q (lane q) takes sum 2q (lane 4q) and 2q + 1 (lane 4q + 2)
                sfq = __shfl_sync(0xffffffffu, v[0], (4 * lane) & 31);
                sgq = __shfl_sync(0xffffffffu, v[0], (4 * lane + 2) & 31);
                if (!done) {
                    S = sfq;
                    const double G = sgq;
                    ++iters;
                    const double F = __dsub_rn(S, St);
                    if (fabs(F) <= tolS) done = true;
                    else if (F < 0. && xh >= H) { ++clamped; done = true; }
                    else if (it + 1 >= HSOLVE_MAXIT) done = true;
                    else {
                        if (F > 0.) { hi = xh; upper = true; }
                        else lo = xh;
                        double xn = G > 0. ? __dsub_rn(xh, __ddiv_rn(__dmul_rn(F, xh), G))
                                           : __dmul_rn(0.5, __dadd_rn(lo, hi));
                        if (!(xn > lo && xn < hi)) xn = (!upper && xn >= hi) ? H : __dmul_rn(0.5, __dadd_rn(lo, hi));
                        if (xn == xh) done = true;
                        else xh = xn;
                    }
                    ++it;
                }
            }
            if (lane < nb && mynr >= 0) {
                hp[myI] = xh;
                hpf[myI] = __double2float_ru(xh);
                if (neff) neff[myI] = __dmul_rn(KD, __dadd_rn(S, 1.));
            }
            __syncwarp();
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        iters += __shfl_xor_sync(0xffffffffu, iters, o);
        clamped += __shfl_xor_sync(0xffffffffu, clamped, o);
    }
    const bool of = __any_sync(0xffffffffu, overflow_any);
    if (lane == 0) {
        if (iters) atomicAdd(hstat, iters);
        if (clamped) atomicAdd(hstat + 1, clamped);
        if (of) flag(status, ST_NGB_OVERFLOW);
    }
}

size_t hsolve_smem_bytes(int K) {
    return nns_cells_bytes() + (size_t)NNS_WARPS * hsolve_warp_bytes(K);
}

size_t nns_smem_bytes(int K, bool adaptive) {
    return nns_cells_bytes() + (size_t)NNS_WARPS * nns_warp_bytes(K, adaptive);
}

// ------------------------------------------------------------------ dt

// Particles::compGlobalTimestep (Particles.cpp:1446-1485): real neighbours
// only, v_sig starting at numeric_limits<double>::min().  The minimum over
// particles is order independent, so an atomicMin on the bit pattern of the
// (positive) per-particle dt is deterministic.
template <int D>
__global__ void __launch_bounds__(256) k_timestep(Params p, const Member *__restrict__ members,
                                                  const int *__restrict__ memberOf, const Prim *__restrict__ prim,
                                                  const Geo *__restrict__ geo, const uint32_t *__restrict__ nbr,
                                                  const double *__restrict__ rr, const int *__restrict__ noi,
                                                  unsigned long long *__restrict__ dtbits,
                                                  const float *__restrict__ dtlo, const unsigned *__restrict__ dtcap) {
    const int lane = threadIdx.x & 31;
    // warp-uniform loop: every lane takes part in the reductions below
    for (int i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; i0 < p.n; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + lane;
        int mi = -1;
        double dti = DBL_MAX_;
        // with dtlo (the single-precision filter of k_gradients): only the
        // particles whose lower bound on dt reaches their simulation's least
        // upper bound can hold the minimum (the others leave dti at DBL_MAX;
        // every lane stays in the loop for the warp's reduction)
        bool cand = i < p.n;
        if (cand && dtlo) {
            const int m = memberOf ? memberOf[i] : 0;
            cand = dtlo[i] <= __uint_as_float(dtcap[m]);
        }
        if (cand) {
            mi = memberOf ? memberOf[i] : 0;
            const Prim pi = prim[i];
            const double ci = geo[i].c;
            double vSig = DBL_MIN_;
            const size_t base = (size_t)i * p.K;
            const int nr = noi[i];
            for (int s = 0; s < nr; ++s) {
                const int j = (int)(nbr[base + s] & IDX_MASK);
                const Prim pj = prim[j];
                const double cj = geo[j].c;
                double xij[3] = {pi.x - pj.x, pi.y - pj.y, pi.z - pj.z};
                double vij[3] = {pi.vx - pj.vx, pi.vy - pj.vy, pi.vz - pj.vz};
                // c_i + c_j - min(0, v_ij . x_ij / r) as one fused multiply-add:
                // 1/r only when the dot product is negative, 0 otherwise
                const double dv = dotD<D>(vij, xij);
                const double ir = dneg(dv) ? frcp(rr[base + s]) : 0.;
                const double vs = fma(-dv, ir, ci + cj);
                vSig = dlt(vSig, vs) ? vs : vSig;
            }
            dti = (p.adaptive_h ? p.cfl * p.hp[i] : members[mi].cfl_h) / vSig;
        }
        // the minimum over particles does not depend on the order of the
        // atomicMin calls: a warp inside one simulation (the common case)
        // reduces first and issues one atomic; a warp that straddles two
        // simulations issues one per lane
        const int m0 = __shfl_sync(0xffffffffu, mi, 0);
        if (__all_sync(0xffffffffu, mi == m0)) {
            double best = dti;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
            if (lane == 0 && m0 >= 0 && best < DBL_MAX_) atomic_min_pos_double(dtbits + m0, best);
        } else if (mi >= 0 && dti < DBL_MAX_) {
            atomic_min_pos_double(dtbits + mi, dti);
        }
    }
}

__global__ void k_dt_final(Params p, int nmembers, const unsigned long long *__restrict__ dtbits, double dt_max,
                           double *__restrict__ dt_out) {
    for (int mi = blockIdx.x * blockDim.x + threadIdx.x; mi < nmembers; mi += gridDim.x * blockDim.x) {
        double dt = p.adaptive ? __longlong_as_double((long long)dtbits[mi]) : p.time_step;
        if (dt_max > 0. && dt > dt_max) dt = dt_max;
        dt_out[mi] = dt;
    }
}

// ------------------------------------------------------------------ face links

// Canonical faces: slot s of particle i with neighbour (or image parent)
// j > i, the side on which Particles::solveRiemannProblems computes the flux
// (Particles.cpp:1838-1858, 1886-1897).  Slot -> face id (+1 canonical, -1
// copied with the opposite sign), face -> (i, slot, reverse slot).  The
// reverse slot of a non-canonical slot is the first entry of j's list (real
// part or image part) that refers to i, as in the reference's searches.
// The face links of particle i (see k_link).
__device__ __forceinline__ void link_particle(int i, const Params &p, const uint32_t *__restrict__ nbr,
                                              const int *__restrict__ noi, const int *__restrict__ noiImg,
                                              const int *__restrict__ faceOff, int *__restrict__ faceOf,
                                              FaceRef *__restrict__ faces, unsigned *__restrict__ status) {
    const size_t base = (size_t)i * p.K;
    const int nr = noi[i], tot = nr + noiImg[i];
    const uint4 *own = reinterpret_cast<const uint4 *>(nbr + base);
    int rank = 0;
    for (int s0 = 0; s0 < tot; s0 += 4) {
        const uint4 q = own[s0 >> 2];
        const uint32_t ev[4] = {q.x, q.y, q.z, q.w};
        // per search: j, the length of j's list, the current 4-entry chunk,
        // the canonical count and flags.  i is sought among j's real
        // entries (no image bits) or among its images (image bits set), so
        // an entry's own bits say whether it lies in the searched part.
        constexpr unsigned ACT = 1u, BWD = 2u, IMG = 4u, FOUND = 8u;
        int jj[4], jt[4], cur[4], cnt[4];
        unsigned fl[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int s = s0 + k;
            const int j = (int)(ev[k] & IDX_MASK);
            jj[k] = j; jt[k] = 0; cur[k] = 0; cnt[k] = 0; fl[k] = 0u;
            if (s >= tot) continue;
            if (j > i) {
                const int fid = faceOff[i] + rank;
                ++rank;
                if (fid >= p.faces_cap) { flag(status, ST_CAPACITY); faceOf[base + s] = 0; continue; }
                faceOf[base + s] = fid + 1;
                faces[fid].i = i;
                faces[fid].slot = s;
                continue;
            }
            jt[k] = noi[j] + noiImg[j];
            const bool img = s >= nr;
            // a particle that is its own image searches forward
            const bool bwd = (img || 2 * s < nr) && j != i;
            cur[k] = bwd ? (jt[k] - 1) >> 2 : 0;
            fl[k] = ACT | (bwd ? BWD : 0u) | (img ? IMG : 0u);
        }
        for (;;) {
            uint4 r[4];
            bool any = false;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                // past either end of j's list: not found
                if ((fl[k] & BWD) ? cur[k] < 0 : cur[k] * 4 >= jt[k]) fl[k] &= ~ACT;
                r[k] = (fl[k] & ACT) ? reinterpret_cast<const uint4 *>(nbr + (size_t)jj[k] * p.K)[cur[k]]
                                     : make_uint4(0u, 0u, 0u, 0u);
                any |= (fl[k] & ACT) != 0u;
            }
            if (!any) break;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if (!(fl[k] & ACT)) continue;
                const bool bwd = (fl[k] & BWD) != 0u, img = (fl[k] & IMG) != 0u;
                const uint32_t v[4] = {r[k].x, r[k].y, r[k].z, r[k].w};
#pragma unroll
                for (int mm = 0; mm < 4; ++mm) {
                    const int m = bwd ? 3 - mm : mm;
                    const int t = cur[k] * 4 + m;
                    const uint32_t e = v[m];
                    const int idx = (int)(e & IDX_MASK);
                    if (!(fl[k] & FOUND) && t < jt[k]) {
                        if (idx == i && ((e >> IMG_SHIFT) != 0u) == img) fl[k] |= FOUND;
                        else cnt[k] += idx > jj[k];
                    }
                }
                if (fl[k] & FOUND) fl[k] &= ~ACT;
                else cur[k] += bwd ? -1 : 1;
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int s = s0 + k;
            if (s >= tot || jj[k] > i) continue;
            if (!(fl[k] & FOUND)) { flag(status, ST_ASYMMETRIC); faceOf[base + s] = 0; continue; }
            const int fid = (fl[k] & BWD) ? faceOff[jj[k] + 1] - 1 - cnt[k] : faceOff[jj[k]] + cnt[k];
            if (fid >= p.faces_cap) { flag(status, ST_CAPACITY); faceOf[base + s] = 0; continue; }
            faceOf[base + s] = -(fid + 1);
            faces[fid].rslot = s;
        }
    }
}

__global__ void __launch_bounds__(256) k_link(Params p, const uint32_t *__restrict__ nbr, const int *__restrict__ noi,
                                              const int *__restrict__ noiImg, const int *__restrict__ faceOff,
                                              int *__restrict__ faceOf, FaceRef *__restrict__ faces,
                                              unsigned *__restrict__ status) {
    // faces[] was set to -1: the owner writes (i, slot), the slot on the other
    // side writes rslot, so each field has exactly one writer.  A slot with
    // j > i owns face faceOff[i] + (its rank among i's canonical slots).  A
    // slot with j < i finds i in j's list (real part or image part) and the
    // face's rank in j's list from j's canonical entries (index > j) on one
    // side of it: searching forward, the rank is the count before i; searching
    // backward from the end of j's list, it is faceCnt[j] - 1 - the count
    // after i, faceCnt[j] = faceOff[j + 1] - faceOff[j] being the number of
    // canonical entries of j's list.  The stencils of i and j mirror each
    // other, so j early in i's list puts i late in j's list: those searches
    // and the image searches (images sit at the end of the list) go backward.
    // The own list is read four slots per load (K is a multiple of 4) and the
    // searches of those four slots advance together, one 4-entry load of each
    // list per round, so that a thread has up to four loads in flight.
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x)
        link_particle(i, p, nbr, noi, noiImg, faceOff, faceOf, faces, status);
}

// ------------------------------------------------------------------ gradients

// Particles::compPsijTilde (Particles.cpp:1186-1254, 2292-2455): E_i =
// sum_j (x_j - x_i)(x_j - x_i)^T W_ij / omega_i, B_i = E_i^-1 (closed form);
// Particles::gradient (:1257-1270, 2457-2502) for rho, vx, vy, (vz), P with
// psi~_j(x_i) = B_i (x_j - x_i) W_ij / omega_i; Particles::slopeLimiter
// (:1313-1444) with the face midpoint x_ij = (x_i + x_j)/2.
template <int D>
__device__ __forceinline__ void neighbour_pos(uint32_t e, const Prim &pj, const GridInfo &g, double *xj) {
    xj[0] = pj.x; xj[1] = pj.y; if (D == 3) xj[2] = pj.z;
    if (e >> IMG_SHIFT) {
#pragma unroll
        for (int a = 0; a < D; ++a)
            if (e & (1u << (IMG_SHIFT + a))) xj[a] = image_coord(xj[a], g, a);
    }
}

template <int D>
__device__ __forceinline__ void invert_closed_form(double *A) {
    if (D == 2) {
        double a = A[0], b = A[1], c = A[2], d = A[3];
        double det = a * d - b * c;
        double id = 1. / det;
        A[0] = d * id; A[1] = -b * id; A[2] = -c * id; A[3] = a * id;
    } else {
        double a00 = A[0], a01 = A[1], a02 = A[2], a10 = A[3], a11 = A[4], a12 = A[5], a20 = A[6], a21 = A[7], a22 = A[8];
        double c00 = a11 * a22 - a12 * a21;
        double c01 = a12 * a20 - a10 * a22;
        double c02 = a10 * a21 - a11 * a20;
        double det = a00 * c00 + a01 * c01 + a02 * c02;
        double id = 1. / det;
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

template <int D>
__device__ __forceinline__ double field_of(const Prim &q, int f) {
    // gradient order of MeshlessScheme.cpp:114-120: rho, vx, vy, (vz), P
    if (f == 0) return q.rho;
    if (f == 1) return q.vx;
    if (f == 2) return q.vy;
    if (D == 3 && f == 3) return q.vz;
    return q.P;
}

//
// With dtbits (adaptive time step), the first pass over the neighbours also
// runs Particles::compGlobalTimestep (Particles.cpp:1446-1485) for the
// particle, as k_timestep does (real neighbours only, v_sig from
// numeric_limits<double>::min(), the same expressions), on the positions and
// velocities that pass loads anyway; the per-particle dt goes into the
// per-member minimum (warp reduction, then one atomicMin on its bit pattern).
// Register caps of the gradients kernel, per dimension.  It waits on
// dependent gathers as much as on the FP64 pipe (Sedov 64^3: FP64 pipe 73 %
// active, 17 % of the warp slots occupied at 146 registers), so warps per SM
// matter: in 3D 128 registers (16 warps per SM, a small spill) took the Sedov
// 128^3 gradients from 11.1-11.4 to 10.1 ms (112: 10.4, 120: +0.2 ms, 136:
// +0.5 ms); in 2D (the KH ensemble, 110 registers uncapped) 96 registers
// gave 7.19 ms against 7.45 at 104 and 7.59 at 128.  Blocks of up to 256
// threads.
#ifndef MLH_GRAD_MAXREG
#define MLH_GRAD_MAXREG 128
#endif
#ifndef MLH_GRAD_MAXREG_2D
#define MLH_GRAD_MAXREG_2D 96
#endif
#define MLH_GRAD_BOUNDS __maxnreg__(D == 3 ? MLH_GRAD_MAXREG : MLH_GRAD_MAXREG_2D)
template <int D>
__global__ void MLH_GRAD_BOUNDS k_gradients(Params p, const Member *__restrict__ members,
                                                   const int *__restrict__ memberOf, const GridInfo *__restrict__ grids,
                                                   const Prim *__restrict__ prim, Geo *__restrict__ geo,
                                                   const uint32_t *__restrict__ nbr, const double *__restrict__ ww,
                                                   const double *__restrict__ rr,
                                                   const int *__restrict__ noi, const int *__restrict__ noiImg,
                                                   Grad *__restrict__ grad, Grad *__restrict__ gradRaw,
                                                   double *__restrict__ psiOut,
                                                   unsigned long long *__restrict__ dtbits,
                                                   const int *__restrict__ faceOff, int *__restrict__ faceOf,
                                                   FaceRef *__restrict__ faces, unsigned *__restrict__ status,
                                                   const float4 *__restrict__ posf, int fp32_filters,
                                                   const float4 *__restrict__ velf, float *__restrict__ dtlo,
                                                   unsigned *__restrict__ dtcap) {
    constexpr int NF = D + 2;
    const int lane = threadIdx.x & 31;
    // warp-uniform loop: every lane takes part in the time-step reduction
    for (int i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31; i0 < p.n; i0 += gridDim.x * blockDim.x) {
      const int i = i0 + lane;
      int mi = -1;
      double dti = DBL_MAX_;
      float dthi = FLT_INF_;   // with dtlo: upper bound on the particle's dt
      if (i < p.n) {
        // with faceOff, the particle's face links first (link_particle):
        // integer searches whose load latency the other warps' FP64 work
        // hides, and whose registers are free again before the passes below
        if (faceOff) link_particle(i, p, nbr, noi, noiImg, faceOff, faceOf, faces, status);
        mi = memberOf ? memberOf[i] : 0;
        const GridInfo g = grids[mi];
        const double h = members[mi].h;
        const double hq = p.adaptive_h ? p.hp[i] : h;   // quadrature-point radius
        const Prim pi = prim[i];
        const double xi[3] = {pi.x, pi.y, pi.z};
        const size_t base = (size_t)i * p.K;
        const int nr = noi[i];
        const int tot = nr + noiImg[i];
        const bool want_dt = dtbits != nullptr;
        const double ci = want_dt ? geo[i].c : 0.;
        double vSig = DBL_MIN_;
        // the time step's single-precision filter (dtlo): bounds on v_sig
        // = max_j (c_i + c_j - min(0, v_ij . x_ij / r_ij)) over the real
        // neighbours from the packed positions, velocities and sound speeds
        const bool want_dtf = dtlo != nullptr;
        float4 vif = make_float4(0.f, 0.f, 0.f, 0.f), xif4 = make_float4(0.f, 0.f, 0.f, 0.f);
        float vlo = 0.f, vhi = 0.f, xbf = 0.f;
        bool dt_exact = false;   // no usable bound: the particle is always a candidate
        if (want_dtf) {
            vif = velf[i];
            xif4 = posf[i];
            double xb = 0.;
#pragma unroll
            for (int a = 0; a < D; ++a) xb = fmax(xb, fmax(fabs(g.lo[a]), fabs(g.hi[a])));
            xbf = __double2float_ru(xb);
        }
        // E_i = V_i E' with E' = sum_j (x_j - x_i)(x_j - x_i)^T W_ij, so that
        // psi~_j(x_i) = E_i^-1 (x_j - x_i) W_ij V_i = E'^-1 (x_j - x_i) W_ij:
        // V_i cancels and neither pass multiplies by it
        double E[9] = {0., 0., 0., 0., 0., 0., 0., 0., 0.};
        for (int s = 0; s < tot; ++s) {
            const uint32_t e = nbr[base + s];
            const Prim pj = prim[e & IDX_MASK];
            double xj[3];
            neighbour_pos<D>(e, pj, g, xj);
            const double wij = ww[base + s];
            double d[3], dp[3];
#pragma unroll
            for (int a = 0; a < D; ++a) { d[a] = xj[a] - xi[a]; dp[a] = d[a] * wij; }
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b = a; b < D; ++b) E[D * a + b] = fma(d[a], dp[b], E[D * a + b]);
            if (want_dt && s < nr) {
                // v_sig = c_i + c_j - min(0, v_ij . x_ij / r) as one fused
                // multiply-add (1/r only when the dot product is negative);
                // x_ij = x_i - x_j is the exact negation of d
                const double cj = geo[e & IDX_MASK].c;
                const double xij[3] = {-d[0], -d[1], D == 3 ? -d[2] : 0.};
                const double vij[3] = {pi.vx - pj.vx, pi.vy - pj.vy, pi.vz - pj.vz};
                const double dv = dotD<D>(vij, xij);
                const double ir = dneg(dv) ? frcp(rr[base + s]) : 0.;
                const double vs = fma(-dv, ir, ci + cj);
                vSig = dlt(vSig, vs) ? vs : vSig;
            }
            if (want_dtf && s < nr) {
                // |vs - vs64| <= B: the inputs' roundings (eps |c|, eps |v|,
                // 3 eps X on each coordinate difference), the estimate's own
                // and the FP64 expression's, at most eps (2 (c_i + c_j) +
                // 2 vs + V (7 X / r + 8)) with V = |v_i|_1 + |v_j|_1; B is
                // twice that
                const int j = (int)(e & IDX_MASK);
                const float4 vj = velf[j], xj4 = posf[j];
                const float dx = __fsub_rn(xj4.x, xif4.x), dy = __fsub_rn(xj4.y, xif4.y),
                            dz = D == 3 ? __fsub_rn(xj4.z, xif4.z) : 0.f;
                const float wx = __fsub_rn(vif.x, vj.x), wy = __fsub_rn(vif.y, vj.y),
                            wz = D == 3 ? __fsub_rn(vif.z, vj.z) : 0.f;
                const float dvd = __fmaf_rn(wz, dz, __fmaf_rn(wy, dy, __fmul_rn(wx, dx)));   // v_ij . (x_j - x_i)
                const float r = __fsqrt_rn(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx))));
                // -min(0, v_ij . x_ij / r) with x_ij = -(x_j - x_i)
                const float T = dvd > 0.f ? __fdiv_rn(dvd, r) : 0.f;
                const float vs = __fadd_rn(__fadd_rn(vif.w, vj.w), T);
                const float V = fabsf(vif.x) + fabsf(vif.y) + fabsf(vif.z) + fabsf(vj.x) + fabsf(vj.y) + fabsf(vj.z);
                constexpr float EPS32 = 5.9604645e-8f;
                const float B = 2.f * EPS32 * (2.f * (vif.w + vj.w) + 2.f * vs + V * (7.f * __fdiv_ru(xbf, r) + 8.f));
                dt_exact = dt_exact || !(r > 0.f) || !(B < 1e30f);
                vlo = fmaxf(vlo, vs - B);
                vhi = fmaxf(vhi, vs + B);
            }
        }
        if (want_dt) dti = (p.adaptive_h ? p.cfl * p.hp[i] : members[mi].cfl_h) / vSig;
        if (want_dtf) {
            // dt = cfl_h / v_sig bounded below by the largest v_sig and above by
            // the smallest (rounded outward, with the FP64 quotient's and the
            // conversion's roundings); v_sig >= DBL_MIN when nothing is found
            const float ch = __double2float_rn(p.adaptive_h ? p.cfl * p.hp[i] : members[mi].cfl_h);
            constexpr float EPS32 = 5.9604645e-8f;
            float lo = 0.f;
            if (!dt_exact && nr > 0 && vhi > 0.f && vhi < FLT_INF_)
                lo = __fmul_rd(__fdiv_rd(ch, vhi), 1.f - 4.f * EPS32);
            if (!(lo < 1e38f)) lo = 0.f;   // below any cap
            if (!dt_exact && nr > 0 && vlo > 0.f)
                dthi = __fmul_ru(__fdiv_ru(ch, vlo), 1.f + 4.f * EPS32);
            dtlo[i] = dt_exact ? 0.f : lo;
            if (dt_exact) dthi = FLT_INF_;
        }
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = 0; b < a; ++b) E[D * a + b] = E[D * b + a];
        invert_closed_form<D>(E);
        double gr[NF][3];
        double fi[NF];
#pragma unroll
        for (int f = 0; f < NF; ++f) { fi[f] = field_of<D>(pi, f); gr[f][0] = gr[f][1] = gr[f][2] = 0.; }
        for (int s = 0; s < tot; ++s) {
            const uint32_t e = nbr[base + s];
            const Prim pj = prim[e & IDX_MASK];
            double xj[3];
            neighbour_pos<D>(e, pj, g, xj);
            const double wij = ww[base + s];
            double d[3], ps[3];
#pragma unroll
            for (int a = 0; a < D; ++a) d[a] = xj[a] - xi[a];
#pragma unroll
            for (int a = 0; a < D; ++a) {
                double t = E[D * a] * d[0];
#pragma unroll
                for (int b = 1; b < D; ++b) t = fma(E[D * a + b], d[b], t);
                ps[a] = t * wij;
            }
            // psi~_j(x_i) of this slot, reused by the face kernel for A_ij
            double *po = psiOut + (base + s) * 3;
#pragma unroll
            for (int a = 0; a < D; ++a) po[a] = ps[a];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const double df = field_of<D>(pj, f) - fi[f];
#pragma unroll
                for (int a = 0; a < D; ++a) gr[f][a] += df * ps[a];
            }
        }
        if (gradRaw) {
            Grad graw;
            for (int k = 0; k < 16; ++k) graw.g[k] = 0.;
            for (int k = 0; k < 8; ++k) graw.t[k] = 0.;
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                int slot = (f == NF - 1) ? 4 : f;
#pragma unroll
                for (int a = 0; a < D; ++a) graw.g[slot * 3 + a] = gr[f][a];
            }
            gradRaw[i] = graw;
        }
        // B_i = E_i^-1 = E'^-1 / V_i = E'^-1 omega_i (kept for inspection; E
        // is not needed after the gradient pass)
        {
            const double omega_i = geo[i].omega;
#pragma unroll
            for (int k = 0; k < D * D; ++k) geo[i].B[k] = E[k] * omega_i;
        }
        if (p.slope) {
            // running extrema as integer keys (ord_key): the comparisons of
            // the reference's if (max < f) max = f stay off the FP64 pipe
            long long mxN[NF], mnN[NF], mxM[NF], mnM[NF];
            const long long kmin = ord_key(DBL_MIN_), kmax = ord_key(DBL_MAX_);
#pragma unroll
            for (int f = 0; f < NF; ++f) { mxN[f] = kmin; mnN[f] = kmax; mxM[f] = kmin; mnM[f] = kmax; }
            // face point x_ij = x_i + c (x_j - x_i): c = 1/2 (first-order
            // quadrature point) or h/4 (the reference's other choice);
            // f_ij = f_i + grad f . (x_ij - x_i) as one FMA chain from f_i, with
            // the gradients scaled by c for the pass instead of every offset
            // (for c = 1/2 both the scaling and its undoing are exact)
            const double cq = p.foqp ? .5 : hq / 4.;
            const double icq = p.foqp ? 2. : 1. / cq;
            if (p.foqp) {   // the halving and doubling on the integer pipe
#pragma unroll
                for (int f = 0; f < NF; ++f)
#pragma unroll
                    for (int a = 0; a < D; ++a) gr[f][a] = half_of(gr[f][a]);
            } else {
#pragma unroll
                for (int f = 0; f < NF; ++f)
#pragma unroll
                    for (int a = 0; a < D; ++a) gr[f][a] *= cq;
            }
            // one neighbour's f_ij of every field, into the extrema
            auto exact_slot = [&](int s) {
                const uint32_t e = nbr[base + s];
                const Prim pj = prim[e & IDX_MASK];
                double xj[3], d[3];
                neighbour_pos<D>(e, pj, g, xj);
#pragma unroll
                for (int a = 0; a < D; ++a) d[a] = xj[a] - xi[a];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    double fij = fma(gr[f][0], d[0], fi[f]);
#pragma unroll
                    for (int a = 1; a < D; ++a) fij = fma(gr[f][a], d[a], fij);
                    const long long kij = ord_key(fij);
                    if (mxM[f] < kij) mxM[f] = kij;
                    if (mnM[f] > kij) mnM[f] = kij;
                }
            };
            if (!(fp32_filters & MLH_FILTER_SLOPE)) {
                for (int s = 0; s < tot; ++s) {
                    const Prim pj = prim[nbr[base + s] & IDX_MASK];
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        const long long kj = ord_key(field_of<D>(pj, f));
                        if (mxN[f] < kj) mxN[f] = kj;
                        if (mnN[f] > kj) mnN[f] = kj;
                    }
                    exact_slot(s);
                }
            } else {
                // Single-precision filter (the FP64 pipe is the step's
                // bound; the FP32 pipe is 64 times wider).  The increment
                // q_j = (c grad f) . (x_j - x_i) is estimated in single
                // precision from the packed positions; |f_ij - (f_i + q_j)|
                // <= B_f for every neighbour, B_f bounding the estimate's
                // rounding (positions, gradients, the chain) and the FP64
                // chain's own.  The neighbour with the largest f_ij then has
                // q_j >= max_k q_k - 2 B_f (and the smallest q_j <= min_k q_k
                // + 2 B_f), so the FP64 chain runs only over the neighbours
                // inside those windows (a handful; every lane of a warp walks
                // its own list): the same extrema, bit for bit.  A field whose
                // gradient is zero has f_ij = f_i at every neighbour.
                float gf[NF][3], xif[3];
#pragma unroll
                for (int f = 0; f < NF; ++f)
#pragma unroll
                    for (int a = 0; a < 3; ++a) gf[f][a] = a < D ? __double2float_rn(gr[f][a]) : 0.f;
#pragma unroll
                for (int a = 0; a < 3; ++a) xif[a] = a < D ? __double2float_rn(xi[a]) : 0.f;
                // bound on |coordinate| of any neighbour or image: the box (the
                // grid spans every particle) and one box length for images
                double xb = 0.;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    const double ext = fmax(fabs(g.lo[a]), fabs(g.hi[a])) + (p.periodic ? g.hi[a] - g.lo[a] : 0.);
                    xb = fmax(xb, ext);
                }
                // x_j - x_i in single precision: the packed position, or the
                // image coordinate (double) rounded once
                auto offset_f = [&](uint32_t e, const Prim *pjp, float *d) {
                    const int j = (int)(e & IDX_MASK);
                    float xj[3];
                    if (e >> IMG_SHIFT) {
                        const Prim pj = pjp ? *pjp : prim[j];
                        double xd[3];
                        neighbour_pos<D>(e, pj, g, xd);
#pragma unroll
                        for (int a = 0; a < 3; ++a) xj[a] = a < D ? __double2float_rn(xd[a]) : 0.f;
                    } else {
                        const float4 q = posf[j];
                        xj[0] = q.x; xj[1] = q.y; xj[2] = q.z;
                    }
#pragma unroll
                    for (int a = 0; a < 3; ++a) d[a] = a < D ? __fsub_rn(xj[a], xif[a]) : 0.f;
                };
                auto incr = [&](int f, const float *d) {
                    float q = __fmul_rn(gf[f][0], d[0]);
#pragma unroll
                    for (int a = 1; a < D; ++a) q = __fmaf_rn(gf[f][a], d[a], q);
                    return q;
                };
                float hiQ[NF], loQ[NF], dmax = 0.f;
#pragma unroll
                for (int f = 0; f < NF; ++f) { hiQ[f] = -FLT_MAX_; loQ[f] = FLT_MAX_; }
                for (int s = 0; s < tot; ++s) {
                    const uint32_t e = nbr[base + s];
                    const Prim pj = prim[e & IDX_MASK];
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        const long long kj = ord_key(field_of<D>(pj, f));
                        if (mxN[f] < kj) mxN[f] = kj;
                        if (mnN[f] > kj) mnN[f] = kj;
                    }
                    float d[3];
                    offset_f(e, &pj, d);
#pragma unroll
                    for (int a = 0; a < D; ++a) dmax = fmaxf(dmax, fabsf(d[a]));
#pragma unroll
                    for (int f = 0; f < NF; ++f) {
                        const float q = incr(f, d);
                        hiQ[f] = fmaxf(hiQ[f], q);
                        loQ[f] = fminf(loQ[f], q);
                    }
                }
                // B_f = 12 eps32 S R + 12 u64 (|f_i| + S R) with S = sum |c grad f|
                // and R = max|x| + max|x_j - x_i|: twice the sum of the
                // single-precision error, at most (6 |x|max + 5 |d|max) eps32 S,
                // and the FP64 chain's, at most 4 u64 (|f_i| + S (|d|max + eps |x|max))
                constexpr float EPS32 = 5.9604645e-8f, U64 = 1.1102230e-16f;
                const float R = __double2float_ru(xb) + dmax;
                float thHi[NF], thLo[NF];
                bool ok = true, flat[NF];
#pragma unroll
                for (int f = 0; f < NF; ++f) {
                    bool z = true;
                    float S = 0.f;
#pragma unroll
                    for (int a = 0; a < D; ++a) {
                        z = z && (__double_as_longlong(gr[f][a]) & 0x7FFFFFFFFFFFFFFFll) == 0;
                        S += fabsf(gf[f][a]);
                    }
                    flat[f] = z;
                    const float fa = fabsf(__double2float_rn(fi[f]));
                    const float SR = S * R;
                    ok = ok && SR < 1e36f && fa < 1e36f;   // false for NaN and infinity
                    const float B = 12.f * EPS32 * SR + 12.f * U64 * (fa + SR) + 1e-36f;
                    thHi[f] = z ? FLT_INF_ : hiQ[f] - 2.f * B;
                    thLo[f] = z ? -FLT_INF_ : loQ[f] + 2.f * B;
                }
                const int t64 = tot < 64 ? tot : 64;
                unsigned long long cand = t64 == 64 ? ~0ull : ((1ull << t64) - 1ull);
                if (ok) {
                    cand = 0ull;
                    for (int s = 0; s < t64; ++s) {
                        float d[3];
                        offset_f(nbr[base + s], nullptr, d);
                        bool c = false;
#pragma unroll
                        for (int f = 0; f < NF; ++f) {
                            const float q = incr(f, d);
                            c = c || q >= thHi[f] || q <= thLo[f];
                        }
                        cand |= (unsigned long long)c << s;
                    }
                }
                while (cand) {
                    const int s = __ffsll((long long)cand) - 1;
                    cand &= cand - 1ull;
                    exact_slot(s);
                }
                for (int s = 64; s < tot; ++s) exact_slot(s);
                if (tot > 0) {
#pragma unroll
                    for (int f = 0; f < NF; ++f)
                        if (flat[f]) mxM[f] = mnM[f] = ord_key(fi[f]);
                }
            }
            if (p.foqp) {
#pragma unroll
                for (int f = 0; f < NF; ++f)
#pragma unroll
                    for (int a = 0; a < D; ++a) gr[f][a] = twice(gr[f][a]);
            } else {
#pragma unroll
                for (int f = 0; f < NF; ++f)
#pragma unroll
                    for (int a = 0; a < D; ++a) gr[f][a] *= icq;
            }
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const double xN = key_double(mxN[f]), nN = key_double(mnN[f]);
                const double xM = key_double(mxM[f]), nM = key_double(mnM[f]);
                double aMax = ref_abs((xN - fi[f]) / (xM - fi[f]), p.int_abs);
                double aMin = ref_abs((fi[f] - nN) / (fi[f] - nM), p.int_abs);
                if (aMin <= aMax && p.beta * aMin < 1.) {
#pragma unroll
                    for (int a = 0; a < D; ++a) gr[f][a] *= aMin;
                } else if (aMax <= aMin && p.beta * aMax < 1.) {
#pragma unroll
                    for (int a = 0; a < D; ++a) gr[f][a] *= aMax;
                }
            }
        }
        Grad go;
#pragma unroll
        for (int k = 0; k < 16; ++k) go.g[k] = 0.;
#pragma unroll
        for (int f = 0; f < NF; ++f) {
            int slot = (f == NF - 1) ? 4 : f;   // P always at slot 4
#pragma unroll
            for (int a = 0; a < D; ++a) go.g[slot * 3 + a] = gr[f][a];
        }
        // div v of the limited gradients, in the face kernel's order
        go.g[15] = D == 3 ? (go.g[3] + go.g[7]) + go.g[11] : go.g[3] + go.g[7];
        {   // the particle part of the half-step prediction (fma chains)
            const double *G = go.g;
            const double div = go.g[15], irho = geo[i].irho;
            const double v[3] = {pi.vx, pi.vy, pi.vz};
            const double src[5] = {pi.rho * div, (p.gamma * pi.P) * div, G[12] * irho, G[13] * irho, G[14] * irho};
            const int blk[5] = {0, 12, 3, 6, 9};
#pragma unroll
            for (int f = 0; f < 8; ++f) go.t[f] = 0.;
#pragma unroll
            for (int f = 0; f < D + 2; ++f) go.t[f] = fma_dotD<D>(v, G + blk[f], src[f]);
        }
        grad[i] = go;
      }   // i < p.n
      if (dtlo) {
        // the least upper bound on dt of each simulation (positive floats
        // order as their bit patterns)
        const int m0 = __shfl_sync(0xffffffffu, mi, 0);
        if (__all_sync(0xffffffffu, mi == m0)) {
            float best = dthi;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_xor_sync(0xffffffffu, best, o));
            if (lane == 0 && m0 >= 0 && best < FLT_INF_) atomicMin(dtcap + m0, __float_as_uint(best));
        } else if (mi >= 0 && dthi < FLT_INF_) {
            atomicMin(dtcap + mi, __float_as_uint(dthi));
        }
      }
      if (dtbits) {
        // the minimum over particles does not depend on the order of the
        // atomicMin calls: a warp inside one simulation reduces first and
        // issues one atomic; a warp that straddles two issues one per lane
        const int m0 = __shfl_sync(0xffffffffu, mi, 0);
        if (__all_sync(0xffffffffu, mi == m0)) {
            double best = dti;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_xor_sync(0xffffffffu, best, o));
            if (lane == 0 && m0 >= 0 && best < DBL_MAX_) atomic_min_pos_double(dtbits + m0, best);
        } else if (mi >= 0 && dti < DBL_MAX_) {
            atomic_min_pos_double(dtbits + mi, dti);
        }
      }
    }
}

// ------------------------------------------------------------------ faces

// Particles::pairwiseLimiter, Particles.cpp:1735-1785, for one side: phi0
// the reconstructed value, phi_i this side's particle value, phi_ij the value
// interpolated to the face, ad = |phi_i - phi_j|, delta1/delta2 = PSI_1/PSI_2
// ad, and i_lt_j = phi_i < phi_j (the two values differ).  Every comparison
// on integer keys (ord_key), off the FP64 pipe.  The shifts phi +- delta are
// fused multiply-adds fma(+-PSI, ad, phi): for the reference's PSI_1 = 0.5
// and PSI_2 = 0.25 the product is exact, so this is the reference's product
// then sum bit for bit, one FP64 instruction instead of two (other PSI: one
// rounding fewer).
__device__ __forceinline__ double pairwise_side(double phi0, double phi_i, double phi_ij, double ad, double psi1,
                                                double psi2, bool i_lt_j, int int_abs) {
    // the bound that is used is phi_minus = phi_min - delta1 when phi_i <
    // phi_j and phi_plus = phi_max + delta1 otherwise, and in both cases the
    // extreme it starts from is phi_i; the reference takes the shift when it
    // keeps the sign, (a >= 0 && b >= 0) || (a < 0 && b < 0), else
    // phi / (1 + delta1 / |phi|)
    // (phi / (1 + delta1 / |phi|) evaluated as phi |phi| / (|phi| + delta1),
    // one division by the Newton-Raphson reciprocal, and only where the
    // shift would change the sign; the same value to a few ulp, also for
    // |phi| = 0 and the int abs binding)
    const double shifted = fma(i_lt_j ? -psi1 : psi1, ad, phi_i);
    double bound = shifted;
    if ((ord_key(shifted) >= 0) != (ord_key(phi_i) >= 0)) {
        const double ra = ref_abs(phi_i, int_abs);
        bound = fdiv(phi_i * ra, fma(psi1, ad, ra));
    }
    const double t = fma(i_lt_j ? psi2 : -psi2, ad, phi_ij);
    if (i_lt_j) {
        const double minPhiD2 = dlt(t, phi0) ? t : phi0;
        return dlt(minPhiD2, bound) ? bound : minPhiD2;
    }
    const double maxPhiD2 = dlt(phi0, t) ? t : phi0;
    return dlt(bound, maxPhiD2) ? bound : maxPhiD2;
}

// The pairwise limiter on both sides of a face: phi0R/phi0L the
// reconstructed values (replaced by the limited ones), phiR/phiL the values
// of particles i and j, rR/rL = |x_ij - x_i| / |x_j - x_i| and
// |x_ij - x_j| / |x_j - x_i|.  The j side's phi_i - phi_j is the exact
// negation of the i side's, so |phi_i - phi_j| is the same double on both
// sides and is computed once; phi_ij on the j side, phi_j + rL (phi_i -
// phi_j), is fma(rL, d, phi_j) with d = phi_i - phi_j.  Equal particle values
// (neither phi_i < phi_j nor phi_i > phi_j) give the particle values back.
__device__ __forceinline__ void pairwise_limiter(const Params &p, double &phi0R, double &phi0L, double phiR,
                                                 double phiL, double rR, double rL) {
    const long long kR = ord_key(phiR), kL = ord_key(phiL);
    if (kR == kL) { phi0R = phiR; phi0L = phiL; return; }
    const bool r_lt_l = kR < kL;
    const double d = phiR - phiL;
    const double ad = ref_abs(d, p.int_abs);
    phi0R = pairwise_side(phi0R, phiR, fma(rR, -d, phiR), ad, p.psi1, p.psi2, r_lt_l, p.int_abs);
    phi0L = pairwise_side(phi0L, phiL, fma(rL, d, phiL), ad, p.psi1, p.psi2, !r_lt_l, p.int_abs);
}

// Network inputs of a face, from its face-frame problem sorted as the
// gamma = 5/3 solver sorts it (riemann5_begin): side A the one with the lower
// pressure (particle i on ties), side B the other, the mirror image negating
// both normal velocities, so that du = uB - uA is the same in both
// orientations:  log(rhoB/rhoA), du/cA, log(pB/pA) >= 0, log(cB/cA), in single
// precision (c = sqrt(gamma p / rho)).  The network predicts
// y = log(p* / p_TR), p_TR the two-rarefaction guess of the face; p* and p_TR
// are the same for both orientations.  p_TR is exact when both waves are rarefactions and its error grows
// with the shock strength p_TR / min(pL, pR) - 1 (about 1e-6 at 0.2, 3e-3 at
// 2-4, 2e-2 beyond 4, measured on random states), so only faces with
// p_TR > PSTAR_HARD * min(pL, pR) are handed to the network; the others are
// solved from p_TR in the first pass.  Where |y| is below PSTAR_GATE the
// correction is within the network's own error (BF16 activations) and Newton
// starts from p_TR as well.
constexpr double PSTAR_HARD = 2.0;
constexpr float PSTAR_GATE = 0.01f;

__device__ __forceinline__ float4 pstar_features_sorted(double rhoA, double pA, double rhoB, double pB, double du,
                                                       float gamma) {
    const float ra = (float)rhoA, rb = (float)rhoB, pa = (float)pA, pb = (float)pB;
    const float ca = sqrtf(gamma * pa / ra), cb = sqrtf(gamma * pb / rb);
    return make_float4(logf(rb / ra), (float)du / ca, logf(pb / pa), logf(cb / ca));
}

// the same from the unsorted face-frame states (R = particle i, left; L = j)
__device__ __forceinline__ float4 pstar_features(const double *R, const double *L, double unR, double unL,
                                                double gamma) {
    const bool mir = dlt(L[1], R[1]);
    return mir ? pstar_features_sorted(L[0], L[1], R[0], R[1], unL - unR, (float)gamma)
               : pstar_features_sorted(R[0], R[1], L[0], L[1], unL - unR, (float)gamma);
}

// One canonical face (i < j): effective face A_ij = psi~_j(x_i)/omega_i -
// psi~_i(x_j)/omega_j from the psi~ of both slots (compEffectiveFace,
// Particles.cpp:1290-1311, 2504-2531); boosted, reconstructed, optionally
// pairwise-limited and half-step-predicted states (compRiemannStatesLR,
// :1488-1733 / 2533-2683, including the vz[i] of :1717,1719); the face-frame
// problem (normal velocity components, face_normal), exact solve with i as
// the left state, back to the lab frame and projection on A_ij
// (Riemann::Riemann/exact/rotateAndProjectFluxes2D/3D,
// demonstrator/src/Riemann.cpp:7-229; project_flux says why no rotation
// matrix is needed).  Output slot order: [mass, energy, px, py, pz].
// MODE 0: the whole face.  MODE 1 (learned guess, first pass): faces with a
// strong shock in p_TR stop before the exact solve and are
// queued (state and network inputs at the queue position, order immaterial:
// each face writes only its own flux); all other faces are finished as in
// MODE 0.  MODE 2 (second pass, over the queue): reload the state, solve from
// the network's guess, project the flux.  `harvest` (MODE 0) records network
// inputs and targets log(p*/p_TR) of every `stride`-th face.
// MODE 3 (plain first pass, gamma = 5/3): one Newton step from the
// two-rarefaction guess; faces that have not converged are queued with their
// iterate, so that the warps of this pass do not all run the second step that
// a fifth of the faces need (nearly every warp holds one).  MODE 4 (second
// pass over that queue): continue Newton from the stored iterate, which is the
// same iteration with the same arithmetic, densely packed.  A full queue
// keeps the face in MODE 3 and finishes it there.
// Riemann::Riemann (demonstrator/src/Riemann.cpp:7-81) rotates both states
// with Helper::rotationMatrix2D/3D(hatA, unitX) (Helper.cpp:39-77), hatA =
// A/|A|.  The one-dimensional problem reads only the first rotated velocity
// component, and the first row of that rotation is hatA: u = hatA . v.  The
// velocities themselves stay unrotated (see project_flux).
template <int D>
__device__ __forceinline__ void face_normal(const double *A, const double *R, const double *L, double *hatA,
                                            double &unR, double &unL) {
    const double iAN = frsqrt(dotD<D>(A, A));
#pragma unroll
    for (int a = 0; a < D; ++a) hatA[a] = iAN * A[a];
    unR = dotD<D>(hatA, R + 2);
    unL = dotD<D>(hatA, L + 2);
}

// Riemann::exact after the solve and rotateAndProjectFluxes2D/3D
// (demonstrator/src/Riemann.cpp:100-229): the sampled velocity takes its
// tangential components from the sampled side, is rotated back and boosted by
// the frame velocity, and the flux is projected on A_ij.  Rotating a state
// into the face frame, replacing its normal component by u* and rotating back
// leaves its tangential part unchanged, so v* = v_side + (u* - u_side) hatA
// (u* hatA for vacuum), without the rotation matrices.  R (particle i, the
// left state) and L: [rho, P, v..] with unrotated velocities, unR/unL their
// normal components.  Fo: [mass, energy, px, py, pz].  Returns ST_VACUUM
// when the solution is vacuum, else 0.
template <int D>
__device__ __forceinline__ unsigned project_flux(const RiemannResult &rs, const double *R, const double *L,
                                                 double unR, double unL, const double *hatA, const double *A,
                                                 const double *vf, double inv_gm1, int mfm, double *Fo) {
    unsigned st = 0;
    double vSol[3] = {0., 0., 0.};
    if (rs.flag == 1 || rs.flag == -1) {
        const double *side = rs.flag == 1 ? L : R;
        const double du = rs.u - (rs.flag == 1 ? unL : unR);
#pragma unroll
        for (int a = 0; a < D; ++a) vSol[a] = fma(du, hatA[a], side[2 + a]);
    } else {
        st = ST_VACUUM;
#pragma unroll
        for (int a = 0; a < D; ++a) vSol[a] = rs.u * hatA[a];
    }
    // F_m = rho* (A . v*), F_p = F_m v_lab + P* A,
    // F_E = (A . v*) (P*/(gamma-1) + rho*/2 |v_lab|^2) + P* (A . v_lab);
    // MESHLESS_FINITE_MASS keeps F_m and drops the advective terms
    const double rhoSol = rs.rho, PSol = rs.p;
    const double pe = PSol * inv_gm1;
    const double Av = dotD<D>(A, vSol);
    double vLab[3] = {0., 0., 0.};
#pragma unroll
    for (int a = 0; a < D; ++a) vLab[a] = vSol[a] + vf[a];
    Fo[0] = rhoSol * Av;
    const double Avm = mfm ? 0. : Av;
    const double mflux = rhoSol * Avm;
#pragma unroll
    for (int a = 0; a < D; ++a) Fo[2 + a] = fma(mflux, vLab[a], PSol * A[a]);
    if (D == 2) Fo[4] = 0.;
    // pe + rho*/2 |v_lab|^2 as one fused multiply-add
    Fo[1] = fma(Avm, fma(half_of(rhoSol), dotD<D>(vLab, vLab), pe), PSol * dotD<D>(A, vLab));
    return st;
}

// Register caps of the face kernels, per dimension: more warps per SM hide
// more of the Riemann iteration's dependency latency, fewer registers spill
// more.  Measured on the face passes: 3D (Sedov 128^3) 168 registers (12
// warps per SM, a small spill) 21.60 ms, against 21.74 / 21.81 / 22.29 /
// 21.80 ms at 152 / 144 / 136 / 128; 2D (the 256-member KH ensemble) 128
// registers (16 warps) 19.34 ms, against 20.95 ms at 168 and 21.6-21.9 ms
// at 136-152.  Blocks of up to 256 threads.
#ifndef MLH_FACE_MAXREG_3D
#define MLH_FACE_MAXREG_3D 168
#endif
#ifndef MLH_FACE_MAXREG_2D
#define MLH_FACE_MAXREG_2D 128
#endif
#define MLH_FACE_BOUNDS __maxnreg__(D == 3 ? MLH_FACE_MAXREG_3D : MLH_FACE_MAXREG_2D)
// The face-frame Riemann problem of canonical face f (i < j): effective face
// A_ij = psi~_j(x_i)/omega_i - psi~_i(x_j)/omega_j from the psi~ of both
// slots (compEffectiveFace, Particles.cpp:1290-1311, 2504-2531); boosted,
// reconstructed, optionally pairwise-limited and half-step-predicted states
// (compRiemannStatesLR, :1488-1733 / 2533-2683, including the vz[i] of
// :1717,1719); the face normal and the normal velocity components
// (face_normal).  R (particle i, the left state) and L: [rho, P, v..] with
// unrotated velocities.  Returns false for a face without its links (the
// status bit is set).
template <int D>
__device__ __forceinline__ bool face_states(const Params &p, const Member *__restrict__ members,
                                            const int *__restrict__ memberOf, const GridInfo *__restrict__ grids,
                                            const Prim *__restrict__ prim, const Geo *__restrict__ geo,
                                            const Grad *__restrict__ grad, const uint32_t *__restrict__ nbr,
                                            const double *__restrict__ psi, const FaceRef *__restrict__ faces,
                                            const double *__restrict__ dtp, int f, unsigned &st_local, double *R,
                                            double *L, double *A, double *vf, double *hatA, double &unR,
                                            double &unL) {
    constexpr int NV = D + 2;
    const FaceRef fr = faces[f];
    if (fr.i < 0 || fr.slot < 0) {
        st_local |= ST_ASYMMETRIC;
        return false;
    }
    const int i = fr.i;
    const int mi = memberOf ? memberOf[i] : 0;
    const double dt = dtp[mi];
    const double h = members[mi].h;
    const double hq = p.adaptive_h ? p.hp[i] : h;   // quadrature-point radius
    const size_t si = (size_t)i * p.K + fr.slot;
    const uint32_t e = nbr[si];
    const int j = (int)(e & IDX_MASK);
    const bool img = (e >> IMG_SHIFT) != 0;
    const Prim pi = prim[i], pj = prim[j];
    const double Vi = geo[i].V, Vj = geo[j].V;
    double xi[3] = {pi.x, pi.y, pi.z}, xj[3];
    if (img) neighbour_pos<D>(e, pj, grids[mi], xj);
    else { xj[0] = pj.x; xj[1] = pj.y; xj[2] = pj.z; }
    // --- effective face
    {
        const double *ps_i = psi + si * 3;
        if (fr.rslot >= 0) {
            const double *ps_j = psi + ((size_t)j * p.K + fr.rslot) * 3;
#pragma unroll
            for (int a = 0; a < D; ++a) A[a] = Vi * ps_i[a] - Vj * ps_j[a];
        } else {
            st_local |= ST_ASYMMETRIC;
#pragma unroll
            for (int a = 0; a < D; ++a) A[a] = Vi * ps_i[a];
        }
    }
    // --- states at the face
    double xijxi[3], xjxi[3], xijxj[3];
#pragma unroll
    for (int a = 0; a < D; ++a) {
        xjxi[a] = xj[a] - xi[a];
        if (p.foqp) {
            // .5 (x_j - x_i) (on the integer pipe), and .5 (x_i - x_j) is its
            // exact negation
            xijxi[a] = half_of(xjxi[a]);
            xijxj[a] = -xijxi[a];
        } else {
            double xij = xi[a] + hq / 4. * xjxi[a];
            xijxi[a] = xij - xi[a];
            xijxj[a] = xij - xj[a];
        }
    }
    const double vi[3] = {pi.vx, pi.vy, pi.vz}, vj[3] = {pj.vx, pj.vy, pj.vz};
    if (p.move) {
        if (p.foqp) {
#pragma unroll
            for (int a = 0; a < D; ++a) vf[a] = half_of(vi[a] + vj[a]);
        } else {
            double dotProd = dotD<D>(xijxi, xjxi);
            double dSqr = dotD<D>(xjxi, xjxi);
#pragma unroll
            for (int a = 0; a < D; ++a) vf[a] = vi[a] + (vj[a] - vi[a]) * dotProd / dSqr;
        }
    }
    const double *Gi = grad[i].g, *Gj = grad[j].g;
    // gradient blocks: 0 rho, 3 vx, 6 vy, 9 vz, 12 P
    R[0] = pi.rho; L[0] = pj.rho;
    R[1] = pi.P; L[1] = pj.P;
#pragma unroll
    for (int a = 0; a < D; ++a) { R[2 + a] = vi[a] - vf[a]; L[2 + a] = vj[a] - vf[a]; }
    // W -= dt/2 (source + (v - v_frame) . grad W): the particle part,
    // source + v . grad W, comes with the gradients (Grad::t); the face adds
    // v_frame . grad W.  The reference uses vz[i] on the j side of the vx and
    // vy terms in 3D (Particles.cpp:1717,1719): (vz_i - vf_z) = (vz_j - vq_z)
    // with the shifted frame velocity vq_z = vf_z - (vz_i - vz_j).
    const double hdt = half_of(dt);
    const double *Ti = grad[i].t, *Tj = grad[j].t;
    const int blk[5] = {0, 12, 3, 6, 9};   // gradient blocks: 0 rho, 3 vx, 6 vy, 9 vz, 12 P
    const double vq2 = D == 3 ? vf[2] - (vi[2] - vj[2]) : 0.;
    if (D == 2 && !p.pairwise) {
        // no limiter between reconstruction and prediction: one FMA chain per
        // field and side, W - dt/2 T + grad W . (x_ij - x_side + dt/2 v_frame)
        // (a run-wide branch: with the limiter on, image faces that skip it
        // keep the other form, so that warps do not run both; 3D keeps the
        // other form, whose registers the 3D face kernels are tuned to)
        double yi[3], yj[3], yq[3];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            yi[a] = fma(hdt, vf[a], xijxi[a]);
            yj[a] = fma(hdt, vf[a], xijxj[a]);
            yq[a] = (D == 3 && a == 2) ? fma(hdt, vq2, xijxj[a]) : yj[a];
        }
#pragma unroll
        for (int f = 0; f < NV; ++f) {
            R[f] = fma_dotD<D>(Gi + blk[f], yi, fma(-hdt, Ti[f], R[f]));
            const double *yy = (D == 3 && (f == 2 || f == 3)) ? yq : yj;
            L[f] = fma_dotD<D>(Gj + blk[f], yy, fma(-hdt, Tj[f], L[f]));
        }
    } else {
        double Rb[5], Lb[5];
#pragma unroll
        for (int k = 0; k < NV; ++k) { Rb[k] = R[k]; Lb[k] = L[k]; }
        // W + grad W . (x_ij - x_side), one FMA chain from W per field
#pragma unroll
        for (int f = 0; f < NV; ++f) {
            R[f] = fma_dotD<D>(Gi + blk[f], xijxi, R[f]);
            L[f] = fma_dotD<D>(Gj + blk[f], xijxj, L[f]);
        }
        if (p.pairwise && (!img || p.img_pw)) {   // image faces skip it (Particles.cpp:2533-2683)
            // |x_ij - x_i| / |x_j - x_i| and |x_ij - x_j| / |x_j - x_i|: with the
            // first-order quadrature point x_ij - x_i = (x_j - x_i) / 2 exactly,
            // so both norms are exactly half of |x_j - x_i| (scaling by 1/2 and
            // 1/4 is exact) and both quotients are exactly 0.5
            double ri = .5, rj = .5;
            if (!p.foqp) {
                double xijxi_abs = 0., xijxj_abs = 0., xjxi_abs = 0.;
#pragma unroll
                for (int a = 0; a < D; ++a) {
                    xijxi_abs += xijxi[a] * xijxi[a];
                    xijxj_abs += xijxj[a] * xijxj[a];
                    xjxi_abs += xjxi[a] * xjxi[a];
                }
                xjxi_abs = sqrt(xjxi_abs);
                ri = sqrt(xijxi_abs) / xjxi_abs;
                rj = sqrt(xijxj_abs) / xjxi_abs;
            }
#pragma unroll
            for (int k = 0; k < NV; ++k) pairwise_limiter(p, R[k], L[k], Rb[k], Lb[k], ri, rj);
        }
        // the prediction, one FMA chain per field and side from the limited value
        const double nvf[3] = {-vf[0], -vf[1], -vf[2]};
        const double nvq[3] = {-vf[0], -vf[1], -vq2};
#pragma unroll
        for (int f = 0; f < NV; ++f) {
            R[f] = fma(-hdt, fma_dotD<D>(nvf, Gi + blk[f], Ti[f]), R[f]);
            const double *nj = (D == 3 && (f == 2 || f == 3)) ? nvq : nvf;
            L[f] = fma(-hdt, fma_dotD<D>(nj, Gj + blk[f], Tj[f]), L[f]);
        }
    }
    if (dneg(R[1]) || dneg(L[1])) st_local |= ST_NEG_PRESSURE;
    // --- Riemann problem in the face frame (i left, j right)
    face_normal<D>(A, R, L, hatA, unR, unL);
    return true;
}

template <int D, bool ROOT5, int MODE>
__global__ void MLH_FACE_BOUNDS k_faces(Params p, const Member *__restrict__ members,
                                               const int *__restrict__ memberOf, const GridInfo *__restrict__ grids,
                                               const Prim *__restrict__ prim, const Geo *__restrict__ geo,
                                               const Grad *__restrict__ grad, const uint32_t *__restrict__ nbr,
                                               const double *__restrict__ psi, const int *__restrict__ faceTotal,
                                               const FaceRef *__restrict__ faces, const double *__restrict__ dtp,
                                               double *__restrict__ Fface, unsigned long long *__restrict__ newtonSum,
                                               unsigned *__restrict__ status, FaceQueue qa, FaceQueue qb,
                                               float4 *__restrict__ feat, const float *__restrict__ yguess,
                                               Harvest hv) {
    int nf = *faceTotal < p.faces_cap ? *faceTotal : p.faces_cap;
    constexpr bool QUEUED = MODE == 2 || MODE == 4;   // passes over the queue
    if (QUEUED) {   // the queue holds min(count, capacity) faces; MODE 3 finished the rest itself
        const int qn = *qa.count < qa.cap ? *qa.count : qa.cap;
        nf = qn < nf ? qn : nf;
    }
    const RiemannConsts rc = make_riemann_consts(p.gamma, p.rtol, p.rmaxit);
    const double gamma = p.gamma;
    unsigned long long iters_local = 0, fallback_local = 0, deferred_local = 0;
    unsigned st_local = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nf; t += gridDim.x * blockDim.x) {
        // MODE 2 walks the queue: t is the queue position, f the face
        const int f = QUEUED ? qa.face[t] : t;
        double R[5], L[5], A[3] = {0., 0., 0.}, vf[3] = {0., 0., 0.}, hatA[3] = {0., 0., 0.};
        double unR = 0., unL = 0.;   // velocity components along the face normal
        double ptr_q = -1.;   // MODE 2: two-rarefaction guess found in MODE 1; MODE 4: Newton iterate
        if (QUEUED) {
            const FaceState &fs = qa.st[t];
            ptr_q = fs.v[19];
#pragma unroll
            for (int k = 0; k < 5; ++k) { R[k] = fs.v[k]; L[k] = fs.v[5 + k]; }
#pragma unroll
            for (int a = 0; a < 3; ++a) { A[a] = fs.v[10 + a]; vf[a] = fs.v[13 + a]; hatA[a] = fs.v[16 + a]; }
            unR = dotD<D>(hatA, R + 2);
            unL = dotD<D>(hatA, L + 2);
        } else {
        if (!face_states<D>(p, members, memberOf, grids, prim, geo, grad, nbr, psi, faces, dtp, f, st_local, R, L, A,
                            vf, hatA, unR, unL))
            continue;
        }   // !QUEUED
        double guess = -1.;
        if (MODE == 2) {
            const float y = yguess[t];
            if (isfinite(y) && fabsf(y) > PSTAR_GATE && fabsf(y) < 30.f)
                guess = ptr_q * (double)__expf(y);
        }
        if (MODE == 4) guess = ptr_q;
        // MODE 1 defers faces whose two-rarefaction guess says strong shock
        const double defer = MODE == 1 ? PSTAR_HARD * (dlt(L[1], R[1]) ? L[1] : R[1]) : 0.;   // min on the keys
        RiemannResult rs = ROOT5 ? riemann_exact5(rc, R[0], unR, R[1], L[0], unL, L[1], guess, defer,
                                                  (MODE == 3 || (MODE == 1 && p.face_split)) ? 1 : 0)
                                 : riemann_exact(rc, R[0], unR, R[1], L[0], unL, L[1], guess, defer);
        // deferred faces: strong shocks of MODE 1 (unsolved, iters 0) go to
        // queue A for the network; faces Newton has not finished after one
        // step go to queue A (MODE 3) or B (MODE 1) with their iterate
        if ((MODE == 1 || MODE == 3) && rs.flag == 2) {
            const bool strong = MODE == 1 && rs.iters == 0;
            const FaceQueue &fq = (MODE == 1 && !strong) ? qb : qa;
            const int q = atomicAdd(fq.count, 1);
            if (q < fq.cap) {
                FaceState &fs = fq.st[q];
#pragma unroll
                for (int k = 0; k < 5; ++k) { fs.v[k] = R[k]; fs.v[5 + k] = L[k]; }
#pragma unroll
                for (int a = 0; a < 3; ++a) { fs.v[10 + a] = A[a]; fs.v[13 + a] = vf[a]; fs.v[16 + a] = hatA[a]; }
                fs.v[19] = rs.pstar;   // the two-rarefaction guess (strong) or the Newton iterate
                fq.face[q] = f;
                if (strong) feat[q] = pstar_features(R, L, unR, unL, gamma);
                else iters_local += (unsigned long long)rs.iters;
                continue;
            }
            // queue full: finish here, from the iterate or from p_TR
            const int done = rs.iters;
            rs = ROOT5 ? riemann_exact5(rc, R[0], unR, R[1], L[0], unL, L[1], strong ? -1. : rs.pstar, 0.)
                       : riemann_exact(rc, R[0], unR, R[1], L[0], unL, L[1], -1., 0.);
            if (rs.iters >= 0) rs.iters += done;
        }
        if (MODE == 0 && hv.stride > 0 && (hv.strong || f % hv.stride == 0)) {
            const double ptr = two_rarefaction_guess<ROOT5>(rc, R[0], unR, R[1], L[0], unL, L[1]);
            if (rs.iters >= 0 && rs.pstar > 0. && ptr > 0.) {
                if (hv.strong) {
                    // the faces the learned step hands to the network
                    if (dlt(PSTAR_HARD * (dlt(L[1], R[1]) ? L[1] : R[1]), ptr)) {
                        const int slot = atomicAdd(hv.count, 1);
                        if (slot < hv.cap) {
                            hv.x[slot] = pstar_features(R, L, unR, unL, gamma);
                            hv.t[slot] = (float)log(rs.pstar / ptr);
                        }
                    }
                } else {
                    const int slot = f / hv.stride;
                    if (slot < hv.cap) {
                        hv.x[slot] = pstar_features(R, L, unR, unL, gamma);
                        hv.t[slot] = (float)log(rs.pstar / ptr);
                        atomicMax(hv.count, slot + 1);
                    }
                }
            }
        }
        if (rs.iters < 0) st_local |= ST_NEWTON;
        else {
            // iters counts every Newton step run: a learned guess that did not
            // converge adds max_iter wasted steps before the restart from the
            // two-rarefaction guess
            if (MODE == 2 && rs.iters > rc.max_iter) ++fallback_local;
            if (MODE == 2) ++deferred_local;
            iters_local += (unsigned long long)rs.iters;
        }
        double Fo[5];
        st_local |= project_flux<D>(rs, R, L, unR, unL, hatA, A, vf, rc.inv_gm1, p.mfm, Fo);
        // the face's Newton steps (the step of the first pass included in
        // MODE 4; -1: no convergence) in the record's sixth double, for parity
        // checks
        const int face_iters = rs.iters < 0 ? -1 : rs.iters + (MODE == 4 ? 1 : 0);
        double2 *dst = reinterpret_cast<double2 *>(Fface + (size_t)f * 6);
        dst[0] = make_double2(Fo[0], Fo[1]);
        dst[1] = make_double2(Fo[2], Fo[3]);
        dst[2] = make_double2(Fo[4], (double)face_iters);
    }
    // block-level accumulation of the counters
    for (int o = 16; o > 0; o >>= 1) {
        iters_local += __shfl_xor_sync(0xffffffffu, iters_local, o);
        fallback_local += __shfl_xor_sync(0xffffffffu, fallback_local, o);
        deferred_local += __shfl_xor_sync(0xffffffffu, deferred_local, o);
        st_local |= __shfl_xor_sync(0xffffffffu, st_local, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (iters_local) atomicAdd(newtonSum, iters_local);
        if (fallback_local) atomicAdd(newtonSum + 1, fallback_local);
        if (deferred_local) atomicAdd(newtonSum + 2, deferred_local);
        if (st_local) flag(status, st_local);
    }
}

// Plain gamma = 5/3 face pass with the faces that need more than one Newton
// step regrouped inside the block (face_split 2).  A warp issues every
// instruction that any of its lanes needs, so the second Newton step of the
// few faces that need it would hold the whole warp.  Instead: every face of
// the block's round sets up its problem and takes the first Newton step
// from p_TR, and leaves its solver state (sorted sides, iterate) in shared
// memory; the block's unfinished faces are listed and continued, densely, by
// its first threads (the iteration riemann_exact5 runs from the iterate as a
// guess, on the stored sides: the same arithmetic as the two-pass split);
// then every face samples its solution and projects its flux, with all
// lanes busy.  The loop runs in block-wide rounds so that every thread
// reaches the barriers.  LEARNED: the learned-guess step.  Strong shocks
// (p_TR > PSTAR_HARD min(pL, pR)) stop before their first Newton step; the
// block lists them, evaluates the network for them on the tensor cores (a
// warp per 16 faces, block_network_guess; a block-uniform branch that a round
// without strong shocks skips) and continues them from p_TR e^y together with
// the other unfinished faces.  Nothing leaves the block: the plain and the
// learned step differ only by that branch.
constexpr int FB_T = 128;   // threads per block of k_faces_block

// The network's guesses for the ns strong-shock faces of a round listed in
// slist (their solver states in sv, s.p = p_TR): warp w takes the faces
// w*16 .. w*16+15, then the next 64, and so on; s.p becomes p_TR e^y where
// PSTAR_GATE < |y| < 30 (finite), and stays p_TR elsewhere.  Every lane of a
// warp runs the MMAs (rows beyond ns are zero inputs whose outputs are
// dropped).  Out of line, so that the rare branch that calls it does not shape
// the register allocation of the face pass.
__device__ __noinline__ void block_network_guess(const PackedMlp *__restrict__ w, Solve5 *sv, const int *slist,
                                                 int ns, float gamma) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = warp * 16; base < ns; base += FB_T / 2) {
        const int row = base + (lane & 15);
        const bool mine = lane < 16 && row < ns;
        float4 xi = make_float4(0.f, 0.f, 0.f, 0.f);
        if (mine) {
            const Solve5 &q = sv[slist[row]];
            xi = pstar_features_sorted(q.A.rho, q.A.p, q.B.rho, q.B.p, q.du, gamma);
        }
        const float y = mlp_rows<1>(w, xi);
        if (mine && isfinite(y) && fabsf(y) > PSTAR_GATE && fabsf(y) < 30.f) {
            Solve5 &q = sv[slist[row]];
            q.p = q.p * (double)__expf(y);
        }
    }
}

template <int D, bool LEARNED>
__global__ void MLH_FACE_BOUNDS k_faces_block(Params p, const Member *__restrict__ members,
                                              const int *__restrict__ memberOf, const GridInfo *__restrict__ grids,
                                              const Prim *__restrict__ prim, const Geo *__restrict__ geo,
                                              const Grad *__restrict__ grad, const uint32_t *__restrict__ nbr,
                                              const double *__restrict__ psi, const int *__restrict__ faceTotal,
                                              const FaceRef *__restrict__ faces, const double *__restrict__ dtp,
                                              double *__restrict__ Fface, unsigned long long *__restrict__ newtonSum,
                                              unsigned *__restrict__ status, const PackedMlp *__restrict__ mlp) {
    __shared__ Solve5 sv[FB_T];
    __shared__ int todo[FB_T];
    __shared__ int slist[LEARNED ? FB_T : 1];
    __shared__ int wcount[FB_T / 32];
    const int nf = *faceTotal < p.faces_cap ? *faceTotal : p.faces_cap;
    const RiemannConsts rc = make_riemann_consts(p.gamma, p.rtol, p.rmaxit);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long iters_local = 0, fallback_local = 0, learned_local = 0;
    unsigned st_local = 0;
    for (int t0 = blockIdx.x * FB_T; t0 < nf; t0 += gridDim.x * FB_T) {
        const int f = t0 + threadIdx.x;
        double R[5], L[5], A[3] = {0., 0., 0.}, vf[3] = {0., 0., 0.}, hatA[3] = {0., 0., 0.};
        double unR = 0., unL = 0.;
        bool valid = f < nf;
        if (valid)
            valid = face_states<D>(p, members, memberOf, grids, prim, geo, grad, nbr, psi, faces, dtp, f, st_local, R,
                                   L, A, vf, hatA, unR, unL);
        bool unfinished = false, strong = false;
        if (valid) {
            // strong shocks of the learned step stop before their first
            // Newton step: p_TR > PSTAR_HARD min(pL, pR) (min on the keys)
            const double defer = LEARNED ? PSTAR_HARD * (dlt(L[1], R[1]) ? L[1] : R[1]) : 0.;
            const Solve5 s0 = riemann5_begin(rc, R[0], unR, R[1], L[0], unL, L[1], -1., defer, 1);
            sv[threadIdx.x] = s0;
            unfinished = s0.stage == 2;
            strong = LEARNED && s0.stage == 3;
        }
        // --- list the block's unfinished faces (and, learned, its strong shocks)
        const unsigned bal = __ballot_sync(0xffffffffu, unfinished || strong);
        const unsigned sbal = LEARNED ? __ballot_sync(0xffffffffu, strong) : 0u;
        if (lane == 0) wcount[warp] = __popc(bal) | (__popc(sbal) << 16);
        __syncthreads();
        int before = 0, nu = 0, sbefore = 0, ns = 0;
#pragma unroll
        for (int w = 0; w < FB_T / 32; ++w) {
            const int c = wcount[w] & 0xffff, cs = wcount[w] >> 16;
            before += w < warp ? c : 0;
            nu += c;
            sbefore += w < warp ? cs : 0;
            ns += cs;
        }
        const unsigned below = (1u << lane) - 1u;
        if (unfinished || strong) todo[before + __popc(bal & below)] = threadIdx.x;
        if (LEARNED && strong) slist[sbefore + __popc(sbal & below)] = threadIdx.x;
        __syncthreads();
        if (LEARNED && ns > 0) {   // block-uniform
            block_network_guess(mlp, sv, slist, ns, (float)p.gamma);
            __syncthreads();
        }
        // --- continue them on the first nu threads
        if ((int)threadIdx.x < nu) {
            const int slot = todo[threadIdx.x];
            Solve5 c = sv[slot];
            const bool from_net = LEARNED && c.stage == 3;
            riemann5_continue(rc, c);
            if (from_net) {
                ++learned_local;
                if (c.iters > rc.max_iter) ++fallback_local;
            }
            sv[slot] = c;
        }
        __syncthreads();
        // --- sample and project, every face of the round
        if (valid) {
            const Solve5 s = sv[threadIdx.x];
            RiemannResult rs;
            if (s.stage == 0) {
                rs.rho = 0.; rs.u = 0.; rs.p = 0.; rs.pstar = 0.; rs.flag = 0; rs.iters = 0;
            } else {
                rs = riemann5_finish(rc, s);
            }
            if (unfinished) iters_local += 1;   // the first step, counted as the two-pass split counts it
            if (rs.iters < 0) st_local |= ST_NEWTON;
            else iters_local += (unsigned long long)rs.iters;
            double Fo[5];
            st_local |= project_flux<D>(rs, R, L, unR, unL, hatA, A, vf, rc.inv_gm1, p.mfm, Fo);
            const int face_iters = rs.iters < 0 ? -1 : rs.iters + (unfinished ? 1 : 0);
            double2 *dst = reinterpret_cast<double2 *>(Fface + (size_t)f * 6);
            dst[0] = make_double2(Fo[0], Fo[1]);
            dst[1] = make_double2(Fo[2], Fo[3]);
            dst[2] = make_double2(Fo[4], (double)face_iters);
        }
        __syncthreads();   // the shared state is rewritten in the next round
    }
    for (int o = 16; o > 0; o >>= 1) {
        iters_local += __shfl_xor_sync(0xffffffffu, iters_local, o);
        if (LEARNED) {
            fallback_local += __shfl_xor_sync(0xffffffffu, fallback_local, o);
            learned_local += __shfl_xor_sync(0xffffffffu, learned_local, o);
        }
        st_local |= __shfl_xor_sync(0xffffffffu, st_local, o);
    }
    if (lane == 0) {
        if (iters_local) atomicAdd(newtonSum, iters_local);
        if (LEARNED && fallback_local) atomicAdd(newtonSum + 1, fallback_local);
        if (LEARNED && learned_local) atomicAdd(newtonSum + 2, learned_local);
        if (st_local) flag(status, st_local);
    }
}

// Riemann::Riemann + Riemann::exact (demonstrator/src/Riemann.cpp:7-229) for a
// batch of independent faces: per face the left state Wi (particle i) and the
// right state Wj (neighbour j), each [rho, P, v_x, v_y(, v_z)], the frame
// velocity and A_ij; one thread per face, the same device functions as
// k_faces.  F: [mass, energy, momentum] per face; iters: Newton iterations
// (-1 when the iteration did not converge).
template <int D, bool ROOT5>
__global__ void __launch_bounds__(256) k_riemann_batch(int n, RiemannConsts rc, int mfm,
                                                       const double *__restrict__ Wi, const double *__restrict__ Wj,
                                                       const double *__restrict__ vFrame,
                                                       const double *__restrict__ Aij, double *__restrict__ F,
                                                       int *__restrict__ iters, unsigned *__restrict__ status) {
    constexpr int NV = D + 2;
    unsigned st = 0;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        double R[5] = {0., 0., 0., 0., 0.}, L[5] = {0., 0., 0., 0., 0.};
        double A[3] = {0., 0., 0.}, vf[3] = {0., 0., 0.}, hatA[3], unR, unL;
#pragma unroll
        for (int k = 0; k < NV; ++k) { R[k] = Wi[(size_t)f * NV + k]; L[k] = Wj[(size_t)f * NV + k]; }
#pragma unroll
        for (int a = 0; a < D; ++a) { A[a] = Aij[(size_t)f * D + a]; vf[a] = vFrame[(size_t)f * D + a]; }
        if (R[1] < 0. || L[1] < 0.) st |= ST_NEG_PRESSURE;
        face_normal<D>(A, R, L, hatA, unR, unL);
        const RiemannResult rs = ROOT5 ? riemann_exact5(rc, R[0], unR, R[1], L[0], unL, L[1], -1., 0.)
                                       : riemann_exact(rc, R[0], unR, R[1], L[0], unL, L[1], -1., 0.);
        if (rs.iters < 0) st |= ST_NEWTON;
        double Fo[5];
        st |= project_flux<D>(rs, R, L, unR, unL, hatA, A, vf, rc.inv_gm1, mfm, Fo);
#pragma unroll
        for (int k = 0; k < NV; ++k) F[(size_t)f * NV + k] = Fo[k];
        if (iters) iters[f] = rs.iters;
    }
    if (st) flag(status, st);
}

void riemann_batch(int dim, int n, double gamma, double rtol, int max_iter, int mfm, const double *Wi,
                   const double *Wj, const double *vFrame, const double *Aij, double *F, int *iters,
                   unsigned *status, cudaStream_t s) {
    const RiemannConsts rc = make_riemann_consts(gamma, rtol, max_iter);
    const int blocks = n > 0 ? (n + 255) / 256 : 1;
#define MLH_RB(DD, R5) k_riemann_batch<DD, R5><<<blocks, 256, 0, s>>>(n, rc, mfm, Wi, Wj, vFrame, Aij, F, iters, status)
    if (dim == 2) { if (rc.root5) MLH_RB(2, true); else MLH_RB(2, false); }
    else { if (rc.root5) MLH_RB(3, true); else MLH_RB(3, false); }
#undef MLH_RB
}

// ------------------------------------------------------------------ gather + update

// Particles::collectFluxes (Particles.cpp:1913-2011) in slot order, then
// Particles::updateStateAndPosition (:2013-2110).  The update is skipped when
// the neighbour search overflowed, so that the host can retry the step with
// more slots.
template <int D>
__global__ void __launch_bounds__(256) k_update(Params p, const int *__restrict__ memberOf,
                                                const GridInfo *__restrict__ grids, const int *__restrict__ noi,
                                                const int *__restrict__ noiImg, const int *__restrict__ faceOf,
                                                const double *__restrict__ Fface, const double *__restrict__ dtp,
                                                double *__restrict__ x, double *__restrict__ y, double *__restrict__ z,
                                                double *__restrict__ vx, double *__restrict__ vy, double *__restrict__ vz,
                                                double *__restrict__ m, double *__restrict__ u, float4 *__restrict__ posf,
                                                double *__restrict__ fluxSums, unsigned *__restrict__ status) {
    const unsigned st0 = *status;
    if (st0 & (ST_NGB_OVERFLOW | ST_CAPACITY | ST_TIMEOUT | ST_GRID)) return;
    double *X[3] = {x, y, z};
    double *Vv[3] = {vx, vy, vz};
    unsigned st_local = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.n; i += gridDim.x * blockDim.x) {
        const int sim = memberOf ? memberOf[i] : 0;
        const double dt = dtp[sim];
        const size_t base = (size_t)i * p.K;
        const int tot = noi[i] + noiImg[i];
        double mF = 0., eF = 0., vF[3] = {0., 0., 0.};
        // four slots at a time: their face ids in one 16-byte load (K is a
        // multiple of 4) and all twelve flux loads issued before the sums,
        // which still run in slot order
        const int4 *fo4 = reinterpret_cast<const int4 *>(faceOf + base);
        for (int s0 = 0; s0 < tot; s0 += 4) {
            const int4 f4 = fo4[s0 >> 2];
            const int fos[4] = {f4.x, f4.y, f4.z, f4.w};
            double2 fa[4], fb[4], fc[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int fo = fos[k];
                const int af = fo > 0 ? fo : -fo;
                if (s0 + k < tot && fo != 0 && af <= p.faces_cap) {
                    const double2 *src = reinterpret_cast<const double2 *>(Fface + (size_t)(af - 1) * 6);
                    fa[k] = src[0]; fb[k] = src[1]; fc[k] = src[2];
                } else {
                    fa[k] = fb[k] = fc[k] = make_double2(0., 0.);
                }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int fo = fos[k];
                const int af = fo > 0 ? fo : -fo;
                if (!(s0 + k < tot && fo != 0 && af <= p.faces_cap)) continue;
                // the flux with the slot's sign: the sign bit flipped on the
                // integer pipe for a copied face, so that both kinds of slot
                // share one set of additions (x + (-f) is the same double as
                // adding the negated flux)
                const long long sg = fo > 0 ? 0ll : (long long)0x8000000000000000ull;
                auto sgn = [sg](double f) { return __longlong_as_double(__double_as_longlong(f) ^ sg); };
                mF += sgn(fa[k].x); vF[0] += sgn(fb[k].x); vF[1] += sgn(fb[k].y);
                if (D == 3) vF[2] += sgn(fc[k].x);
                eF += sgn(fa[k].y);
            }
        }
        if (fluxSums) {
            fluxSums[(size_t)i * 5 + 0] = mF;
            fluxSums[(size_t)i * 5 + 1] = eF;
            fluxSums[(size_t)i * 5 + 2] = vF[0];
            fluxSums[(size_t)i * 5 + 3] = vF[1];
            fluxSums[(size_t)i * 5 + 4] = vF[2];
        }
        double mi = m[i], ui = u[i];
        double vo[3] = {vx[i], vy[i], D == 3 ? vz[i] : 0.};
        double Q0 = D == 3 ? mi * (ui + .5 * (vo[0] * vo[0] + vo[1] * vo[1] + vo[2] * vo[2]))
                           : mi * (ui + .5 * (vo[0] * vo[0] + vo[1] * vo[1]));
        double Qv[3] = {mi * vo[0], mi * vo[1], mi * vo[2]};
        if (!p.mfm) mi -= dt * mF;
        // sign and NaN tests on the bit patterns; one reciprocal of the mass
        const long long mb_ = __double_as_longlong(mi);
        if (mb_ <= 0) st_local |= ST_NEG_MASS;   // mi <= 0 (or a negative NaN)
        const double imi = frcp(mi);
        double vn[3];
#pragma unroll
        for (int a = 0; a < D; ++a) { Qv[a] -= dt * vF[a]; vn[a] = Qv[a] * imi; }
        Q0 -= dt * eF;
        double un = D == 3 ? Q0 * imi - .5 * (vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2])
                           : Q0 * imi - .5 * (vn[0] * vn[0] + vn[1] * vn[1]);
        const long long ub = __double_as_longlong(un);
        if (ub <= 0) st_local |= ST_NEG_ENERGY;
        if ((ub & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll || (mb_ & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll)
            st_local |= ST_NAN;
        m[i] = mi;
        u[i] = un;
#pragma unroll
        for (int a = 0; a < D; ++a) Vv[a][i] = vn[a];
        double xn[3] = {0., 0., 0.};
#pragma unroll
        for (int a = 0; a < D; ++a) {
            double xa = X[a][i];
            if (p.move) {
                xa += vo[a] * dt;
                if (p.periodic) {
                    // the box tests on integer keys (ord_key), off the FP64 pipe
                    const double lo = grids[sim].lo[a], hi = grids[sim].hi[a];
                    if (dlt(xa, lo)) xa = hi - (lo - xa);
                    else if (!dlt(xa, hi)) xa = lo + (xa - hi);
                }
                X[a][i] = xa;
            }
            xn[a] = xa;
        }
        posf[i] = make_float4((float)xn[0], (float)xn[1], (float)xn[2], 0.f);
    }
    for (int o = 16; o > 0; o >>= 1) st_local |= __shfl_xor_sync(0xffffffffu, st_local, o);
    if ((threadIdx.x & 31) == 0 && st_local) flag(status, st_local);
}

// Simulation time of every member and the count of completed steps (skipped,
// like the update, when the step is to be repeated with more capacity).
__global__ void k_advance_time(int nmembers, const double *__restrict__ dt, double *__restrict__ simTime,
                               int *__restrict__ stepsDone, const unsigned *__restrict__ status) {
    if (*status & (ST_NGB_OVERFLOW | ST_CAPACITY | ST_TIMEOUT | ST_GRID)) return;
    for (int mi = blockIdx.x * blockDim.x + threadIdx.x; mi < nmembers; mi += gridDim.x * blockDim.x)
        simTime[mi] += dt[mi];
    if (blockIdx.x == 0 && threadIdx.x == 0) *stepsDone += 1;
}

template <int D>
__global__ void k_pack_posf(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                            int n, float4 *__restrict__ posf) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        posf[i] = make_float4((float)x[i], (float)y[i], D == 3 ? (float)z[i] : 0.f, 0.f);
}

// ------------------------------------------------------------------ launchers

// Particles::getDomainLimits + Domain::createGrid + assignParticlesAndCells
// (Particles.cpp:228-322, Domain.cpp:9-54): grids, cell of every particle,
// cell lists sorted by particle index.
template <int D>
void launch_binning(StepArgs &a) {
    const Params &p = a.p;
    cudaStream_t s = a.stream;
    const int T = 128;
    const int blocksN = (p.n + T - 1) / T;
    if (a.tune.persistent_binning && a.bar && a.bin_blocks > 0) {
        // one cooperative launch of at most the blocks resident at once
        cudaMemsetAsync(a.bar, 0, 2 * sizeof(unsigned), s);
        GridBar bar{a.bar, a.bar + 1, (unsigned)a.bin_blocks + a.bar_extra, a.bar_spin};
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(a.bin_blocks);
        cfg.blockDim = dim3(PB_T);
        cfg.dynamicSmemBytes = 0;
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        cudaLaunchKernelEx(&cfg, k_binning<D>, (const double *)a.x, (const double *)a.y, (const double *)a.z, p,
                           (const Member *)a.members, a.memberOf, a.nmembers, a.bpm, a.boundsPart, a.grids,
                           a.cellTotal, a.cell, a.cellCount, a.cellStart, a.cellFill, a.cellList, a.scanTiles,
                           a.scanTotal, a.status, bar);
        return;
    }
    k_bounds_partial<D><<<a.nmembers * a.bpm, BOUNDS_T, 0, s>>>(a.x, a.y, a.z, p, a.members, a.bpm, a.boundsPart);
    k_bounds_final<D><<<1, 256, 0, s>>>(a.x, a.y, a.z, a.boundsPart, a.bpm, p, a.members, a.nmembers, a.grids,
                                        a.cellTotal, a.status);
    cudaMemsetAsync(a.cellCount, 0, sizeof(int) * (size_t)(p.ncells_cap + 1), s);
    cudaMemsetAsync(a.cellFill, 0, sizeof(int) * (size_t)(p.ncells_cap + 1), s);
    k_assign<D><<<blocksN, T, 0, s>>>(a.x, a.y, a.z, p.n, a.memberOf, a.grids, a.cell, a.cellCount, a.status);
    exclusive_scan(a.cellCount, p.ncells_cap, a.cellStart, a.scanTiles, a.scanTotal, s);
    k_fill_cells<<<blocksN, T, 0, s>>>(a.cell, p.n, a.cellStart, a.cellFill, a.cellList, a.status);
    k_sort_cells<<<(p.ncells_cap + T - 1) / T, T, 0, s>>>(a.cellTotal, a.cellStart, a.cellList, a.status);
}

// Smoothing lengths of every particle on the current grid (k_hsolve).
template <int D>
void launch_hsolve(StepArgs &a) {
    const Params &p = a.p;
    cudaStream_t s = a.stream;
    cudaMemsetAsync(a.hstat, 0, 2 * sizeof(unsigned long long), s);
    const int warps_total = a.sm_count * a.tune.nns_warps_per_sm;
    const int blocks = (warps_total + NNS_WARPS - 1) / NNS_WARPS;
    const size_t smem = hsolve_smem_bytes(p.K);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_hsolve<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_hsolve<D><<<blocks, NNS_WARPS * 32, smem, s>>>(p, a.members, a.memberOf, a.grids, a.x, a.y, a.z, a.posf, a.cellTotal,
                                                     a.cellStart, a.cellList, a.hp, a.hpf, a.neff, a.hstat, a.status);
}

template <int D>
void launch_step(StepArgs &a) {
    const Params &p = a.p;
    cudaStream_t s = a.stream;
    const int T = 128;
    const int blocksN = (p.n + T - 1) / T;
    auto tick = [&](int id) { if (a.timer) a.timer(a.timer_ctx, id, 0); };
    auto tock = [&](int id) { if (a.timer) a.timer(a.timer_ctx, id, 1); };

    tick(KT_GRID);
    launch_binning<D>(a);
    tock(KT_GRID);

    if (p.adaptive_h) {
        tick(KT_HSOLVE);
        launch_hsolve<D>(a);
        tock(KT_HSOLVE);
    }

    tick(KT_NNS);
    {
        const int warps_total = a.sm_count * a.tune.nns_warps_per_sm;   // grid-stride, one warp per cell
        const int blocks = (warps_total + NNS_WARPS - 1) / NNS_WARPS;
        const size_t smem = nns_smem_bytes(p.K, p.adaptive_h);
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(k_neighbours<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_neighbours<D><<<blocks, NNS_WARPS * 32, smem, s>>>(
            p, a.members, a.memberOf, a.grids, a.x, a.y, a.z, a.posf, a.vx, a.vy, a.vz, a.m, a.u, a.cellTotal,
            a.cellStart, a.cellList, a.nbr, a.rr, a.ww, a.noi, a.noiImg, a.faceCnt, a.prim, a.geo, a.velf, a.status);
    }
    tock(KT_NNS);

    // the face links (integer work) need only the neighbour lists: without
    // per-kernel timing they run on the second stream while the time step and
    // the gradients keep the FP64 pipe busy
    // link_overlap 2: the links inside the gradients kernel (after the scan of
    // the canonical counts); 1: on the second stream beside the gradients;
    // 0: in order
    const bool fused = a.tune.link_overlap == 2 && !a.stop_after_gradients;
    const bool overlap = !fused && a.stream2 && !a.timer && !a.stop_after_gradients && a.tune.link_overlap == 1;
    const int blocksLink = blocksN;
    auto launch_links = [&](cudaStream_t ls) {
        exclusive_scan(a.faceCnt, p.n, a.faceOff, a.scanTiles, a.scanTotal, ls);
        cudaMemsetAsync(a.faces, 0xff, sizeof(FaceRef) * a.faces_cap, ls);
        k_link<<<blocksLink, T, 0, ls>>>(p, a.nbr, a.noi, a.noiImg, a.faceOff, a.faceOf, a.faces, a.status);
    };
    if (overlap) {
        cudaEventRecord(a.ev_fork, s);
        cudaStreamWaitEvent(a.stream2, a.ev_fork, 0);
        launch_links(a.stream2);
        cudaEventRecord(a.ev_join, a.stream2);
    }

    // the time step runs inside the gradients' first neighbour pass
    // (k_gradients with dtbits; k_timestep, the separate kernel of the same
    // arithmetic, is the fallback when the time step is timed on its own)
    const int gT = a.tune.grad_threads;
    cudaMemsetAsync(a.dtbits, 0xff, sizeof(unsigned long long) * (size_t)a.nmembers, s);
    // with the single-precision filters the gradients kernel bounds every
    // particle's dt (dtlo, and the least upper bound per simulation in dtcap,
    // 0x7F7F7F7F = 3.4e38 to start) and k_timestep evaluates v_sig in FP64
    // for the particles whose bound reaches it
    const bool dt_filter = p.adaptive && !a.separate_dt && (a.tune.fp32_filters & MLH_FILTER_TIMESTEP) && a.velf &&
                           a.dtlo && a.dtcap;
    if (dt_filter) cudaMemsetAsync(a.dtcap, 0x7f, sizeof(unsigned) * (size_t)a.nmembers, s);
    if (a.separate_dt) {
        tick(KT_DT);
        k_timestep<D><<<(p.n + 255) / 256, 256, 0, s>>>(p, a.members, a.memberOf, a.prim, a.geo, a.nbr, a.rr,
                                                        a.noi, a.dtbits, nullptr, nullptr);
        tock(KT_DT);
    }
    tick(KT_GRAD);
    if (fused) {
        exclusive_scan(a.faceCnt, p.n, a.faceOff, a.scanTiles, a.scanTotal, s);
        cudaMemsetAsync(a.faces, 0xff, sizeof(FaceRef) * a.faces_cap, s);
    }
    k_gradients<D><<<(p.n + gT - 1) / gT, gT, 0, s>>>(p, a.members, a.memberOf, a.grids, a.prim, a.geo, a.nbr, a.ww,
                                                      a.rr, a.noi, a.noiImg, a.grad, a.gradRaw, a.psi,
                                                      (p.adaptive && !a.separate_dt && !dt_filter) ? a.dtbits : nullptr,
                                                      fused ? a.faceOff : nullptr, a.faceOf, a.faces, a.status,
                                                      a.posf, a.tune.fp32_filters, a.velf, dt_filter ? a.dtlo : nullptr,
                                                      a.dtcap);
    if (dt_filter)
        k_timestep<D><<<(p.n + 255) / 256, 256, 0, s>>>(p, a.members, a.memberOf, a.prim, a.geo, a.nbr, a.rr,
                                                        a.noi, a.dtbits, a.dtlo, a.dtcap);
    k_dt_final<<<(a.nmembers + 127) / 128, 128, 0, s>>>(p, a.nmembers, a.dtbits, a.dt_max, a.dt);
    tock(KT_GRAD);
    if (a.stop_after_gradients) return;

    if (overlap) {
        cudaStreamWaitEvent(s, a.ev_join, 0);
    } else if (!fused) {
        tick(KT_LINK);
        launch_links(s);
        tock(KT_LINK);
    }

    tick(KT_FACES);
    const int fT = a.tune.face_threads, fB = a.sm_count * a.tune.face_blocks_per_sm;
    Params pf = p;   // the face passes see the tuned split
    pf.face_split = a.tune.face_split;
    const FaceQueue qa{a.fstate, a.queueFace, a.queueCount, a.qcap};
    const FaceQueue qb{a.fstate2, a.queueFace2, a.queueCount2, a.qcap2};
#define MLH_FACES(R5, MODE, QA, QB)                                                                              \
    k_faces<D, R5, MODE><<<fB, fT, 0, s>>>(pf, a.members, a.memberOf, a.grids, a.prim, a.geo, a.grad, a.nbr, a.psi, \
                                           a.faceOff + p.n, a.faces, a.dt, a.Fface, a.newtonSum, a.status, QA,   \
                                           QB, a.feat, a.yguess, a.harvest)
    if (a.learned) {
        // strong shocks: network guess (queue A); the rest as the plain step
        cudaMemsetAsync(a.queueCount, 0, sizeof(int), s);
        if (a.queueCount2) cudaMemsetAsync(a.queueCount2, 0, sizeof(int), s);
        if (a.root5 && a.tune.face_split == 2) {
            // unfinished faces continued inside the block, strong shocks from
            // the network's guess evaluated there
            k_faces_block<D, true><<<fB, FB_T, 0, s>>>(pf, a.members, a.memberOf, a.grids, a.prim, a.geo, a.grad,
                                                       a.nbr, a.psi, a.faceOff + p.n, a.faces, a.dt, a.Fface,
                                                       a.newtonSum, a.status, (const PackedMlp *)a.mlp_packed);
        } else {
            if (a.root5) MLH_FACES(true, 1, qa, qb);
            else MLH_FACES(false, 1, qa, qb);
            pstar_infer_dev(a.feat, a.queueCount, (int)a.faces_cap, a.mlp_packed, a.yguess, a.sm_count, s);
            if (a.root5) MLH_FACES(true, 2, qa, qb); else MLH_FACES(false, 2, qa, qb);
            if (a.root5 && a.fstate2 && a.tune.face_split == 1) MLH_FACES(true, 4, qb, qb);
        }
    } else if (a.root5 && a.harvest.stride == 0 && a.tune.face_split == 2) {
        // unconverged faces after one Newton step continued inside the block
        k_faces_block<D, false><<<fB, FB_T, 0, s>>>(pf, a.members, a.memberOf, a.grids, a.prim, a.geo, a.grad, a.nbr,
                                                    a.psi, a.faceOff + p.n, a.faces, a.dt, a.Fface, a.newtonSum,
                                                    a.status, nullptr);
    } else if (a.root5 && a.fstate && a.harvest.stride == 0 && a.tune.face_split) {
        // unconverged faces after one Newton step go to a second, dense pass
        cudaMemsetAsync(a.queueCount, 0, sizeof(int), s);
        MLH_FACES(true, 3, qa, qb);
        MLH_FACES(true, 4, qa, qb);
    } else {
        if (a.root5) MLH_FACES(true, 0, qa, qb); else MLH_FACES(false, 0, qa, qb);
    }
#undef MLH_FACES
    tock(KT_FACES);

    tick(KT_UPDATE);
    k_update<D><<<blocksN, T, 0, s>>>(p, a.memberOf, a.grids, a.noi, a.noiImg, a.faceOf, a.Fface, a.dt, a.x, a.y,
                                      a.z, a.vx, a.vy, a.vz, a.m, a.u, a.posf, a.fluxSums, a.status);
    k_advance_time<<<(a.nmembers + 127) / 128, 128, 0, s>>>(a.nmembers, a.dt, a.simTime, a.stepsDone, a.status);
    tock(KT_UPDATE);
}

void launch_grid_bounds(const double *x, const double *y, const double *z, const Params &p,
                        const Member *members, int nmembers, int bpm, double *partials, GridInfo *grids,
                        int *cellTotal, unsigned *status, cudaStream_t s) {
    const int blocks = nmembers * bpm;
    if (p.dim == 2) {
        k_bounds_partial<2><<<blocks, BOUNDS_T, 0, s>>>(x, y, z, p, members, bpm, partials);
        k_bounds_final<2><<<1, 256, 0, s>>>(x, y, z, partials, bpm, p, members, nmembers, grids, cellTotal, status);
    } else {
        k_bounds_partial<3><<<blocks, BOUNDS_T, 0, s>>>(x, y, z, p, members, bpm, partials);
        k_bounds_final<3><<<1, 256, 0, s>>>(x, y, z, partials, bpm, p, members, nmembers, grids, cellTotal, status);
    }
}

int binning_blocks(int dim, int sm_count) {
    int per_sm = 0;
    cudaError_t e = dim == 3 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_binning<3>, PB_T, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_binning<2>, PB_T, 0);
    if (e != cudaSuccess || per_sm < 1) return 0;
    return per_sm * sm_count;
}

void step(StepArgs &a) {
    if (a.p.dim == 2) launch_step<2>(a);
    else launch_step<3>(a);
}

void smoothing_lengths(StepArgs &a) {
    if (a.p.dim == 2) { launch_binning<2>(a); launch_hsolve<2>(a); }
    else { launch_binning<3>(a); launch_hsolve<3>(a); }
}

void pack_posf(const double *x, const double *y, const double *z, int n, int dim, float4 *posf, cudaStream_t s) {
    int blocks = (n + 255) / 256;
    if (blocks < 1) blocks = 1;
    if (dim == 2) k_pack_posf<2><<<blocks, 256, 0, s>>>(x, y, z, n, posf);
    else k_pack_posf<3><<<blocks, 256, 0, s>>>(x, y, z, n, posf);
}

const char *kernel_timer_name(int id) {
    switch (id) {
        case KT_GRID: return "grid_bin";
        case KT_NNS: return "neighbours_density";
        case KT_DT: return "timestep";
        case KT_GRAD: return "gradients_limiter";
        case KT_LINK: return "face_links";
        case KT_FACES: return "faces_riemann";
        case KT_UPDATE: return "gather_update";
        case KT_HSOLVE: return "smoothing_lengths";
    }
    return "?";
}

}  // namespace mlh
