// Allocation-free variant of the grid-bounds reduction.
//
// Some callers cannot call cudaMalloc: a host framework that owns all device
// memory through its own pool and forbids raw allocations, or a real-time loop
// that must not allocate after start-up.  For them mlh_grid_bounds_noalloc
// computes the search grid of the reference's non-periodic step
// (Particles::getDomainLimits with its quirks + Domain::createGrid) from
// caller-owned device arrays, with its scratch in the file-scope device array
// below instead of memory from cudaMalloc.
#include "../../include/mlh.h"
#include "mlh_kernels.h"

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

using namespace mlh;

namespace {

// 16 KiB of scratch on every device that loads the library, kept until exit:
// BOUNDS_BLOCKS * 6 doubles of per-block partials, then the GridInfo result,
// the status word, the simulation's parameters and the cell count, each on a
// 256-byte boundary.
constexpr size_t SCRATCH_BYTES = 16384;
constexpr size_t PARTIALS_BYTES = sizeof(double) * 6 * BOUNDS_BLOCKS;
constexpr size_t GRID_OFFSET = (PARTIALS_BYTES + 255) / 256 * 256;
constexpr size_t STATUS_OFFSET = GRID_OFFSET + (sizeof(GridInfo) + 255) / 256 * 256;
constexpr size_t MEMBER_OFFSET = STATUS_OFFSET + 256;
constexpr size_t CELLS_OFFSET = MEMBER_OFFSET + (sizeof(Member) + 255) / 256 * 256;
static_assert(CELLS_OFFSET + sizeof(int) <= SCRATCH_BYTES, "scratch too small");

static __device__ __align__(256) unsigned char g_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_mutex;
void *g_scratch_addr[MAX_DEVICES] = {nullptr};
// message for mlh_last_error()
struct ErrorSink {
    void operator=(const std::string &m) { set_last_error(m.c_str()); }
    void operator=(const char *m) { set_last_error(m); }
} g_error;

// Device address of g_scratch on the current device, looked up once per device.
int scratch_address(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { g_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e); return MLH_ERR_NO_DEVICE; }
    if (dev < 0 || dev >= MAX_DEVICES) { g_error = "device index out of range"; return MLH_ERR_CAPACITY; }
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void *ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_scratch);
        if (e != cudaSuccess || !ptr) {
            g_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
            return MLH_ERR_CUDA;
        }
        g_scratch_addr[dev] = ptr;
    }
    *out = g_scratch_addr[dev];
    return 0;
}

__global__ void k_set_member(Member m, Member *__restrict__ dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = m;
}

__global__ void k_grid_to_doubles(const GridInfo *__restrict__ g, int dim, double *__restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    for (int a = 0; a < 3; ++a) {
        out[a] = a < dim ? g->lo[a] : 0.;
        out[3 + a] = a < dim ? g->hi[a] : 0.;
        out[6 + a] = a < dim ? (double)g->cells[a] : 0.;
    }
}

}  // namespace

extern "C" int mlh_grid_bounds_noalloc(int dim, int periodic, int n, const double *x, const double *y,
                                       const double *z, const double *box_lo, const double *box_hi,
                                       double kernel_size, double *grid_out, void *stream) {
    if (dim != 2 && dim != 3) { g_error = "dim must be 2 or 3"; return MLH_ERR_INVALID; }
    if (n < 1) { g_error = "n must be >= 1"; return MLH_ERR_INVALID; }
    if (n > MLH_NOALLOC_MAX_PARTICLES) {
        g_error = "n exceeds MLH_NOALLOC_MAX_PARTICLES (2^29 - 1)";
        return MLH_ERR_CAPACITY;
    }
    if (!x || !y || (dim == 3 && !z) || !grid_out) { g_error = "null device pointer"; return MLH_ERR_INVALID; }
    if (!(kernel_size > 0.) || !std::isfinite(kernel_size)) { g_error = "kernel_size must be > 0"; return MLH_ERR_INVALID; }
    if (periodic && (!box_lo || !box_hi)) { g_error = "periodic runs need box_lo and box_hi"; return MLH_ERR_INVALID; }
    // an error left pending by the caller's earlier work is reported, not
    // consumed: cudaPeekAtLastError leaves it for the caller to read
    cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        g_error = std::string("a CUDA error from earlier work is pending: ") + cudaGetErrorString(pending);
        return MLH_ERR_CUDA;
    }
    void *base = nullptr;
    if (int rc = scratch_address(&base)) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    double *partials = (double *)base;
    GridInfo *grid = (GridInfo *)((unsigned char *)base + GRID_OFFSET);
    unsigned *status = (unsigned *)((unsigned char *)base + STATUS_OFFSET);
    Member *member = (Member *)((unsigned char *)base + MEMBER_OFFSET);
    int *cellTotal = (int *)((unsigned char *)base + CELLS_OFFSET);

    Params p;
    std::memset(&p, 0, sizeof(p));
    p.n = n;
    p.dim = dim;
    p.periodic = periodic ? 1 : 0;
    p.h = kernel_size;
    p.ncells_cap = 0x7fffffff;
    for (int a = 0; a < 3; ++a) {
        p.box_lo[a] = (periodic && a < dim) ? box_lo[a] : 0.;
        p.box_hi[a] = (periodic && a < dim) ? box_hi[a] : 0.;
    }
    // the status word accumulates flags with atomicOr, so it starts at zero;
    // the partials and the GridInfo are overwritten completely
    cudaError_t e = cudaMemsetAsync(status, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) { g_error = std::string("cudaMemsetAsync: ") + cudaGetErrorString(e); return MLH_ERR_CUDA; }
    Member mb;
    std::memset(&mb, 0, sizeof(mb));
    mb.h = kernel_size;
    mb.first = 0;
    mb.count = n;
    for (int a = 0; a < 3; ++a) { mb.box_lo[a] = p.box_lo[a]; mb.box_hi[a] = p.box_hi[a]; }
    k_set_member<<<1, 1, 0, s>>>(mb, member);
    launch_grid_bounds(x, y, dim == 3 ? z : x, p, member, 1, BOUNDS_BLOCKS, partials, grid, cellTotal, status, s);
    k_grid_to_doubles<<<1, 1, 0, s>>>(grid, dim, grid_out);
    // launch errors of the kernels above (none was pending on entry)
    e = cudaGetLastError();
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&st, status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { g_error = std::string("CUDA: ") + cudaGetErrorString(e); return MLH_ERR_CUDA; }
    int rc = 0;
    std::string msg;
    if (st & ST_GRID) {
        rc |= MLH_ERR_GRID;
        msg = "degenerate grid (fewer than 1 cell per axis, or fewer than 3 on a periodic axis)";
    }
    if (st & ST_CAPACITY) {
        rc |= MLH_ERR_CAPACITY;
        if (!msg.empty()) msg += "; ";
        msg += "too many cells (the grid needs more than 2^31 - 1 cells of size kernel_size)";
    }
    if (rc) g_error = msg;
    return rc;
}
