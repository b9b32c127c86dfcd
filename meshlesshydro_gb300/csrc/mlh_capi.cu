// C ABI of the MFV step (include/mlh.h): context, device memory, copies,
// step driver with capacity retries, parity dumps and kernel timing.
#include "../../include/mlh.h"
#include "mlh_kernels.h"
#include "mlh_pstar.h"
#include "mlh_riemann.cuh"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

using namespace mlh;

namespace {

thread_local std::string g_last_error;

int cuda_fail(cudaError_t e, const char *what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return MLH_ERR_CUDA;
}

#define CK(call)                                          \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// the smallest float >= x (x finite, positive)
float float_up(double x) {
    float f = (float)x;
    if ((double)f < x) f = std::nextafter(f, INFINITY);
    return f;
}

template <class T>
cudaError_t dalloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, sizeof(T) * count);
}

}  // namespace

namespace mlh {
// message for mlh_last_error from other translation units of the library
void set_last_error(const char *msg) { g_last_error = msg ? msg : ""; }
}  // namespace mlh

struct mlh_ctx {
    mlh_config cfg;
    Params p;
    int n = 0;
    int device = 0;
    int sm_count = 152;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;              // face links, overlapped
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // state
    double *x = nullptr, *y = nullptr, *z = nullptr, *vx = nullptr, *vy = nullptr, *vz = nullptr, *m = nullptr, *u = nullptr;
    float4 *posf = nullptr;
    float4 *velf = nullptr;       // velocity and sound speed in single precision
    float *dtlo = nullptr;        // time-step filter: lower bound on each particle's dt
    unsigned *dtcap = nullptr;    // and the least upper bound of each simulation
    // simulations held by the context (1, or an ensemble stored back to back)
    int nmembers = 1;
    int bpm = 1;
    std::vector<Member> hmembers;
    Member *members = nullptr;
    int *memberOf = nullptr;
    // grids (one per member)
    GridInfo *grids = nullptr;
    int *cellTotal = nullptr;
    double *boundsPart = nullptr;
    int *cell = nullptr, *cellCount = nullptr, *cellStart = nullptr, *cellFill = nullptr, *cellList = nullptr;
    // neighbours (capacity K slots per particle)
    uint32_t *nbr = nullptr;
    double *rr = nullptr, *ww = nullptr, *psi = nullptr;
    size_t faces_cap = 0;
    size_t queue_cap = 0, queue_cap2 = 0;
    int *noi = nullptr, *noiImg = nullptr, *faceCnt = nullptr, *faceOff = nullptr, *faceOf = nullptr;
    FaceRef *faces = nullptr;
    double *Fface = nullptr;
    Prim *prim = nullptr;
    Geo *geo = nullptr;
    Grad *grad = nullptr, *gradRaw = nullptr;
    double *fluxSums = nullptr;
    // per-particle smoothing lengths and the effective neighbour number of
    // the last solve; counters [iterations, clamped]
    double *hp = nullptr, *neff = nullptr;
    float *hpf = nullptr;
    unsigned long long *hstat = nullptr;
    // scalars
    unsigned *status = nullptr;
    unsigned long long *dtbits = nullptr, *newtonSum = nullptr;
    double *dt = nullptr, *simTime = nullptr;
    int *stepsDone = nullptr;
    int *scanTiles = nullptr, *scanTotal = nullptr;
    bool debug_arrays = true;
    Tuning tune;
    // learned p* guess
    bool learned = false;
    float *mlp_w = nullptr;
    void *mlp_packed = nullptr;
    FaceState *fstate = nullptr, *fstate2 = nullptr;
    int *queueFace2 = nullptr, *queueCount2 = nullptr;
    float4 *feat = nullptr;
    float *yguess = nullptr;
    int *queueFace = nullptr;   // faces handed to the network (learned guess)
    int *queueCount = nullptr;
    Harvest harvest{};
    // CUDA graph of one step, replayed by mlh_step in graph mode
    bool graph_mode = false;
    cudaGraphExec_t graph_exec = nullptr;
    double graph_dt_max = -1.;
    // persistent binning: grid-barrier words, resident blocks, test-hook
    // settings of the barriers
    unsigned *bar = nullptr;
    int bin_blocks = 0;
    unsigned bar_extra = 0, bar_spin = 0;
    // kernel timing
    bool timing = false;
    std::vector<cudaEvent_t> tev;   // pairs, in launch order
    std::vector<int> tid;
    double kt_ms[KT_COUNT] = {0};
    long long kt_launches[KT_COUNT] = {0};
};

namespace {

int round_slots(int k) { return (k + 3) & ~3; }

void free_neighbour_buffers(mlh_ctx *c) {
    cudaFree(c->nbr); cudaFree(c->rr); cudaFree(c->ww); cudaFree(c->psi); cudaFree(c->faceOf); cudaFree(c->faces);
    cudaFree(c->Fface);
    cudaFree(c->fstate); cudaFree(c->feat); cudaFree(c->yguess); cudaFree(c->queueFace); cudaFree(c->queueCount);
    cudaFree(c->fstate2); cudaFree(c->queueFace2); cudaFree(c->queueCount2);
    c->queueFace = nullptr; c->queueCount = nullptr;
    c->fstate2 = nullptr; c->queueFace2 = nullptr; c->queueCount2 = nullptr;
    c->nbr = nullptr; c->rr = nullptr; c->ww = nullptr; c->psi = nullptr; c->faceOf = nullptr; c->faces = nullptr;
    c->Fface = nullptr; c->fstate = nullptr; c->feat = nullptr; c->yguess = nullptr;
}

// Face ids and face offsets are 32-bit: the face table may hold at most
// 2^31 - 1 faces (half the neighbour slots, plus one per particle).
size_t face_capacity(long long n, int K) { return (size_t)n * (size_t)K / 2 + (size_t)n + 16; }
constexpr size_t MAX_FACES = 0x7fffffff;

int alloc_neighbour_buffers(mlh_ctx *c) {
    size_t slots = (size_t)c->n * c->p.K;
    size_t faces = face_capacity(c->n, c->p.K);
    if (faces > MAX_FACES) {
        g_last_error = "too many faces for 32-bit face ids (particles x neighbour slots / 2 above 2^31 - 1)";
        return MLH_ERR_CAPACITY;
    }
    CK(dalloc(&c->nbr, slots));
    CK(dalloc(&c->rr, slots));
    CK(dalloc(&c->ww, slots));
    CK(dalloc(&c->psi, slots * 3));
    c->faces_cap = faces;
    CK(dalloc(&c->faceOf, slots));
    CK(dalloc(&c->faces, faces));
    CK(dalloc(&c->Fface, faces * 6));
    // queues of faces for second face passes.  A: in the plain step the
    // faces Newton has not finished after one step (a fifth to two thirds of
    // them; faces_cap is about twice the faces of a step; a full queue
    // finishes its faces in the first pass); with the learned guess the
    // strong shocks handed to the network (room for every face).  B (learned
    // guess only): the faces Newton has not finished after one step.
    const size_t half = faces / 2 + 1024;
    c->queue_cap = c->learned ? faces : half;
    CK(dalloc(&c->fstate, c->queue_cap));
    CK(dalloc(&c->queueFace, c->queue_cap));
    CK(dalloc(&c->queueCount, 1));
    c->queue_cap2 = 0;
    if (c->learned) {
        CK(dalloc(&c->feat, faces));
        CK(dalloc(&c->yguess, faces));
        c->queue_cap2 = half;
        CK(dalloc(&c->fstate2, half));
        CK(dalloc(&c->queueFace2, half));
        CK(dalloc(&c->queueCount2, 1));
    }
    return 0;
}

void free_cell_buffers(mlh_ctx *c) {
    cudaFree(c->cellCount); cudaFree(c->cellStart); cudaFree(c->cellFill);
    c->cellCount = c->cellStart = c->cellFill = nullptr;
}

int alloc_cell_buffers(mlh_ctx *c) {
    size_t nc = (size_t)c->p.ncells_cap + 1;
    CK(dalloc(&c->cellCount, nc));
    CK(dalloc(&c->cellStart, nc + 1));
    CK(dalloc(&c->cellFill, nc));
    // tile sums of the scans over the cell counts and over the particles
    cudaFree(c->scanTiles);
    const size_t m = nc > (size_t)c->n ? nc : (size_t)c->n;
    CK(dalloc(&c->scanTiles, m / 4096 + 1024));
    return 0;
}

long long estimate_cells(const mlh_config &cfg, const mlh_particles_view *v, const Member &mb) {
    double lo[3], hi[3];
    const double *X[3] = {v->x, v->y, v->z};
    long long total = 1;
    for (int a = 0; a < cfg.dim; ++a) {
        if (cfg.periodic) { lo[a] = mb.box_lo[a]; hi[a] = mb.box_hi[a]; }
        else {
            lo[a] = hi[a] = X[a][mb.first];
            for (int i = mb.first + 1; i < mb.first + mb.count; ++i) {
                lo[a] = std::fmin(lo[a], X[a][i]);
                hi[a] = std::fmax(hi[a], X[a][i]);
            }
        }
        double c = std::floor((hi[a] - lo[a]) / mb.h);
        long long ci = c >= 1. ? (long long)c : 1;
        if (!cfg.periodic) ci = ci + ci / 4 + 4;   // room for an expanding bounding box
        total *= ci;
    }
    return total;
}

// Kernel::cubicSpline normalisation (demonstrator/src/Particles.cpp:10-15)
// and the other per-simulation constants.
Member make_member(const mlh_config &f, double h, const double *lo, const double *hi, int first, int count) {
    Member m;
    std::memset(&m, 0, sizeof(m));
    m.h = h;
    m.hsq = h * h;
    m.h2 = h / 2.;
    m.ih2 = 1. / m.h2;
    const double h2 = m.h2;
    m.sigma = f.dim == 2 ? 10. / (7. * M_PI * h2 * h2) : 1. / (M_PI * h2 * h2 * h2);
    m.w0 = m.sigma * (1. - 3. / 2. * 0. * 0. * (1. - 0. / 2.));
    m.cfl_h = f.cfl * h;
    // single-precision pre-filter bound: positions rounded to float move a
    // distance of ~1e-7 relative to the box; 1e-3 relative on h^2 is ample
    m.hsq_f = (float)(m.hsq * (1. + 1e-3));
    for (int a = 0; a < 3; ++a) { m.box_lo[a] = lo[a]; m.box_hi[a] = hi[a]; }
    m.first = first;
    m.count = count;
    return m;
}

void timer_cb(void *vc, int id, int phase) {
    mlh_ctx *c = (mlh_ctx *)vc;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, c->stream);
    c->tev.push_back(e);
    if (phase == 0) c->tid.push_back(id);
}

void collect_timers(mlh_ctx *c) {
    for (size_t k = 0; k + 1 < c->tev.size(); k += 2) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->tev[k], c->tev[k + 1]);
        int id = c->tid[k / 2];
        c->kt_ms[id] += ms;
        c->kt_launches[id] += 1;
    }
    for (auto e : c->tev) cudaEventDestroy(e);
    c->tev.clear();
    c->tid.clear();
}

StepArgs make_args(mlh_ctx *c, double dt_max) {
    StepArgs a{};   // zeroed pointers and counts, the tuning's defaults
    a.p = c->p;
    a.stream = c->stream;
    a.stream2 = c->stream2;
    a.ev_fork = c->ev_fork;
    a.ev_join = c->ev_join;
    a.tune = c->tune;
    a.face_blocks = c->sm_count * 8;
    a.sm_count = c->sm_count;
    a.faces_cap = c->faces_cap;
    a.p.faces_cap = c->faces_cap > 0x7fffffff ? 0x7fffffff : (int)c->faces_cap;
    a.qcap = c->queue_cap > 0x7fffffff ? 0x7fffffff : (int)c->queue_cap;
    a.qcap2 = c->queue_cap2 > 0x7fffffff ? 0x7fffffff : (int)c->queue_cap2;
    a.root5 = make_riemann_consts(c->p.gamma, c->p.rtol, c->p.rmaxit).root5;
    a.dt_max = dt_max;
    a.x = c->x; a.y = c->y; a.z = c->z; a.vx = c->vx; a.vy = c->vy; a.vz = c->vz; a.m = c->m; a.u = c->u;
    a.posf = c->posf;
    a.velf = c->velf; a.dtlo = c->dtlo; a.dtcap = c->dtcap;
    a.nmembers = c->nmembers; a.bpm = c->bpm;
    a.members = c->members; a.memberOf = c->memberOf;
    a.grids = c->grids; a.cellTotal = c->cellTotal; a.boundsPart = c->boundsPart;
    a.cell = c->cell; a.cellCount = c->cellCount; a.cellStart = c->cellStart; a.cellFill = c->cellFill;
    a.cellList = c->cellList;
    a.nbr = c->nbr; a.rr = c->rr; a.ww = c->ww; a.psi = c->psi;
    a.noi = c->noi; a.noiImg = c->noiImg; a.faceCnt = c->faceCnt; a.faceOff = c->faceOff; a.faceOf = c->faceOf;
    a.faces = c->faces;
    a.prim = c->prim; a.geo = c->geo; a.grad = c->grad; a.gradRaw = c->debug_arrays ? c->gradRaw : nullptr;
    a.Fface = c->Fface; a.fluxSums = c->debug_arrays ? c->fluxSums : nullptr;
    a.status = c->status; a.dtbits = c->dtbits; a.newtonSum = c->newtonSum;
    a.dt = c->dt; a.simTime = c->simTime; a.stepsDone = c->stepsDone;
    a.scanTiles = c->scanTiles; a.scanTotal = c->scanTotal;
    a.learned = (c->learned && c->tune.learned_guess) ? 1 : 0;
    a.fstate = c->fstate; a.feat = c->feat; a.yguess = c->yguess;
    a.queueFace = c->queueFace; a.queueCount = c->queueCount; a.mlp_packed = c->mlp_packed;
    a.fstate2 = c->fstate2; a.queueFace2 = c->queueFace2; a.queueCount2 = c->queueCount2;
    a.harvest = c->harvest;
    a.bar = c->bar;
    a.bin_blocks = c->bin_blocks;
    a.bar_extra = c->bar_extra;
    a.bar_spin = c->bar_spin ? c->bar_spin : (1u << 21);   // polls of ~0.3 us: about half a second
    a.hp = c->hp; a.neff = c->neff; a.hstat = c->hstat; a.hpf = c->hpf;
    a.p.hp = c->hp; a.p.hpf = c->hpf;
    a.timer = c->timing ? timer_cb : nullptr;
    a.timer_ctx = c;
    return a;
}

// Target of S = sum_j f(2 r_ij / h_i) for an effective neighbour number
// n_ngb: n_ngb / K_D - 1 (K_D = 32/3 in 3D, 40/7 in 2D, the count of the
// particle itself).
double sngb_target(int dim, double n_ngb) {
    const double KD = dim == 3 ? 32. / 3. : 40. / 7.;
    return n_ngb / KD - 1.;
}

void fill_params(mlh_ctx *c) {
    const mlh_config &f = c->cfg;
    Params &p = c->p;
    p.n = c->n;
    p.dim = f.dim;
    p.periodic = f.periodic;
    p.adaptive = f.adaptive_timestep;
    p.slope = f.slope_limiting;
    p.pairwise = f.pairwise_limiter;
    p.mfm = f.meshless_finite_mass;
    p.move = f.move_particles;
    p.foqp = f.first_order_quad_point;
    p.int_abs = f.int_abs;
    p.img_pw = f.image_pairwise_limiter;
    p.rmaxit = f.riemann_max_iter > 0 ? f.riemann_max_iter : 100;
    p.h = f.kernel_size;
    p.hsq = f.kernel_size * f.kernel_size;
    p.h2 = f.kernel_size / 2.;
    // Kernel::cubicSpline normalisation, demonstrator/src/Particles.cpp:10-15
    const double h2 = p.h2;
    p.sigma = f.dim == 2 ? 10. / (7. * M_PI * h2 * h2) : 1. / (M_PI * h2 * h2 * h2);
    p.w0 = p.sigma * (1. - 3. / 2. * 0. * 0. * (1. - 0. / 2.));
    p.gamma = f.gamma;
    p.cfl_h = f.cfl * f.kernel_size;
    p.beta = f.beta;
    p.psi1 = f.psi1;
    p.psi2 = f.psi2;
    p.rtol = f.riemann_tol > 0. ? f.riemann_tol : 1e-10;
    p.time_step = f.time_step;
    for (int a = 0; a < 3; ++a) { p.box_lo[a] = f.box_lo[a]; p.box_hi[a] = f.box_hi[a]; }
    // single-precision pre-filter bound: positions rounded to float move a
    // distance of ~1e-7 relative to the box; 1e-3 relative on h^2 is ample
    p.hsq_f = (float)(p.hsq * (1. + 1e-3));
    p.adaptive_h = f.adaptive_h;
    p.cfl = f.cfl;
    p.sngb_t = sngb_target(f.dim, f.n_ngb);
}

int upload(mlh_ctx *c, const mlh_particles_view *v) {
    size_t b = sizeof(double) * (size_t)c->n;
    CK(cudaMemcpyAsync(c->x, v->x, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->y, v->y, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->vx, v->vx, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->vy, v->vy, b, cudaMemcpyHostToDevice, c->stream));
    if (c->cfg.dim == 3) {
        CK(cudaMemcpyAsync(c->z, v->z, b, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->vz, v->vz, b, cudaMemcpyHostToDevice, c->stream));
    } else {
        CK(cudaMemsetAsync(c->z, 0, b, c->stream));
        CK(cudaMemsetAsync(c->vz, 0, b, c->stream));
    }
    CK(cudaMemcpyAsync(c->m, v->m, b, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->u, v->u, b, cudaMemcpyHostToDevice, c->stream));
    pack_posf(c->x, c->y, c->z, c->n, c->cfg.dim, c->posf, c->stream);
    CK(cudaGetLastError());
    return 0;
}

}  // namespace

extern "C" {

int mlh_abi_version(void) { return MLH_ABI_VERSION; }
const char *mlh_last_error(void) { return g_last_error.c_str(); }

static int create_impl(const mlh_config *cfg, int nmembers, const mlh_member *mdesc, const mlh_particles_view *init,
                       mlh_ctx **out) {
    if (!cfg || !init || !out) { g_last_error = "null argument"; return MLH_ERR_INVALID; }
    *out = nullptr;
    if ((cfg->dim != 2 && cfg->dim != 3) || init->n < 1 || !init->x || !init->y || !init->vx || !init->vy ||
        !init->m || !init->u || (cfg->dim == 3 && (!init->z || !init->vz)) || nmembers < 1) {
        g_last_error = "invalid configuration or particle view";
        return MLH_ERR_INVALID;
    }
    if (init->n > (int)IDX_MASK) { g_last_error = "too many particles"; return MLH_ERR_CAPACITY; }
    if (face_capacity(init->n, round_slots(cfg->max_neighbours > 0 ? cfg->max_neighbours : (cfg->dim == 2 ? 40 : 64))) >
        MAX_FACES) {
        g_last_error = "too many faces for 32-bit face ids (particles x neighbour slots / 2 above 2^31 - 1)";
        return MLH_ERR_CAPACITY;
    }
    if (cfg->adaptive_h && !(sngb_target(cfg->dim, cfg->n_ngb) > 0.)) {
        g_last_error = "adaptive_h needs n_ngb above the particle's own count (32/3 in 3D, 40/7 in 2D)";
        return MLH_ERR_INVALID;
    }
    std::vector<Member> mem;
    {
        int first = 0;
        for (int k = 0; k < nmembers; ++k) {
            const double h = mdesc ? mdesc[k].kernel_size : cfg->kernel_size;
            const int cnt = mdesc ? mdesc[k].n : init->n;
            if (!(h > 0.) || cnt < 1) { g_last_error = "invalid member"; return MLH_ERR_INVALID; }
            const double *lo = mdesc ? mdesc[k].box_lo : cfg->box_lo, *hi = mdesc ? mdesc[k].box_hi : cfg->box_hi;
            mem.push_back(make_member(*cfg, h, lo, hi, first, cnt));
            first += cnt;
        }
        if (first != init->n) { g_last_error = "member sizes do not add up to n"; return MLH_ERR_INVALID; }
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_last_error = "no CUDA device"; return MLH_ERR_NO_DEVICE; }
    mlh_ctx *c = new mlh_ctx();
    c->cfg = *cfg;
    c->n = init->n;
    c->nmembers = nmembers;
    c->hmembers = mem;
    c->bpm = nmembers >= BOUNDS_BLOCKS ? 1 : (BOUNDS_BLOCKS + nmembers - 1) / nmembers;
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    fill_params(c);
    // slots per particle: a multiple of 4, so that every particle's list
    // starts on a 16-byte boundary (read as uint4 by k_link)
    c->p.K = round_slots(cfg->max_neighbours > 0 ? cfg->max_neighbours : (cfg->dim == 2 ? 40 : 64));
    long long nc = 0;
    for (const Member &mb : mem) nc += estimate_cells(*cfg, init, mb);
    if (nc > (1ll << 30)) { delete c; g_last_error = "grid too large"; return MLH_ERR_CAPACITY; }
    c->p.ncells_cap = (int)nc;
    int rc = 0;
    auto fail = [&](int r) { mlh_destroy(c); return r; };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "stream"));
    cudaEventCreate(&c->ev0);
    cudaEventCreate(&c->ev1);
    if (cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "second stream"));
    size_t n = (size_t)c->n, nm = (size_t)nmembers;
#define A(ptr, cnt) if (dalloc(&c->ptr, cnt) != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "cudaMalloc " #ptr))
    A(x, n); A(y, n); A(z, n); A(vx, n); A(vy, n); A(vz, n); A(m, n); A(u, n);
    A(posf, n); A(velf, n); A(dtlo, n); A(dtcap, nm);
    A(members, nm); A(grids, nm); A(cellTotal, 1); A(boundsPart, nm * (size_t)c->bpm * 6);
    if (nmembers > 1) A(memberOf, n);
    A(cell, n); A(cellList, n);
    A(noi, n); A(noiImg, n); A(faceCnt, n); A(faceOff, n + 1);
    A(prim, n); A(geo, n); A(grad, n); A(gradRaw, n); A(fluxSums, n * 5);
    A(status, 1); A(dtbits, nm); A(newtonSum, 3); A(dt, nm); A(simTime, nm); A(stepsDone, 1);
    A(hp, n); A(neff, n); A(hstat, 2); A(hpf, n);
    A(scanTotal, 1);
    A(bar, 2);
#undef A
    if ((rc = alloc_cell_buffers(c))) return fail(rc);
    if ((rc = alloc_neighbour_buffers(c))) return fail(rc);
    if (cudaMemcpyAsync(c->members, mem.data(), sizeof(Member) * nm, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
        return fail(cuda_fail(cudaGetLastError(), "members"));
    if (nmembers > 1) {
        std::vector<int> mo(n);
        for (int k = 0; k < nmembers; ++k)
            for (int i = mem[k].first; i < mem[k].first + mem[k].count; ++i) mo[i] = k;
        if (cudaMemcpy(c->memberOf, mo.data(), sizeof(int) * n, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError(), "memberOf"));
    }
    cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream);
    cudaMemsetAsync(c->simTime, 0, sizeof(double) * nm, c->stream);
    cudaMemsetAsync(c->dt, 0, sizeof(double) * nm, c->stream);
    cudaMemsetAsync(c->newtonSum, 0, 3 * sizeof(unsigned long long), c->stream);
    cudaMemsetAsync(c->stepsDone, 0, sizeof(int), c->stream);
    cudaMemsetAsync(c->neff, 0, sizeof(double) * n, c->stream);
    cudaMemsetAsync(c->hstat, 0, 2 * sizeof(unsigned long long), c->stream);
    // empty lists until the first search (kernels after a binning that gave
    // up a bounded wait read them)
    cudaMemsetAsync(c->noi, 0, sizeof(int) * n, c->stream);
    cudaMemsetAsync(c->noiImg, 0, sizeof(int) * n, c->stream);
    cudaMemsetAsync(c->faceCnt, 0, sizeof(int) * n, c->stream);
    // the persistent binning needs its launch's blocks resident at once
    {
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device);
        c->bin_blocks = coop ? binning_blocks(cfg->dim, c->sm_count) : 0;
    }
    {
        // every particle starts at its simulation's kernelSize
        std::vector<double> h0(n);
        for (const Member &mb : mem)
            for (int i = mb.first; i < mb.first + mb.count; ++i) h0[i] = mb.h;
        if (cudaMemcpy(c->hp, h0.data(), sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError(), "hp"));
        std::vector<float> h0f(n);
        for (size_t i = 0; i < n; ++i) h0f[i] = float_up(h0[i]);
        if (cudaMemcpy(c->hpf, h0f.data(), sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(cuda_fail(cudaGetLastError(), "hpf"));
    }
    if ((rc = upload(c, init))) return fail(rc);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(cuda_fail(cudaGetLastError(), "create sync"));
    *out = c;
    return 0;
}

int mlh_create(const mlh_config *cfg, const mlh_particles_view *init, mlh_ctx **out) {
    return create_impl(cfg, 1, nullptr, init, out);
}

int mlh_ensemble_create(const mlh_config *cfg, int nmembers, const mlh_member *members,
                        const mlh_particles_view *all, mlh_ctx **out) {
    if (!members || nmembers < 1) { g_last_error = "no members"; return MLH_ERR_INVALID; }
    return create_impl(cfg, nmembers, members, all, out);
}

static void drop_graph(mlh_ctx *c) {
    if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
    c->graph_exec = nullptr;
}

// After a launch sequence reported a capacity overflow: 1.5x neighbour slots
// (MLH_ERR_NGB_OVERFLOW) and/or 2x cells (ST_CAPACITY); the work is repeated
// by the caller.
static int grow_buffers(mlh_ctx *c, unsigned st) {
    if (st & MLH_ERR_NGB_OVERFLOW) {
        free_neighbour_buffers(c);
        c->p.K = round_slots(c->p.K + c->p.K / 2);
        if (int rc = alloc_neighbour_buffers(c)) return rc;
    }
    if (st & ST_CAPACITY) {
        if (c->p.ncells_cap >= (1 << 30)) {
            g_last_error = "the grid needs more than 2^31 - 1 cells of size kernelSize";
            return MLH_ERR_CAPACITY;
        }
        free_cell_buffers(c);
        c->p.ncells_cap = c->p.ncells_cap * 2;
        if (int rc = alloc_cell_buffers(c)) return rc;
    }
    drop_graph(c);   // buffers changed
    return 0;
}

void mlh_destroy(mlh_ctx *c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graph(c);
    void *ptrs[] = {c->x, c->y, c->z, c->vx, c->vy, c->vz, c->m, c->u, c->posf, c->members, c->memberOf, c->grids,
                    c->cellTotal, c->boundsPart, c->cell, c->cellList, c->noi, c->noiImg, c->faceCnt, c->faceOff,
                    c->prim, c->geo, c->grad, c->gradRaw, c->fluxSums, c->status, c->dtbits, c->newtonSum, c->dt,
                    c->simTime, c->stepsDone, c->scanTiles, c->scanTotal, c->hp, c->neff, c->hstat, c->hpf, c->bar,
                    c->velf, c->dtlo, c->dtcap};
    for (void *q : ptrs) if (q) cudaFree(q);
    free_cell_buffers(c);
    free_neighbour_buffers(c);
    if (c->mlp_w) cudaFree(c->mlp_w);
    if (c->mlp_packed) cudaFree(c->mlp_packed);
    for (auto e : c->tev) cudaEventDestroy(e);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream2) { cudaStreamSynchronize(c->stream2); cudaStreamDestroy(c->stream2); }
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int mlh_set_fields(mlh_ctx *c, const mlh_particles_view *v) {
    if (!c || !v || v->n != c->n) { g_last_error = "size mismatch"; return MLH_ERR_INVALID; }
    int rc = upload(c, v);
    if (rc) return rc;
    return 0;
}

int mlh_get_fields(mlh_ctx *c, mlh_particles_view *v) {
    if (!c || !v || v->n != c->n) { g_last_error = "size mismatch"; return MLH_ERR_INVALID; }
    size_t b = sizeof(double) * (size_t)c->n;
    double *src[8] = {c->x, c->y, c->z, c->vx, c->vy, c->vz, c->m, c->u};
    double *dst[8] = {v->x, v->y, v->z, v->vx, v->vy, v->vz, v->m, v->u};
    for (int k = 0; k < 8; ++k) {
        if (c->cfg.dim == 2 && (k == 2 || k == 5)) continue;
        if (!dst[k]) continue;
        CK(cudaMemcpyAsync(dst[k], src[k], b, cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// One step into a CUDA graph on the context's stream (no host work inside the
// step, so the captured launches are replayed as they are).
static int capture_step(mlh_ctx *c, double dt_max) {
    drop_graph(c);
    StepArgs a = make_args(c, dt_max);
    a.timer = nullptr;
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    step(a);
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->graph_exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { c->graph_exec = nullptr; return cuda_fail(e, "cudaGraphInstantiate"); }
    c->graph_dt_max = dt_max;
    return 0;
}

int mlh_step(mlh_ctx *c, int nsteps, double dt_max, mlh_step_stats *stats) {
    if (!c || nsteps < 0) { g_last_error = "invalid argument"; return MLH_ERR_INVALID; }
    unsigned accumulated = 0;
    long long pairs = 0, faces = 0;
    unsigned long long newton = 0, fallbacks = 0, deferred = 0;
    double dev_ms = 0.;
    int done_total = 0;
    int remaining = nsteps;
    int retries = 0;
    while (remaining > 0) {
        const bool use_graph = c->graph_mode && !c->timing;
        if (use_graph && (!c->graph_exec || c->graph_dt_max != dt_max)) {
            int rc = capture_step(c, dt_max);
            if (rc) return rc;
        }
        CK(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
        CK(cudaMemsetAsync(c->stepsDone, 0, sizeof(int), c->stream));
        CK(cudaMemsetAsync(c->newtonSum, 0, 3 * sizeof(unsigned long long), c->stream));
        CK(cudaEventRecord(c->ev0, c->stream));
        if (use_graph) {
            for (int k = 0; k < remaining; ++k) CK(cudaGraphLaunch(c->graph_exec, c->stream));
        } else {
            StepArgs a = make_args(c, dt_max);
            for (int k = 0; k < remaining; ++k) step(a);
        }
        CK(cudaEventRecord(c->ev1, c->stream));
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(c->stream));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, c->ev0, c->ev1);
        dev_ms += ms;
        if (c->timing) collect_timers(c);
        unsigned st = 0;
        int done = 0;
        unsigned long long nsum[3] = {0, 0, 0};
        CK(cudaMemcpy(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(&done, c->stepsDone, sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(nsum, c->newtonSum, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
        newton += nsum[0];
        fallbacks += nsum[1];
        deferred += nsum[2];
        done_total += done;
        remaining -= done;
        // per-step interaction counts of the last step
        int ftot = 0;
        CK(cudaMemcpy(&ftot, c->faceOff + c->n, sizeof(int), cudaMemcpyDeviceToHost));
        faces += (long long)ftot * done;
        pairs += 2ll * ftot * done;
        if (st & (MLH_ERR_NGB_OVERFLOW | ST_CAPACITY)) {
            if (++retries > 8) { accumulated |= st; g_last_error = "capacity retries exhausted"; break; }
            if (int rc = grow_buffers(c, st)) return rc;
            // the step is repeated: faces recorded by the aborted attempt go
            if (c->harvest.count) CK(cudaMemsetAsync(c->harvest.count, 0, sizeof(int), c->stream));
            continue;
        }
        accumulated |= st;
        if (done == 0) break;
    }
    if (stats) {
        stats->steps = done_total;
        stats->status = accumulated;
        cudaMemcpy(&stats->dt, c->dt, sizeof(double), cudaMemcpyDeviceToHost);
        cudaMemcpy(&stats->time, c->simTime, sizeof(double), cudaMemcpyDeviceToHost);
        stats->pair_interactions = pairs;
        stats->faces = faces;
        stats->newton_iterations = (long long)newton;
        stats->device_ms = dev_ms;
        stats->newton_fallbacks = (long long)fallbacks;
        stats->learned_faces = (long long)deferred;
    }
    return (int)(accumulated & ~(unsigned)MLH_ERR_NGB_OVERFLOW & ~ST_CAPACITY) ? (int)accumulated : 0;
}

// Coordinate search over the launch shapes: each candidate runs `trial_steps`
// steps with per-kernel timing from a saved copy of the state, which is put
// back afterwards (positions, velocities, masses, energies, member times).
int mlh_set_tuning(mlh_ctx *c, const mlh_tuning *t) {
    auto threads_ok = [](int v) { return v == 64 || v == 128 || v == 256; };
    if (!c || !t || !threads_ok(t->face_threads) || !threads_ok(t->grad_threads) || t->face_blocks_per_sm < 1 ||
        t->face_blocks_per_sm > 32 || t->nns_warps_per_sm < 8 || t->nns_warps_per_sm > 256 ||
        t->face_split < 0 || t->face_split > 2 || t->link_overlap < 0 || t->link_overlap > 2 ||
        t->persistent_binning < 0 || t->persistent_binning > 1 || (t->persistent_binning && c->bin_blocks < 1) ||
        t->fp32_filters < 0 || t->fp32_filters > 3 || t->learned_guess < 0 || t->learned_guess > 1) {
        g_last_error = "invalid tuning";
        return MLH_ERR_INVALID;
    }
    CK(cudaStreamSynchronize(c->stream));
    c->tune.face_threads = t->face_threads;
    c->tune.face_blocks_per_sm = t->face_blocks_per_sm;
    c->tune.grad_threads = t->grad_threads;
    c->tune.nns_warps_per_sm = t->nns_warps_per_sm;
    c->tune.face_split = t->face_split;
    c->tune.link_overlap = t->link_overlap;
    c->tune.persistent_binning = t->persistent_binning;
    c->tune.fp32_filters = t->fp32_filters;
    c->tune.learned_guess = t->learned_guess;
    drop_graph(c);
    return 0;
}

int mlh_test_binning_barrier(mlh_ctx *c, unsigned extra_arrivals, unsigned spin_limit) {
    if (!c) { g_last_error = "null context"; return MLH_ERR_INVALID; }
    CK(cudaStreamSynchronize(c->stream));
    c->bar_extra = extra_arrivals;
    c->bar_spin = spin_limit;
    drop_graph(c);
    return 0;
}

int mlh_autotune(mlh_ctx *c, int trial_steps, mlh_tuning *out) {
    if (!c || trial_steps < 1) { g_last_error = "invalid argument"; return MLH_ERR_INVALID; }
    const size_t n = (size_t)c->n, nm = (size_t)c->nmembers;
    double *save = nullptr;
    // the state, and the smoothing lengths (the start of the next solve)
    CK(cudaMalloc(&save, sizeof(double) * (9 * n + 2 * nm)));
    double *src[9] = {c->x, c->y, c->z, c->vx, c->vy, c->vz, c->m, c->u, c->hp};
    for (int k = 0; k < 9; ++k) CK(cudaMemcpyAsync(save + k * n, src[k], sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(save + 9 * n, c->simTime, sizeof(double) * nm, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpyAsync(save + 9 * n + nm, c->dt, sizeof(double) * nm, cudaMemcpyDeviceToDevice, c->stream));
    const bool timing0 = c->timing, graph0 = c->graph_mode;
    c->graph_mode = false;
    drop_graph(c);
    auto restore = [&]() -> int {
        for (int k = 0; k < 9; ++k) CK(cudaMemcpyAsync(src[k], save + k * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(c->simTime, save + 9 * n, sizeof(double) * nm, cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(c->dt, save + 9 * n + nm, sizeof(double) * nm, cudaMemcpyDeviceToDevice, c->stream));
        pack_posf(c->x, c->y, c->z, c->n, c->cfg.dim, c->posf, c->stream);
        return 0;
    };
    // time of kernel `id` over trial_steps steps with the current tuning
    auto trial = [&](int id, double &ms) -> int {
        if (int rc = restore()) return rc;
        c->timing = true;
        mlh_reset_kernel_times(c);
        mlh_step_stats st;
        int rc = mlh_step(c, trial_steps, 0., &st);
        c->timing = false;
        if (rc & (MLH_ERR_CUDA | MLH_ERR_INVALID)) return rc;
        ms = c->kt_ms[id];
        return 0;
    };
    int rc = 0;
    {   // warm-up so that buffers have reached their final capacity
        double dummy;
        if ((rc = trial(KT_FACES, dummy))) goto done;
    }
    {
        // with star-pressure weights set, the whole search once per face
        // pipeline (learned, then plain: `learned_guess`), each tuned for
        // itself, and the faster kept: the network pays only where strong
        // shocks are frequent enough to outweigh its evaluation and passes
        const Tuning init = c->tune;
        Tuning chosen = c->tune;
        double chosen_ms = 1e300;
        const int npipes = c->learned ? 2 : 1;
        for (int pipe = 0; pipe < npipes; ++pipe) {
            c->tune = init;
            if (c->learned) c->tune.learned_guess = pipe == 0 ? 1 : 0;
            {
                const int cand_t[] = {64, 128, 256};
                const int cand_b[] = {2, 4, 8, 16, 32};
                Tuning best = c->tune;
                double best_ms = 1e300;
                // the face passes: one (0), a second over a queue (1) or the
                // unfinished faces continued inside the block (2), each over the
                // candidate grids (the structures favour different grids); which
                // pays depends on how many faces need a second Newton step
                for (int split : {1, 2, 0}) {
                    for (int b : cand_b) {
                        c->tune.face_split = split;
                        c->tune.face_blocks_per_sm = b;
                        double ms;
                        if ((rc = trial(KT_FACES, ms))) goto done;
                        if (ms < best_ms) { best_ms = ms; best.face_split = split; best.face_blocks_per_sm = b; }
                    }
                }
                c->tune.face_split = best.face_split;
                c->tune.face_blocks_per_sm = best.face_blocks_per_sm;
                for (int t : cand_t) {
                    c->tune.face_threads = t;
                    double ms;
                    if ((rc = trial(KT_FACES, ms))) goto done;
                    if (ms < best_ms) { best_ms = ms; best.face_threads = t; }
                }
                c->tune.face_threads = best.face_threads;
                for (int b : cand_b) {   // the grid again, for the chosen block size
                    c->tune.face_blocks_per_sm = b;
                    double ms;
                    if ((rc = trial(KT_FACES, ms))) goto done;
                    if (ms < best_ms) { best_ms = ms; best.face_blocks_per_sm = b; }
                }
                c->tune.face_blocks_per_sm = best.face_blocks_per_sm;
                best_ms = 1e300;
                for (int t : cand_t) {
                    c->tune.grad_threads = t;
                    double ms;
                    if ((rc = trial(KT_GRAD, ms))) goto done;
                    if (ms < best_ms) { best_ms = ms; best.grad_threads = t; }
                }
                c->tune.grad_threads = best.grad_threads;
                best_ms = 1e300;
                const int cand_w[] = {16, 32, 64, 128};
                for (int w : cand_w) {
                    c->tune.nns_warps_per_sm = w;
                    double ms;
                    if ((rc = trial(KT_NNS, ms))) goto done;
                    if (ms < best_ms) { best_ms = ms; best.nns_warps_per_sm = w; }
                }
                c->tune.nns_warps_per_sm = best.nns_warps_per_sm;
                // the face links beside the time step and the gradients, or in order:
                // whole steps without per-kernel timing (which serialises the
                // streams), the better of two trials each
                double best_step = 1e300;
                for (int ov : {1, 0, 2}) {
                    c->tune.link_overlap = ov;
                    for (int rep = 0; rep < 2; ++rep) {
                        if ((rc = restore())) goto done;
                        mlh_step_stats st;
                        rc = mlh_step(c, trial_steps, 0., &st);
                        if (rc & (MLH_ERR_CUDA | MLH_ERR_INVALID)) goto done;
                        rc = 0;
                        if (st.device_ms < best_step) { best_step = st.device_ms; best.link_overlap = ov; }
                    }
                }
                c->tune.link_overlap = best.link_overlap;
                // the binning as one persistent kernel or one launch per phase
                best_step = 1e300;
                for (int pb : {0, 1}) {
                    if (pb && c->bin_blocks < 1) continue;
                    c->tune.persistent_binning = pb;
                    for (int rep = 0; rep < 2; ++rep) {
                        if ((rc = restore())) goto done;
                        mlh_step_stats st;
                        rc = mlh_step(c, trial_steps, 0., &st);
                        if (rc & (MLH_ERR_CUDA | MLH_ERR_INVALID | MLH_ERR_TIMEOUT)) goto done;
                        rc = 0;
                        if (st.device_ms < best_step) { best_step = st.device_ms; best.persistent_binning = pb; }
                    }
                }
                c->tune.persistent_binning = best.persistent_binning;
                // the slope limiter's single-precision filter on or off (the same
                // bits either way; it trades FP64 work for two single-precision
                // passes, which pays or not with the gradients' occupancy)
                best_step = 1e300;
                const int keep = c->tune.fp32_filters & MLH_FILTER_TIMESTEP;
                for (int sf : {keep | MLH_FILTER_SLOPE, keep}) {
                    c->tune.fp32_filters = sf;
                    for (int rep = 0; rep < 2; ++rep) {
                        if ((rc = restore())) goto done;
                        mlh_step_stats st;
                        rc = mlh_step(c, trial_steps, 0., &st);
                        if (rc & (MLH_ERR_CUDA | MLH_ERR_INVALID | MLH_ERR_TIMEOUT)) goto done;
                        rc = 0;
                        if (st.device_ms < best_step) { best_step = st.device_ms; best.fp32_filters = sf; }
                    }
                }
                c->tune.fp32_filters = best.fp32_filters;
            }
            // the pipeline's whole step with its shapes
            double pipe_ms = 1e300;
            for (int rep = 0; rep < 2; ++rep) {
                if ((rc = restore())) goto done;
                mlh_step_stats st;
                rc = mlh_step(c, trial_steps, 0., &st);
                if (rc & (MLH_ERR_CUDA | MLH_ERR_INVALID | MLH_ERR_TIMEOUT)) goto done;
                rc = 0;
                if (st.device_ms < pipe_ms) pipe_ms = st.device_ms;
            }
            if (pipe_ms < chosen_ms) { chosen_ms = pipe_ms; chosen = c->tune; }
        }
        c->tune = chosen;
    }
done:
    {
        int rc2 = restore();
        CK(cudaStreamSynchronize(c->stream));
        cudaFree(save);
        c->timing = timing0;
        c->graph_mode = graph0;
        mlh_reset_kernel_times(c);
        if (!rc) rc = rc2;
    }
    if (out) {
        out->face_threads = c->tune.face_threads;
        out->face_blocks_per_sm = c->tune.face_blocks_per_sm;
        out->grad_threads = c->tune.grad_threads;
        out->nns_warps_per_sm = c->tune.nns_warps_per_sm;
        out->face_split = c->tune.face_split;
        out->link_overlap = c->tune.link_overlap;
        out->persistent_binning = c->tune.persistent_binning;
        out->fp32_filters = c->tune.fp32_filters;
        out->learned_guess = c->tune.learned_guess;
    }
    return rc;
}

// Learned p* guess on (weights: 8705 floats, host) or off (NULL).
int mlh_set_pstar_weights(mlh_ctx *c, const float *weights) {
    if (!c) return MLH_ERR_INVALID;
    CK(cudaStreamSynchronize(c->stream));
    drop_graph(c);
    if (!weights) {
        c->learned = false;
        return 0;
    }
    if (!c->mlp_w) CK(dalloc(&c->mlp_w, PSTAR_PARAMS));
    if (!c->mlp_packed) CK(cudaMalloc(&c->mlp_packed, pstar_packed_bytes()));
    CK(cudaMemcpy(c->mlp_w, weights, sizeof(float) * PSTAR_PARAMS, cudaMemcpyHostToDevice));
    pstar_pack(c->mlp_w, c->mlp_packed, c->stream);
    if (!c->learned) {
        c->learned = true;
        free_neighbour_buffers(c);
        if (int rc = alloc_neighbour_buffers(c)) return rc;
    }
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// One step that also records network inputs and targets log(p*/p_TR) of
// every `stride`-th face (plain face pipeline).
static int harvest_impl(mlh_ctx *c, int stride, int strong, float *x, float *t, long long capacity,
                        long long *count);

int mlh_pstar_harvest(mlh_ctx *c, int stride, float *x, float *t, long long capacity, long long *count) {
    return harvest_impl(c, stride, 0, x, t, capacity, count);
}

int mlh_pstar_harvest_strong(mlh_ctx *c, float *x, float *t, long long capacity, long long *count) {
    return harvest_impl(c, 1, 1, x, t, capacity, count);
}

static int harvest_impl(mlh_ctx *c, int stride, int strong, float *x, float *t, long long capacity,
                        long long *count) {
    if (!c || stride < 1 || !x || !t || capacity < 1 || capacity > 0x7fffffff) {
        g_last_error = "invalid argument";
        return MLH_ERR_INVALID;
    }
    const bool learned0 = c->learned;
    c->learned = false;
    drop_graph(c);
    float4 *hx = nullptr;
    float *ht = nullptr;
    int *hc = nullptr;
    CK(cudaMalloc(&hx, sizeof(float4) * (size_t)capacity));
    CK(cudaMalloc(&ht, sizeof(float) * (size_t)capacity));
    CK(cudaMalloc(&hc, sizeof(int)));
    CK(cudaMemsetAsync(hc, 0, sizeof(int), c->stream));
    c->harvest.x = hx; c->harvest.t = ht; c->harvest.count = hc;
    c->harvest.stride = stride; c->harvest.cap = (int)capacity; c->harvest.strong = strong;
    mlh_step_stats st;
    int rc = mlh_step(c, 1, 0., &st);
    c->harvest = Harvest{};
    c->learned = learned0;
    int cnt = 0;
    cudaMemcpy(&cnt, hc, sizeof(int), cudaMemcpyDeviceToHost);
    if (cnt > capacity) cnt = (int)capacity;
    cudaMemcpy(x, hx, sizeof(float4) * (size_t)cnt, cudaMemcpyDeviceToHost);
    cudaMemcpy(t, ht, sizeof(float) * (size_t)cnt, cudaMemcpyDeviceToHost);
    cudaFree(hx); cudaFree(ht); cudaFree(hc);
    if (count) *count = cnt;
    return rc;
}

int mlh_smoothing_lengths(mlh_ctx *c, double n_ngb, double *h_out, double *n_eff_out, long long *clamped) {
    if (!c) { g_last_error = "null context"; return MLH_ERR_INVALID; }
    if (!(sngb_target(c->cfg.dim, n_ngb) > 0.)) {
        g_last_error = "n_ngb must exceed the particle's own count (32/3 in 3D, 40/7 in 2D)";
        return MLH_ERR_INVALID;
    }
    for (int retries = 0;; ++retries) {
        StepArgs a = make_args(c, 0.);
        a.p.sngb_t = sngb_target(c->cfg.dim, n_ngb);
        CK(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
        smoothing_lengths(a);
        CK(cudaGetLastError());
        unsigned st = 0;
        CK(cudaMemcpyAsync(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (st & (MLH_ERR_NGB_OVERFLOW | ST_CAPACITY)) {
            if (retries >= 8) { g_last_error = "capacity retries exhausted"; return (int)st; }
            if (int rc = grow_buffers(c, st)) return rc;
            continue;
        }
        if (st) return (int)st;
        break;
    }
    const size_t b = sizeof(double) * (size_t)c->n;
    if (h_out) CK(cudaMemcpy(h_out, c->hp, b, cudaMemcpyDeviceToHost));
    if (n_eff_out) CK(cudaMemcpy(n_eff_out, c->neff, b, cudaMemcpyDeviceToHost));
    if (clamped) {
        unsigned long long hs[2];
        CK(cudaMemcpy(hs, c->hstat, sizeof(hs), cudaMemcpyDeviceToHost));
        *clamped = (long long)hs[1];
    }
    return 0;
}

int mlh_prepare(mlh_ctx *c, double dt_max) {
    if (!c) { g_last_error = "null context"; return MLH_ERR_INVALID; }
    for (int retries = 0;; ++retries) {
        StepArgs a = make_args(c, dt_max);
        a.stop_after_gradients = 1;
        a.timer = nullptr;
        CK(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
        step(a);
        CK(cudaGetLastError());
        unsigned st = 0;
        CK(cudaMemcpyAsync(&st, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (st & (MLH_ERR_NGB_OVERFLOW | ST_CAPACITY)) {
            if (retries >= 8) { g_last_error = "capacity retries exhausted"; return (int)st; }
            if (int rc = grow_buffers(c, st)) return rc;
            continue;
        }
        return (int)st;
    }
}

int mlh_riemann_fluxes(int dim, int n, const double *Wi, const double *Wj, const double *vFrame, const double *Aij,
                       double gamma, int mfm, double *F, int *iters) {
    if ((dim != 2 && dim != 3) || n < 0 || !(gamma > 1.) || (n > 0 && (!Wi || !Wj || !vFrame || !Aij || !F))) {
        g_last_error = "invalid argument";
        return MLH_ERR_INVALID;
    }
    if (n == 0) return 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_last_error = "no CUDA device"; return MLH_ERR_NO_DEVICE; }
    const size_t NV = (size_t)dim + 2, nn = (size_t)n;
    double *d = nullptr;
    int *dit = nullptr;
    unsigned *dst = nullptr;
    const size_t doubles = nn * (3 * NV + 2 * dim);
    CK(cudaMalloc(&d, sizeof(double) * doubles));
    auto cleanup = [&]() { cudaFree(d); cudaFree(dit); cudaFree(dst); };
    double *dWi = d, *dWj = d + nn * NV, *dv = d + 2 * nn * NV, *dA = dv + nn * dim, *dF = dA + nn * dim;
    cudaError_t e = cudaMalloc(&dit, sizeof(int) * nn);
    if (e == cudaSuccess) e = cudaMalloc(&dst, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(dst, 0, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemcpy(dWi, Wi, sizeof(double) * nn * NV, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dWj, Wj, sizeof(double) * nn * NV, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dv, vFrame, sizeof(double) * nn * dim, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dA, Aij, sizeof(double) * nn * dim, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        riemann_batch(dim, n, gamma, 1e-10, 100, mfm, dWi, dWj, dv, dA, dF, dit, dst, 0);
        e = cudaGetLastError();
    }
    unsigned st = 0;
    if (e == cudaSuccess) e = cudaMemcpy(F, dF, sizeof(double) * nn * NV, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && iters) e = cudaMemcpy(iters, dit, sizeof(int) * nn, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&st, dst, sizeof(unsigned), cudaMemcpyDeviceToHost);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "mlh_riemann_fluxes");
    return (int)st;
}

int mlh_set_graph_mode(mlh_ctx *c, int enable) {
    if (!c) return MLH_ERR_INVALID;
    c->graph_mode = enable != 0;
    if (!c->graph_mode) drop_graph(c);
    return 0;
}

int mlh_member_times(mlh_ctx *c, double *dt, double *time, int nmembers) {
    if (!c || nmembers != c->nmembers) { g_last_error = "member count mismatch"; return MLH_ERR_INVALID; }
    CK(cudaStreamSynchronize(c->stream));
    if (dt) CK(cudaMemcpy(dt, c->dt, sizeof(double) * nmembers, cudaMemcpyDeviceToHost));
    if (time) CK(cudaMemcpy(time, c->simTime, sizeof(double) * nmembers, cudaMemcpyDeviceToHost));
    return 0;
}

int mlh_stage_array(mlh_ctx *c, const char *name, void *out, long long capacity, long long *count) {
    if (!c || !name) return MLH_ERR_INVALID;
    const std::string nm(name);
    const int n = c->n, K = c->p.K, D = c->cfg.dim;
    std::vector<int> noi(n), noiImg(n);
    auto need_lists = [&]() -> int {
        CK(cudaMemcpy(noi.data(), c->noi, sizeof(int) * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(noiImg.data(), c->noiImg, sizeof(int) * n, cudaMemcpyDeviceToHost));
        return 0;
    };
    CK(cudaStreamSynchronize(c->stream));
    auto put = [&](const void *src, size_t elems, size_t esize) -> int {
        if (count) *count = (long long)elems;
        if (!out) return 0;
        if ((long long)elems > capacity) { g_last_error = "capacity too small"; return MLH_ERR_INVALID; }
        std::memcpy(out, src, elems * esize);
        return 0;
    };
    if (nm == "noi" || nm == "noi_img" || nm == "off") {
        if (int rc = need_lists()) return rc;
        if (nm == "noi") return put(noi.data(), n, 4);
        if (nm == "noi_img") return put(noiImg.data(), n, 4);
        std::vector<int> off(n + 1, 0);
        for (int i = 0; i < n; ++i) off[i + 1] = off[i] + noi[i] + noiImg[i];
        return put(off.data(), n + 1, 4);
    }
    if (nm == "nnl" || nm == "face_of" || nm == "F" || nm == "face_iters") {
        if (int rc = need_lists()) return rc;
        std::vector<uint32_t> nb((size_t)n * K);
        std::vector<int> fo((size_t)n * K);
        CK(cudaMemcpy(nb.data(), c->nbr, sizeof(uint32_t) * nb.size(), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(fo.data(), c->faceOf, sizeof(int) * fo.size(), cudaMemcpyDeviceToHost));
        if (nm == "nnl" || nm == "face_of") {
            std::vector<uint32_t> o;
            for (int i = 0; i < n; ++i)
                for (int s = 0; s < noi[i] + noiImg[i]; ++s)
                    o.push_back(nm == "nnl" ? nb[(size_t)i * K + s] : (uint32_t)fo[(size_t)i * K + s]);
            return put(o.data(), o.size(), 4);
        }
        int ftot = 0;
        CK(cudaMemcpy(&ftot, c->faceOff + n, sizeof(int), cudaMemcpyDeviceToHost));
        std::vector<double> F((size_t)ftot * 6 + 6);
        CK(cudaMemcpy(F.data(), c->Fface, sizeof(double) * (size_t)ftot * 6, cudaMemcpyDeviceToHost));
        if (nm == "face_iters") {   // Newton steps of each slot's face (the record's sixth double)
            std::vector<int> it;
            for (int i = 0; i < n; ++i)
                for (int s = 0; s < noi[i] + noiImg[i]; ++s) {
                    const int f = fo[(size_t)i * K + s];
                    const int id = (f > 0 ? f : -f) - 1;
                    it.push_back(f == 0 ? 0 : (int)F[(size_t)id * 6 + 5]);
                }
            return put(it.data(), it.size(), 4);
        }
        std::vector<double> o;
        const int NV = D + 2;
        for (int i = 0; i < n; ++i)
            for (int s = 0; s < noi[i] + noiImg[i]; ++s) {
                int f = fo[(size_t)i * K + s];
                double sg = f > 0 ? 1. : -1.;
                int id = (f > 0 ? f : -f) - 1;
                for (int k = 0; k < NV; ++k) o.push_back(f == 0 ? 0. : sg * F[(size_t)id * 6 + k]);
            }
        return put(o.data(), o.size(), 8);
    }
    if (nm == "omega" || nm == "rho" || nm == "P" || nm == "c" || nm == "B") {
        std::vector<Prim> pr(n);
        std::vector<Geo> ge(n);
        CK(cudaMemcpy(pr.data(), c->prim, sizeof(Prim) * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(ge.data(), c->geo, sizeof(Geo) * n, cudaMemcpyDeviceToHost));
        std::vector<double> o;
        for (int i = 0; i < n; ++i) {
            if (nm == "omega") o.push_back(ge[i].omega);
            else if (nm == "rho") o.push_back(pr[i].rho);
            else if (nm == "P") o.push_back(pr[i].P);
            else if (nm == "c") o.push_back(ge[i].c);
            else for (int k = 0; k < D * D; ++k) o.push_back(ge[i].B[k]);
        }
        return put(o.data(), o.size(), 8);
    }
    if (nm.compare(0, 5, "grad_") == 0 || nm.compare(0, 8, "gradraw_") == 0) {
        const bool raw = nm.compare(0, 8, "gradraw_") == 0;
        const std::string f = nm.substr(raw ? 8 : 5);
        int blk = f == "rho" ? 0 : f == "vx" ? 1 : f == "vy" ? 2 : f == "vz" ? 3 : f == "P" ? 4 : -1;
        if (blk < 0 || (raw && !c->debug_arrays)) return MLH_ERR_INVALID;
        std::vector<Grad> g(n);
        CK(cudaMemcpy(g.data(), raw ? c->gradRaw : c->grad, sizeof(Grad) * n, cudaMemcpyDeviceToHost));
        std::vector<double> o((size_t)n * 3);
        for (int i = 0; i < n; ++i)
            for (int a = 0; a < 3; ++a) o[(size_t)i * 3 + a] = g[i].g[blk * 3 + a];
        return put(o.data(), o.size(), 8);
    }
    if (nm == "mF" || nm == "eF" || nm == "vF") {
        std::vector<double> fs((size_t)n * 5);
        CK(cudaMemcpy(fs.data(), c->fluxSums, sizeof(double) * fs.size(), cudaMemcpyDeviceToHost));
        std::vector<double> o;
        for (int i = 0; i < n; ++i) {
            if (nm == "mF") o.push_back(fs[(size_t)i * 5]);
            else if (nm == "eF") o.push_back(fs[(size_t)i * 5 + 1]);
            else for (int a = 0; a < 3; ++a) o.push_back(fs[(size_t)i * 5 + 2 + a]);
        }
        return put(o.data(), o.size(), 8);
    }
    if (nm == "h" || nm == "n_eff") {
        std::vector<double> o(n);
        CK(cudaMemcpy(o.data(), nm == "h" ? c->hp : c->neff, sizeof(double) * n, cudaMemcpyDeviceToHost));
        return put(o.data(), o.size(), 8);
    }
    if (nm == "h_stats") {
        unsigned long long hs[2];
        CK(cudaMemcpy(hs, c->hstat, sizeof(hs), cudaMemcpyDeviceToHost));
        double o[2] = {(double)hs[0], (double)hs[1]};
        return put(o, 2, 8);
    }
    if (nm == "dt") {
        double d;
        CK(cudaMemcpy(&d, c->dt, sizeof(double), cudaMemcpyDeviceToHost));
        return put(&d, 1, 8);
    }
    if (nm == "grid") {
        GridInfo g;
        CK(cudaMemcpy(&g, c->grids, sizeof(GridInfo), cudaMemcpyDeviceToHost));
        double o[9];
        for (int a = 0; a < 3; ++a) {
            o[a] = a < D ? g.lo[a] : 0.;
            o[3 + a] = a < D ? g.hi[a] : 0.;
            o[6 + a] = a < D ? g.cells[a] : 0.;
        }
        return put(o, 9, 8);
    }
    g_last_error = "unknown array " + nm;
    return MLH_ERR_INVALID;
}

int mlh_set_kernel_timing(mlh_ctx *c, int enable) {
    if (!c) return MLH_ERR_INVALID;
    c->timing = enable != 0;
    return 0;
}

int mlh_kernel_times(mlh_ctx *c, const char **names, long long *launches, double *total_ms, int max) {
    if (!c) return -1;
    int k = 0;
    for (int id = 0; id < KT_COUNT && k < max; ++id, ++k) {
        if (names) names[k] = kernel_timer_name(id);
        if (launches) launches[k] = c->kt_launches[id];
        if (total_ms) total_ms[k] = c->kt_ms[id];
    }
    return k;
}

void mlh_reset_kernel_times(mlh_ctx *c) {
    if (!c) return;
    for (int id = 0; id < KT_COUNT; ++id) { c->kt_ms[id] = 0.; c->kt_launches[id] = 0; }
}

}  // extern "C"
