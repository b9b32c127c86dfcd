/*
 * meshlesshydro-gb300: C++ host classes with the reference's names and
 * signatures (jammartin/meshlessHydro, demonstrator/include/): ConfigParser,
 * InitialDistribution, Particles, Domain, MeshlessScheme and Riemann, in
 * namespace mlh, on top of the C ABI (mlh.h, mlh_io.h).  A driver written
 * against the reference (demonstrator/src/main.cpp:16-117) compiles against
 * these with `using namespace mlh;`; MeshlessScheme::run advances the state
 * with the GB300 step instead of the Particles stage methods.
 *
 * Header only.  The reference's compile-time switches (DIM,
 * PERIODIC_BOUNDARIES, ADAPTIVE_TIMESTEP, CFL, ...) are read from the
 * including translation unit's macros when it defines them (parameter.h
 * included first), or given at run time as an mlh_run_config
 * (mlh_read_parameter_header).  Errors throw mlh::Error (the reference calls
 * exit()).
 */
#ifndef MLH_HPP
#define MLH_HPP

#include "mlh.h"
#include "mlh_io.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iomanip>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace mlh {

class Error : public std::runtime_error {
public:
    Error(const std::string &where, int st)
        : std::runtime_error(where + ": " + mlh_last_error() + " (status 0x" + hex(st) + ")"), status(st) {}
    int status;

private:
    static std::string hex(int v) {
        std::ostringstream o;
        o << std::hex << v;
        return o.str();
    }
};

inline void check(int status, const char *where) {
    if (status) throw Error(where, status);
}

// Status bits after which a run cannot go on; the others (negative density,
// pressure, mass or energy, vacuum, Newton non-convergence, one-sided pairs)
// are the reference's warnings (Logger(WARN), Particles.cpp:1156-1158,
// 1284-1286, 1639-1655, 1813-1834, 2044-2075).
constexpr int FATAL_STATUS = MLH_ERR_INVALID | MLH_ERR_CUDA | MLH_ERR_NO_DEVICE | MLH_ERR_CAPACITY | MLH_ERR_NAN |
                             MLH_ERR_GRID | MLH_ERR_NGB_OVERFLOW | MLH_ERR_TIMEOUT;

inline int check_fatal(int status, const char *where) {
    if (status & FATAL_STATUS) throw Error(where, status);
    return status;
}

// The settings of demonstrator/include/parameter.h as the including file's
// macros give them (an undefined switch is 0, as in the reference's #if),
// over mlh_default_run_config.
inline mlh_run_config settings_from_macros() {
    mlh_run_config r;
    mlh_default_run_config(&r);
    mlh_config &c = r.cfg;
#ifdef DIM
    c.dim = DIM;
    c.periodic = 0; c.adaptive_timestep = 0; c.slope_limiting = 0; c.pairwise_limiter = 0;
    c.meshless_finite_mass = 0; c.move_particles = 0; c.first_order_quad_point = 0;
#ifdef PERIODIC_BOUNDARIES
    c.periodic = PERIODIC_BOUNDARIES;
#endif
#ifdef ADAPTIVE_TIMESTEP
    c.adaptive_timestep = ADAPTIVE_TIMESTEP;
#endif
#ifdef CFL
    c.cfl = CFL;
#endif
#ifdef SLOPE_LIMITING
    c.slope_limiting = SLOPE_LIMITING;
#endif
#ifdef BETA
    c.beta = BETA;
#endif
#ifdef PAIRWISE_LIMITER
    c.pairwise_limiter = PAIRWISE_LIMITER;
#endif
#ifdef PSI_1
    c.psi1 = PSI_1;
#endif
#ifdef PSI_2
    c.psi2 = PSI_2;
#endif
#ifdef MESHLESS_FINITE_MASS
    c.meshless_finite_mass = MESHLESS_FINITE_MASS;
#endif
#ifdef MOVE_PARTICLES
    c.move_particles = MOVE_PARTICLES;
#endif
#ifdef FIRST_ORDER_QUAD_POINT
    c.first_order_quad_point = FIRST_ORDER_QUAD_POINT;
#endif
#ifdef MAX_NUM_INTERACTIONS
    c.max_neighbours = MAX_NUM_INTERACTIONS;
#endif
#ifdef DEBUG_LVL
    r.debug_lvl = DEBUG_LVL;
#endif
#endif  // DIM
    return r;
}

// ConfigParser (demonstrator/include/ConfigParser.h:13-53): getVal<T>(key)
// and getObj(key) over a config.info.
class ConfigParser {
public:
    explicit ConfigParser(const std::string &file, const std::string &prefix = "") : file(file), prefix(prefix) {}
    template <typename T>
    T getVal(const std::string &key) const {
        std::istringstream is(text(key));
        T v{};
        is >> v;
        if (is.fail()) throw Error("ConfigParser::getVal(" + prefix + key + ")", MLH_ERR_INVALID);
        return v;
    }
    ConfigParser getObj(const std::string &key) const { return ConfigParser(file, prefix + key + "."); }

private:
    std::string text(const std::string &key) const {
        std::vector<char> buf(4096);
        check(mlh_info_get(file.c_str(), (prefix + key).c_str(), buf.data(), (int)buf.size()), "ConfigParser");
        return std::string(buf.data());
    }
    std::string file, prefix;
};
template <>
inline std::string ConfigParser::getVal<std::string>(const std::string &key) const {
    return text(key);
}

// Particles (demonstrator/include/Particles.h:18-240): the state arrays the
// driver reads and writes, in host memory.  The stage methods of the
// reference are replaced by MeshlessScheme::run on the GPU; the arrays of the
// last prepared step (rho, P, omega, rhoGrad, noi) are filled for dumps.
class Particles {
public:
    explicit Particles(int N, bool ghosts = false, int dim = settings_from_macros().cfg.dim)
        : N(N), dim(dim), ghosts(ghosts), store_((size_t)N * 11, 0.), ints_((size_t)N * 2, 0),
          grad_((size_t)N * 3, 0.) {
        double *b = store_.data();
        double **f[] = {&x, &y, &z, &vx, &vy, &vz, &m, &u, &rho, &P, &omega};
        for (int k = 0; k < 11; ++k) *f[k] = b + (size_t)k * N;
        matId = ints_.data();
        noi = ints_.data() + N;
        rhoGrad = reinterpret_cast<double (*)[3]>(grad_.data());
    }
    Particles(const Particles &) = delete;
    Particles &operator=(const Particles &) = delete;

    int N;
    int dim;
    bool ghosts;
    double *x, *y, *z, *vx, *vy, *vz, *m, *u, *rho, *P, *omega;
    int *matId, *noi;
    double (*rhoGrad)[3];

    mlh_particles_view view() {
        mlh_particles_view v = {N, x, y, dim == 3 ? z : nullptr, vx, vy, dim == 3 ? vz : nullptr, m, u};
        return v;
    }

    // Particles::getDomainLimits (Particles.cpp:228-267), with its else-if
    // and numeric_limits<double>::min() start values; layout
    // [minX, minY, (minZ), maxX, maxY, (maxZ)].
    void getDomainLimits(double *domainLimits) const {
        const double *X[3] = {x, y, z};
        for (int a = 0; a < dim; ++a) {
            double mn = std::numeric_limits<double>::max(), mx = std::numeric_limits<double>::min();
            for (int i = 0; i < N; ++i) {
                if (X[a][i] < mn) mn = X[a][i];
                else if (X[a][i] > mx) mx = X[a][i];
            }
            domainLimits[a] = mn;
            domainLimits[dim + a] = mx;
        }
    }

    // Particles::sumMass .. sumVolume (Particles.cpp:2830-2886)
    double sumMass() const { double M = 0.; for (int i = 0; i < N; ++i) M += m[i]; return M; }
    double sumEnergy() const {
        double E = 0.;
        for (int i = 0; i < N; ++i) {
            if (dim == 2) E += m[i] * (u[i] + .5 * (vx[i] * vx[i] + vy[i] * vy[i]));
            else E += m[i] * (u[i] + .5 * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]));
        }
        return E;
    }
    double sumMomentumX() const { double p = 0.; for (int i = 0; i < N; ++i) p += m[i] * vx[i]; return p; }
    double sumMomentumY() const { double p = 0.; for (int i = 0; i < N; ++i) p += m[i] * vy[i]; return p; }
    double sumMomentumZ() const { double p = 0.; for (int i = 0; i < N; ++i) p += m[i] * vz[i]; return p; }
    double sumVolume() const { double V = 0.; for (int i = 0; i < N; ++i) V += 1. / omega[i]; return V; }

    // Particles::dump2file (Particles.cpp:2978-3076), plus /materialId so
    // that the snapshot reads back as an initial distribution.
    void dump2file(const std::string &filename, double simTime) {
        mlh_particles_view v = view();
        check(mlh_write_snapshot(filename.c_str(), dim, &v, rho, P, &rhoGrad[0][0], noi, matId, simTime),
              "Particles::dump2file");
    }

private:
    std::vector<double> store_;
    std::vector<int> ints_;
    std::vector<double> grad_;
};

// InitialDistribution (demonstrator/src/InitialDistribution.cpp:7-59).
class InitialDistribution {
public:
    explicit InitialDistribution(const std::string &file) : file(file) {
        check(mlh_read_initial_count(file.c_str(), &n), "InitialDistribution");
    }
    int getNumberOfParticles() const { return n; }
    void getAllParticles(Particles &particles) {
        mlh_particles_view v = particles.view();
        check(mlh_read_initial_distribution(file.c_str(), particles.dim, &v, particles.matId),
              "InitialDistribution::getAllParticles");
    }

private:
    std::string file;
    int n = 0;
};

// Domain (demonstrator/include/Domain.h:14-75, demonstrator/src/Domain.cpp):
// the bounds of a simulation and its uniform cell grid.  The GPU step builds
// the same grid itself; this class serves drivers that use it.
class Domain {
public:
    struct Cell {
        Cell() {}
        // bounds: [minX, minY, (minZ), maxX, maxY, (maxZ)] for `dim` axes
        explicit Cell(const double *bounds, int dim = settings_from_macros().cfg.dim) {
            minX = bounds[0]; maxX = bounds[dim];
            minY = bounds[1]; maxY = bounds[dim + 1];
            if (dim == 3) { minZ = bounds[2]; maxZ = bounds[dim + 2]; }
        }
        double minX = 0., maxX = 0., minY = 0., maxY = 0., minZ = 0., maxZ = 0.;
        std::vector<int> prtcls{};
    };

    explicit Domain(Cell bounds, int dim = settings_from_macros().cfg.dim) : bounds(bounds), dim(dim) {}

    // Domain::createGrid (Domain.cpp:9-54)
    void createGrid(const double &kernelSize) {
        cellsX = (int)std::floor((bounds.maxX - bounds.minX) / kernelSize);
        cellsY = (int)std::floor((bounds.maxY - bounds.minY) / kernelSize);
        cellsZ = dim == 3 ? (int)std::floor((bounds.maxZ - bounds.minZ) / kernelSize) : 1;
        numGridCells = cellsX * cellsY * (dim == 3 ? cellsZ : 1);
        cellSizeX = (bounds.maxX - bounds.minX) / (double)cellsX;
        cellSizeY = (bounds.maxY - bounds.minY) / (double)cellsY;
        if (dim == 3) cellSizeZ = (bounds.maxZ - bounds.minZ) / (double)cellsZ;
        grid.assign(numGridCells > 0 ? numGridCells : 0, Cell());
        for (int c = 0; c < numGridCells; ++c) {
            const int iX = c % cellsX, iY = (c / cellsX) % cellsY, iZ = dim == 3 ? c / (cellsX * cellsY) : 0;
            Cell &g = grid[c];
            g.minX = iX * cellSizeX + bounds.minX; g.maxX = (iX + 1) * cellSizeX + bounds.minX;
            g.minY = iY * cellSizeY + bounds.minY; g.maxY = (iY + 1) * cellSizeY + bounds.minY;
            if (dim == 3) { g.minZ = iZ * cellSizeZ + bounds.minZ; g.maxZ = (iZ + 1) * cellSizeZ + bounds.minZ; }
        }
    }

    // Domain::getNeighborCells (Domain.cpp:83-118): 3^dim cells, x outermost,
    // -1 outside the grid.
    void getNeighborCells(const int &iCell, int *neighborCells) const {
        const int iX = iCell % cellsX, iY = (iCell / cellsX) % cellsY, iZ = dim == 3 ? iCell / (cellsX * cellsY) : 0;
        int k = 0;
        for (int a = iX - 1; a <= iX + 1; ++a)
            for (int b = iY - 1; b <= iY + 1; ++b)
                for (int c = (dim == 3 ? iZ - 1 : 0); c <= (dim == 3 ? iZ + 1 : 0); ++c) {
                    const bool out = a < 0 || a >= cellsX || b < 0 || b >= cellsY || (dim == 3 && (c < 0 || c >= cellsZ));
                    neighborCells[k++] = out ? -1 : a + b * cellsX + c * cellsX * cellsY;
                }
    }

    int numGridCells = 0;
    std::vector<Cell> grid;
    Cell bounds;
    int dim;
    int cellsX = 0, cellsY = 0, cellsZ = 0;
    double cellSizeX = 0., cellSizeY = 0., cellSizeZ = 0.;
};

// Riemann (demonstrator/include/Riemann.h:15-41): one face, WL the left
// (particle i) and WR the right state, [rho, P, v...] in the frame of
// vFrame, as Particles::solveRiemannProblems passes them.  exact() solves it
// on the GPU (mlh_riemann_fluxes); a batch of faces is far cheaper through
// that call directly.  Unlike the reference, the constructor does not rotate
// WR and WL in place.
class Riemann {
public:
    Riemann(double *WR, double *WL, double *vFrame, double *Aij, int i, int dim = settings_from_macros().cfg.dim)
        : WR(WR), WL(WL), vFrame(vFrame), Aij(Aij), i(i), dim(dim) {}
    void exact(double *Fij, const double &gamma, int meshlessFiniteMass = settings_from_macros().cfg.meshless_finite_mass) {
        int iters = 0;
        const int st = mlh_riemann_fluxes(dim, 1, WL, WR, vFrame, Aij, gamma, meshlessFiniteMass, Fij, &iters);
        if (st & (MLH_ERR_INVALID | MLH_ERR_CUDA | MLH_ERR_NO_DEVICE)) throw Error("Riemann::exact", st);
        status = st;
    }
    int status = 0;   // MLH_ERR_NEWTON / MLH_ERR_VACUUM of the last solve (the reference only warns)

private:
    double *WR, *WL, *vFrame, *Aij;
    int i, dim;
};

// MeshlessScheme (demonstrator/include/MeshlessScheme.h:17-45): the time
// loop of MeshlessScheme::run (demonstrator/src/MeshlessScheme.cpp:21-253)
// with its dump schedule, each step on the GPU.
class MeshlessScheme {
public:
    struct Configuration {
        std::string initFile;
        std::string outDir;
        double timeStep = 0.;
        double timeEnd = 0.;
        int h5DumpInterval = 1;
        double periodicBoxLimits[6] = {0., 0., 0., 0., 0., 0.};   // [lower.., upper..] for DIM axes
        double kernelSize = 0.;
        double gamma = 5. / 3.;
    };

    MeshlessScheme(Configuration config, Particles *particles, Domain::Cell bounds,
                   const mlh_run_config &settings = settings_from_macros())
        : config(config), particles(particles), domain(bounds, settings.cfg.dim), settings(settings) {
        mlh_config &c = this->settings.cfg;
        c.kernel_size = config.kernelSize;
        c.gamma = config.gamma;
        c.time_step = config.timeStep;
        const double lo[3] = {bounds.minX, bounds.minY, bounds.minZ}, hi[3] = {bounds.maxX, bounds.maxY, bounds.maxZ};
        for (int a = 0; a < 3; ++a) {
            c.box_lo[a] = a < c.dim ? (c.periodic ? config.periodicBoxLimits[a] : lo[a]) : 0.;
            c.box_hi[a] = a < c.dim ? (c.periodic ? config.periodicBoxLimits[c.dim + a] : hi[a]) : 0.;
        }
        domain.createGrid(config.kernelSize);
        mlh_particles_view v = particles->view();
        check(mlh_create(&c, &v, &ctx), "MeshlessScheme");
    }
    ~MeshlessScheme() { mlh_destroy(ctx); }
    MeshlessScheme(const MeshlessScheme &) = delete;
    MeshlessScheme &operator=(const MeshlessScheme &) = delete;

    // Called with (time, step) after every completed step, when set.
    void (*onStep)(double, int, const mlh_step_stats &) = nullptr;
    // Called with the status bits of a step that reported non-physical
    // values; the default prints a warning to stderr and the run goes on.
    void (*onWarning)(int, double, int) = nullptr;
    // Stops the loop after this many steps (0: run to timeEnd).
    int maxSteps = 0;

    void run() {
        const bool adaptive = settings.cfg.adaptive_timestep != 0;
        double t = 0., timeStep = config.timeStep;
        int step = 0;
        // MeshlessScheme.cpp:25-36
        const int numDumpTimes = adaptive ? (int)(config.timeEnd / config.timeStep) / config.h5DumpInterval + 1 : 0;
        std::vector<double> dumpTimes((size_t)std::max(numDumpTimes, 1));
        for (int k = 0; k < numDumpTimes; ++k) dumpTimes[k] = k * config.timeStep * config.h5DumpInterval;
        int dumpStep = 0;
        bool dump = true, dumpNext = false;
        do {
            double dtMax = 0., target = 0.;
            bool hasTarget = false;
            if (adaptive) {
                // MeshlessScheme.cpp:93-101: the step ends on the next dump time
                if (dumpStep >= numDumpTimes) throw Error("MeshlessScheme::run: no dump time left before timeEnd", MLH_ERR_INVALID);
                if (dumpStep + 1 < numDumpTimes) {
                    hasTarget = true;
                    target = dumpTimes[dumpStep + 1];
                    dtMax = target - t;
                }
            }
            const bool dumpNow = adaptive ? dump : (step % config.h5DumpInterval == 0);
            if (dumpNow) {
                // the fields the reference dumps are those of this step's first
                // stages (MeshlessScheme.cpp:163-190)
                warn(check_fatal(mlh_prepare(ctx, dtMax), "mlh_prepare"), t, step);
                fetchFields();
                std::ostringstream name;
                name << std::setw(6) << std::setfill('0') << (adaptive ? dumpStep : step);
                particles->dump2file(config.outDir + "/" + name.str() + ".h5", t);
                ++dumpStep;
                if (adaptive) dump = false;
            }
            if (t >= config.timeEnd) break;
            if (maxSteps > 0 && step >= maxSteps) break;
            mlh_step_stats st;
            warn(check_fatal(mlh_step(ctx, 1, dtMax, &st), "mlh_step"), t, step);
            timeStep = st.dt;
            // the reference sets dumpNext when t + dt reaches the dump time it
            // clamped to (MeshlessScheme.cpp:98-101)
            if (adaptive) dumpNext = hasTarget && (timeStep == dtMax || t + timeStep >= target);
            t += timeStep;
            ++step;
            if (onStep) onStep(t, step, st);
            if (adaptive && dumpNext) { dump = true; dumpNext = false; }
        } while (t < config.timeEnd + timeStep);
        fetchState();
        time = t;
        steps = step;
    }

    mlh_ctx *context() { return ctx; }
    double time = 0.;
    int steps = 0;

private:
    void warn(int status, double t, int step) {
        if (!status) return;
        if (onWarning) { onWarning(status, t, step); return; }
        std::fprintf(stderr, "WARNING: step %d (t = %g): status 0x%x (see mlh_status_bits)\n", step, t, status);
    }
    void fetchState() {
        mlh_particles_view v = particles->view();
        check(mlh_get_fields(ctx, &v), "mlh_get_fields");
    }
    void fetchFields() {
        fetchState();
        const long long n = particles->N;
        long long cnt = 0;
        check(mlh_stage_array(ctx, "rho", particles->rho, n, &cnt), "rho");
        check(mlh_stage_array(ctx, "P", particles->P, n, &cnt), "P");
        check(mlh_stage_array(ctx, "omega", particles->omega, n, &cnt), "omega");
        check(mlh_stage_array(ctx, "noi", particles->noi, n, &cnt), "noi");
        std::vector<double> g((size_t)n * 3);
        check(mlh_stage_array(ctx, "grad_rho", g.data(), n * 3, &cnt), "grad_rho");
        std::memcpy(&particles->rhoGrad[0][0], g.data(), sizeof(double) * g.size());
    }

    Configuration config;
    Particles *particles;
    Domain domain;
    mlh_run_config settings;
    mlh_ctx *ctx = nullptr;
};

}  // namespace mlh

#endif  // MLH_HPP
