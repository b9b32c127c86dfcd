// TEST INFRASTRUCTURE (oracle build of the reference).
//
// Drives the reference demonstrator's own Particles / Domain / Helper code,
// compiled unmodified from the reference tree by oracle/build_ref.sh, through
// the stage sequence of MeshlessScheme::run (demonstrator/src/MeshlessScheme.cpp:
// 39-253) without snapshot dumps and without the dump-time clamp of dt, and
// writes the per-stage arrays of the first step plus the state after the
// last step to a binary file (read by tests/golden/make_golden.py).
//
// Usage: ref_harness IN OUT NSTEPS kernelSize gamma timeStep lo0 lo1 lo2 hi0 hi1 hi2
// IN holds int64 N followed by x, y, (z), vx, vy, (vz), m, u as float64[N].
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "Particles.h"
#include "Domain.h"
#include "Helper.h"

structlog LOGCFG = {};

namespace {

FILE *out_fp = nullptr;

void put(const std::string &name, char type, const void *data, uint64_t count) {
    uint32_t len = (uint32_t)name.size();
    fwrite(&len, 4, 1, out_fp);
    fwrite(name.data(), 1, len, out_fp);
    fwrite(&type, 1, 1, out_fp);
    fwrite(&count, 8, 1, out_fp);
    fwrite(data, type == 'd' ? 8 : 4, count, out_fp);
}
void putd(const std::string &n, const std::vector<double> &v) { put(n, 'd', v.data(), v.size()); }
void puti(const std::string &n, const std::vector<int32_t> &v) { put(n, 'i', v.data(), v.size()); }

const unsigned IMG_SHIFT = 29;

struct Dumper {
    Particles &p;
#if PERIODIC_BOUNDARIES
    Particles &g;
    Dumper(Particles &p_, Particles &g_) : p(p_), g(g_) {}
#else
    explicit Dumper(Particles &p_) : p(p_) {}
#endif
    int N() const { return p.N; }
    int noiG(int i) const {
#if PERIODIC_BOUNDARIES
        return p.noiGhosts[i];
#else
        (void)i; return 0;
#endif
    }
    // slot -> pointer into a per-interaction array (real, then ghosts)
    template <class T, int W>
    void slots(const std::string &name, T (*real)[W], T (*ghost)[W], int width) {
        std::vector<double> v;
        for (int i = 0; i < N(); ++i) {
            for (int j = 0; j < p.noi[i]; ++j)
                for (int k = 0; k < width; ++k) v.push_back(real[i * MAX_NUM_INTERACTIONS + j][k]);
#if PERIODIC_BOUNDARIES
            for (int j = 0; j < noiG(i); ++j)
                for (int k = 0; k < width; ++k) v.push_back(ghost[i * MAX_NUM_GHOST_INTERACTIONS + j][k]);
#else
            (void)ghost;
#endif
        }
        putd(name, v);
    }
    void lists() {
        std::vector<int32_t> off(1, 0), noi, noiImg, nnl;
        for (int i = 0; i < N(); ++i) {
            for (int j = 0; j < p.noi[i]; ++j) nnl.push_back(p.nnl[i * MAX_NUM_INTERACTIONS + j]);
#if PERIODIC_BOUNDARIES
            for (int j = 0; j < noiG(i); ++j) {
                int gi = p.nnlGhosts[i * MAX_NUM_GHOST_INTERACTIONS + j];
                int par = g.parent[gi];
                uint32_t e = (uint32_t)par;
                if (g.x[gi] != p.x[par]) e |= 1u << IMG_SHIFT;
                if (g.y[gi] != p.y[par]) e |= 1u << (IMG_SHIFT + 1);
                nnl.push_back((int32_t)e);
            }
#endif
            noi.push_back(p.noi[i]);
            noiImg.push_back(noiG(i));
            off.push_back(off.back() + p.noi[i] + noiG(i));
        }
        puti("off", off); puti("noi", noi); puti("noi_img", noiImg); puti("nnl", nnl);
    }
    void vec(const std::string &name, double *a) { putd(name, std::vector<double>(a, a + N())); }
    void grad(const std::string &name, double (*a)[DIM]) {
        std::vector<double> v;
        for (int i = 0; i < N(); ++i) for (int k = 0; k < 3; ++k) v.push_back(k < DIM ? a[i][k] : 0.);
        putd(name, v);
    }
    void state(const std::string &pre) {
        vec(pre + "x", p.x); vec(pre + "y", p.y);
#if DIM == 3
        vec(pre + "z", p.z);
#endif
        vec(pre + "vx", p.vx); vec(pre + "vy", p.vy);
#if DIM == 3
        vec(pre + "vz", p.vz);
#endif
        vec(pre + "m", p.m); vec(pre + "u", p.u);
    }
    void grads(const std::string &pre) {
        grad(pre + "rho", p.rhoGrad); grad(pre + "vx", p.vxGrad); grad(pre + "vy", p.vyGrad);
#if DIM == 3
        grad(pre + "vz", p.vzGrad);
#endif
        grad(pre + "P", p.PGrad);
    }
};

}  // namespace

int main(int argc, char **argv) {
    if (argc < 13) { fprintf(stderr, "usage: %s IN OUT NSTEPS h gamma dt lo0 lo1 lo2 hi0 hi1 hi2\n", argv[0]); return 2; }
    LOGCFG.level = ERROR;
    const char *in = argv[1];
    int nsteps = atoi(argv[3]);
    double kernelSize = atof(argv[4]), gamma = atof(argv[5]), timeStepCfg = atof(argv[6]);
    double box[2 * DIM];
    for (int a = 0; a < DIM; ++a) { box[a] = atof(argv[7 + a]); box[DIM + a] = atof(argv[10 + a]); }

    FILE *fi = fopen(in, "rb");
    if (!fi) return 3;
    int64_t n64;
    if (fread(&n64, 8, 1, fi) != 1) return 3;
    int N = (int)n64;
    Particles particles(N);
    double *dst[8] = {particles.x, particles.y,
#if DIM == 3
                      particles.z,
#endif
                      particles.vx, particles.vy,
#if DIM == 3
                      particles.vz,
#endif
                      particles.m, particles.u};
    for (int k = 0; k < 2 * DIM + 2; ++k)
        if (fread(dst[k], 8, N, fi) != (size_t)N) return 3;
    fclose(fi);
    for (int i = 0; i < N; ++i) particles.matId[i] = 0;

    out_fp = fopen(argv[2], "wb");
    if (!out_fp) return 4;

#if PERIODIC_BOUNDARIES
    double *domainLimits = box;
#else
    double domainLimits[DIM * 2];
    particles.getDomainLimits(domainLimits);
#endif
    Domain domain(Domain::Cell{domainLimits});
#if PERIODIC_BOUNDARIES
    Particles ghostParticles(DIM * N, true);
    Dumper dump(particles, ghostParticles);
#else
    Particles ghostParticles(0, true);
    Dumper dump(particles);
#endif
    Helper helper{};
    domain.createGrid(kernelSize);
    std::vector<double> dts;

    for (int step = 0; step < nsteps; ++step) {
        const bool first = step == 0;
#if !PERIODIC_BOUNDARIES
        double lim[DIM * 2];
        particles.getDomainLimits(lim);
        domain.bounds = Domain::Cell{lim};
        domain.createGrid(kernelSize);
#endif
        particles.assignParticlesAndCells(domain);
#if PERIODIC_BOUNDARIES
        particles.createGhostParticles(domain, ghostParticles, kernelSize);
#endif
        particles.gridNNS(domain, kernelSize);
#if PERIODIC_BOUNDARIES
        particles.ghostNNS(domain, ghostParticles, kernelSize);
#endif
        particles.compDensity(kernelSize);
#if PERIODIC_BOUNDARIES
        particles.compDensity(ghostParticles, kernelSize);
#endif
        particles.compPressure(gamma);
#if ADAPTIVE_TIMESTEP
        double timeStep = particles.compGlobalTimestep(gamma, kernelSize);
#else
        double timeStep = timeStepCfg;
#endif
        dts.push_back(timeStep);
        if (first) {
            dump.state("in_");
            dump.lists();
            dump.vec("omega", particles.omega);
            dump.vec("rho", particles.rho);
            dump.vec("P", particles.P);
            putd("dt", std::vector<double>(1, timeStep));
            std::vector<double> grid = {domain.bounds.minX, domain.bounds.minY,
#if DIM == 3
                                        domain.bounds.minZ,
#else
                                        0.,
#endif
                                        domain.bounds.maxX, domain.bounds.maxY,
#if DIM == 3
                                        domain.bounds.maxZ,
#else
                                        0.,
#endif
                                        (double)domain.cellsX, (double)domain.cellsY,
#if DIM == 3
                                        (double)domain.cellsZ
#else
                                        0.
#endif
            };
            putd("grid", grid);
        }
#if PERIODIC_BOUNDARIES
        particles.updateGhostState(ghostParticles);
        particles.compPsijTilde(helper, ghostParticles, kernelSize);
        particles.gradient(particles.rho, particles.rhoGrad, ghostParticles.rho, ghostParticles);
        particles.gradient(particles.vx, particles.vxGrad, ghostParticles.vx, ghostParticles);
        particles.gradient(particles.vy, particles.vyGrad, ghostParticles.vy, ghostParticles);
#if DIM == 3
        particles.gradient(particles.vz, particles.vzGrad, ghostParticles.vz, ghostParticles);
#endif
        particles.gradient(particles.P, particles.PGrad, ghostParticles.P, ghostParticles);
        particles.updateGhostGradients(ghostParticles);
        if (first) dump.grads("gradraw_");
#if SLOPE_LIMITING
        particles.slopeLimiter(kernelSize, &ghostParticles);
        particles.updateGhostGradients(ghostParticles);
#endif
#else
        particles.compPsijTilde(helper, kernelSize);
        particles.gradient(particles.rho, particles.rhoGrad);
        particles.gradient(particles.vx, particles.vxGrad);
        particles.gradient(particles.vy, particles.vyGrad);
#if DIM == 3
        particles.gradient(particles.vz, particles.vzGrad);
#endif
        particles.gradient(particles.P, particles.PGrad);
        if (first) dump.grads("gradraw_");
#if SLOPE_LIMITING
        particles.slopeLimiter(kernelSize);
#endif
#endif
        if (first) dump.grads("grad_");
        particles.compEffectiveFace();
#if PERIODIC_BOUNDARIES
        particles.compEffectiveFace(ghostParticles);
#endif
        particles.compRiemannStatesLR(timeStep, kernelSize, gamma);
#if PERIODIC_BOUNDARIES
        particles.compRiemannStatesLR(timeStep, kernelSize, gamma, ghostParticles);
#endif
        if (first) {
#if PERIODIC_BOUNDARIES
            dump.slots<double, DIM>("psi", particles.psijTilde_xi, particles.psijTilde_xiGhosts, DIM);
            dump.slots<double, DIM>("Aij", particles.Aij, particles.AijGhosts, DIM);
            dump.slots<double, DIM>("vFrame", particles.vFrame, particles.vFrameGhosts, DIM);
            dump.slots<double, DIM + 2>("WL", particles.WijL, particles.WijLGhosts, DIM + 2);
            dump.slots<double, DIM + 2>("WR", particles.WijR, particles.WijRGhosts, DIM + 2);
#else
            dump.slots<double, DIM>("psi", particles.psijTilde_xi, particles.psijTilde_xi, DIM);
            dump.slots<double, DIM>("Aij", particles.Aij, particles.Aij, DIM);
            dump.slots<double, DIM>("vFrame", particles.vFrame, particles.vFrame, DIM);
            dump.slots<double, DIM + 2>("WL", particles.WijL, particles.WijL, DIM + 2);
            dump.slots<double, DIM + 2>("WR", particles.WijR, particles.WijR, DIM + 2);
#endif
        }
        particles.solveRiemannProblems(gamma, ghostParticles);
        particles.collectFluxes(helper, ghostParticles);
        if (first) {
#if PERIODIC_BOUNDARIES
            dump.slots<double, DIM + 2>("F", particles.Fij, particles.FijGhosts, DIM + 2);
#else
            dump.slots<double, DIM + 2>("F", particles.Fij, particles.Fij, DIM + 2);
#endif
            dump.vec("mF", particles.mF);
            dump.vec("eF", particles.eF);
            dump.grad("vF", particles.vF);
        }
        particles.updateStateAndPosition(timeStep, domain);
        if (first) dump.state("s1_");
    }
    putd("dts", dts);
    dump.state("out_");
    fclose(out_fp);
    return 0;
}
