// mlh: command-line driver of the GB300 MFV step with the reference's command
// line and inputs (demonstrator/src/main.cpp:16-117):
//
//     mlh -c config.info [-p parameter.h] [-v | -s] [--max-steps N]
//
// config.info as the reference reads it (initFile, outDir, timeStep, timeEnd,
// h5DumpInterval, periodicBoxLimits, kernelSize, gamma); the compile-time
// switches of the reference's parameter.h are read at run time from -p (the
// defaults are the MFV settings of demonstrator/include/parameter.h).  The
// initial distribution and the snapshots are the reference's HDF5 files.
#include "../../include/mlh.hpp"

#include <cstdlib>
#include <iostream>
#include <sys/stat.h>

namespace {

int verbosity = 1;   // 0 silent, 1 info, 2 debug

void usage() {
    std::cout << "mlh: GB300 meshless finite volume (MFV) step\n"
                 "  -c, --config FILE      config.info (default config.info)\n"
                 "  -p, --parameters FILE  parameter.h with the run's DIM, PERIODIC_BOUNDARIES, ... switches\n"
                 "  -v, --verbose          print every step\n"
                 "  -s, --silent           print warnings only\n"
                 "      --max-steps N      stop after N steps\n"
                 "  -h, --help             this text\n";
}

void on_step(double t, int step, const mlh_step_stats &st) {
    if (verbosity >= 2)
        std::cout << "  > TIME: " << t << ", STEP: " << step << ", dt = " << st.dt << ", faces " << st.faces
                  << ", device " << st.device_ms << " ms" << std::endl;
}

}  // namespace

int main(int argc, char **argv) {
    std::string config = "config.info", params;
    int max_steps = 0;
    bool verbose = false, silent = false;
    for (int k = 1; k < argc; ++k) {
        const std::string a = argv[k];
        auto next = [&]() -> std::string {
            if (k + 1 >= argc) { std::cerr << "missing value after " << a << "\n"; std::exit(2); }
            return argv[++k];
        };
        if (a == "-c" || a == "--config") config = next();
        else if (a == "-p" || a == "--parameters") params = next();
        else if (a == "-v" || a == "--verbose") verbose = true;
        else if (a == "-s" || a == "--silent") silent = true;
        else if (a == "--max-steps") max_steps = std::atoi(next().c_str());
        else if (a == "-h" || a == "--help") { usage(); return 0; }
        else { std::cerr << "unknown option " << a << "\n"; usage(); return 2; }
    }
    if (verbose && silent) {
        std::cerr << "Command line options -s and -v are incompatible\n";
        return 2;
    }
    verbosity = silent ? 0 : (verbose ? 2 : 1);
    try {
        mlh_run_config run;
        mlh_default_run_config(&run);
        if (!params.empty()) mlh::check(mlh_read_parameter_header(params.c_str(), &run), "parameter.h");
        mlh::check(mlh_read_config_info(config.c_str(), &run), "config.info");
        const int dim = run.cfg.dim;
        mlh::MeshlessScheme::Configuration conf;
        conf.initFile = run.init_file;
        conf.outDir = run.out_dir;
        conf.timeStep = run.cfg.time_step;
        conf.timeEnd = run.time_end;
        conf.h5DumpInterval = run.h5_dump_interval;
        conf.kernelSize = run.cfg.kernel_size;
        conf.gamma = run.cfg.gamma;
        for (int a = 0; a < dim; ++a) {
            conf.periodicBoxLimits[a] = run.cfg.box_lo[a];
            conf.periodicBoxLimits[dim + a] = run.cfg.box_hi[a];
        }
        if (verbosity >= 1)
            std::cout << "Reading configuration ... DIM " << dim << ", periodic " << run.cfg.periodic << ", adaptive dt "
                      << run.cfg.adaptive_timestep << ", kernelSize " << conf.kernelSize << ", gamma " << conf.gamma
                      << ", timeStep " << conf.timeStep << ", timeEnd " << conf.timeEnd << std::endl;
        mlh::InitialDistribution init(conf.initFile);
        mlh::Particles particles(init.getNumberOfParticles(), false, dim);
        init.getAllParticles(particles);
        if (verbosity >= 1) std::cout << "    > N = " << particles.N << std::endl;
        double limits[6];
        if (run.cfg.periodic) for (int a = 0; a < 2 * dim; ++a) limits[a] = conf.periodicBoxLimits[a];
        else particles.getDomainLimits(limits);
        mlh::Domain::Cell bbox(limits, dim);
        mkdir(conf.outDir.c_str(), 0755);
        mlh::MeshlessScheme scheme(conf, &particles, bbox, run);
        scheme.onStep = on_step;
        scheme.maxSteps = max_steps;
        if (verbosity >= 1) std::cout << "Starting time integration ..." << std::endl;
        scheme.run();
        if (verbosity >= 1)
            std::cout << "... done: t = " << scheme.time << " after " << scheme.steps << " steps" << std::endl;
    } catch (const std::exception &e) {
        std::cerr << "mlh: " << e.what() << std::endl;
        return 1;
    }
    return 0;
}
