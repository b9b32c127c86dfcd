/*
 * meshlesshydro-gb300: host-side input and output of the reference's run
 * (jammartin/meshlessHydro, demonstrator/): config.info, parameter.h and the
 * HDF5 initial-condition and snapshot files.  Plain C ABI; nothing here needs
 * a GPU.  Every function returns 0 or MLH_ERR_* bits (include/mlh.h) with a
 * message in mlh_last_error().
 */
#ifndef MLH_IO_H
#define MLH_IO_H

#include "mlh.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Everything the reference's main() and MeshlessScheme::Configuration read
 * (demonstrator/src/main.cpp:55-85, demonstrator/include/MeshlessScheme.h:20-29)
 * plus the step settings. */
typedef struct mlh_run_config {
    mlh_config cfg;            /* parameter.h switches + kernelSize, gamma, timeStep, box */
    char init_file[1024];      /* initFile */
    char out_dir[1024];        /* outDir */
    double time_end;           /* timeEnd */
    int h5_dump_interval;      /* h5DumpInterval */
    int debug_lvl;             /* DEBUG_LVL */
} mlh_run_config;

/* Settings of the reference's defaults (demonstrator/include/parameter.h with
 * RUNSPH off): DIM 2, PERIODIC_BOUNDARIES 1, ADAPTIVE_TIMESTEP 1, CFL .2,
 * SLOPE_LIMITING 1, BETA 4, PAIRWISE_LIMITER 1, PSI_1 .5, PSI_2 .25,
 * MESHLESS_FINITE_MASS 0, MOVE_PARTICLES 1, FIRST_ORDER_QUAD_POINT 1,
 * kernelSize .025, gamma 5/3. */
void mlh_default_run_config(mlh_run_config *run);

/* Applies the `#define NAME value` lines of a parameter.h
 * (demonstrator/include/parameter.h:9-74, testcases/<case>/parameter.h) to
 * run->cfg with the preprocessor's meaning: a switch that the file does not
 * define reads as 0 in the reference's `#if`, so every switch is first set to
 * 0 and numbers keep their defaults.  RUNSPH 1 (the SPH path) and
 * ENFORCE_FLUX_SYM 0 are rejected (MLH_ERR_INVALID); MAX_NUM_INTERACTIONS
 * sets max_neighbours; DEBUG_LVL is recorded. */
int mlh_read_parameter_header(const char *path, mlh_run_config *run);

/* Reads a config.info (Boost property_tree INFO syntax: `key value` lines,
 * `;` comments, `name { ... }` blocks; demonstrator/config.info:1-33) into
 * run: initFile, outDir, timeStep, timeEnd, h5DumpInterval, kernelSize,
 * gamma and, when run->cfg.periodic, periodicBoxLimits (lowerX .. upperZ) as
 * main.cpp:55-85 reads them.  A missing key is an error, as getVal throws
 * in the reference (periodicBoxLimits only when periodic, lowerZ/upperZ only
 * in 3D). */
int mlh_read_config_info(const char *path, mlh_run_config *run);

/* Value of one key of a config.info, found by its path of block names and
 * key joined by '.' ("kernelSize", "periodicBoxLimits.lowerX"), as text
 * (what ConfigParser::getVal / getObj of demonstrator/src/ConfigParser.cpp
 * reach).  A missing key returns MLH_ERR_INVALID; out (cap bytes) receives
 * the value, truncated to fit. */
int mlh_info_get(const char *file, const char *key_path, char *out, int cap);

/* ---------------------------------------------------------------- HDF5 */
/* A minimal HDF5 (file-format specification, superblock versions 0 and 1)
 * reader and writer for what the reference exchanges: datasets of rank 1 or
 * 2 in the root group, little- or big-endian IEEE floats and integers,
 * contiguous or compact storage.  Groups below the root, chunked or filtered
 * (compressed) datasets and superblock versions 2 and 3 are rejected with a
 * message.  Files are written with superblock version 0, a symbol-table root
 * group and contiguous little-endian datasets. */

/* Rank (1 or 2), dimensions and element class (0 floating point, 1 integer)
 * and size in bytes of dataset `name` ("/x" or "x") of an HDF5 file. */
int mlh_h5_dataset_info(const char *file, const char *name, int *rank, long long dims[2], int *elem_class,
                        int *elem_size);
/* All elements of a dataset converted to double or int (count must equal the
 * product of its dimensions; row-major). */
int mlh_h5_read_f64(const char *file, const char *name, double *out, long long count);
int mlh_h5_read_i32(const char *file, const char *name, int *out, long long count);

typedef struct mlh_h5_writer mlh_h5_writer;
int mlh_h5_create(const char *file, mlh_h5_writer **out);
/* Adds a dataset (copied at once); rank 1 or 2, dims[0] x dims[1]. */
int mlh_h5_add_f64(mlh_h5_writer *w, const char *name, int rank, const long long *dims, const double *data);
int mlh_h5_add_i32(mlh_h5_writer *w, const char *name, int rank, const long long *dims, const int *data);
/* Writes the file and frees the writer (also on error). */
int mlh_h5_close(mlh_h5_writer *w);

/* InitialDistribution (demonstrator/src/InitialDistribution.cpp:7-59): number
 * of particles of an initial-condition file (/m, /x, /v, /u, /materialId must
 * agree in length, else MLH_ERR_INVALID as the reference's length_error). */
int mlh_read_initial_count(const char *file, int *n);
/* Fills the caller's arrays (n = v->n particles): x, y (, z), vx, vy (, vz)
 * from the first dim columns of /x and /v, m, u and, when material_id is not
 * NULL, /materialId. */
int mlh_read_initial_distribution(const char *file, int dim, mlh_particles_view *v, int *material_id);

/* Particles::dump2file (demonstrator/src/Particles.cpp:2978-3076): /time,
 * /totalMass, /energy, /xMomentum, /yMomentum (, /zMomentum) (the sums of
 * Particles.cpp:2839-2886, in particle order), /rho, /m, /u, /P, /noi, /x,
 * /v, /rhoGrad (N x dim) and, when material_id is not NULL, /materialId, so
 * that a snapshot can be read back as an initial distribution.  rho_grad:
 * N x 3 doubles per particle (the first dim written). */
int mlh_write_snapshot(const char *file, int dim, const mlh_particles_view *v, const double *rho, const double *P,
                       const double *rho_grad, const int *noi, const int *material_id, double time);

#ifdef __cplusplus
}
#endif
#endif /* MLH_IO_H */
