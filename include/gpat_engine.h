/*
 * gpat_engine.h -- C ABI of the GB300 particle-mover engine for GPAT
 * (stochastic integration of Parker's transport equation).
 *
 * The entry points replace, one for one, the Fortran module procedures the
 * reference driver calls on its hot path (paths are relative to the
 * xiaocanli/stochastic-parker project root).  The Fortran driver reaches them
 * through an ISO_C_BINDING interface module; every argument is a plain
 * pointer, integer or double, and no call retains a caller pointer.
 *
 * Conventions
 *  - Every call returns GPAT_OK (0) or a negative GPAT_ERR_* code;
 *    gpat_last_error() gives a message.  Nothing throws across the ABI.
 *  - Host buffers stay owned by the caller; device memory is owned by the
 *    handle.  Calls are synchronous on return.
 *  - One host thread per handle; a handle is bound to one CUDA device.
 *  - Frame indices (ct_mhd, mhd_tframe) are 1-based as in the reference.
 *
 * Reference differences that are part of the contract
 *  - Random increments come from Philox-4x32-10 keyed by (seed, particle
 *    tags, push counter) instead of per-thread MT19937 streams, so results
 *    are reproducible for any launch shape.
 *  - remove_particles keeps the survivors in their original order on the
 *    FP64 path and bins them by field cell on the split-precision path; the
 *    reference swaps removed particles to the end.  Particle sets, counters
 *    and histograms are unaffected by the order.
 *  - leak, leak_negp and all histogram weights are accumulated as exact
 *    128-bit fixed point (64 fraction bits), so sums do not depend on order.
 */
#ifndef GPAT_ENGINE_H
#define GPAT_ENGINE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPAT_OK 0
#define GPAT_ERR_ARG (-1)          /* invalid argument or NULL pointer          */
#define GPAT_ERR_OOM (-2)          /* device or host allocation failed          */
#define GPAT_ERR_CAPACITY (-3)     /* nptl_max reached (data kept up to the cap) */
#define GPAT_ERR_TIMEOUT (-4)      /* a bounded device wait gave up              */
#define GPAT_ERR_CUDA (-5)         /* CUDA runtime error                         */
#define GPAT_ERR_UNSUPPORTED (-6)  /* option outside the engine's scope          */
#define GPAT_ERR_IO (-7)           /* file missing, short or malformed           */
#define GPAT_ERR_STATE (-8)        /* call out of order (e.g. no fields yet)     */
#define GPAT_ERR_DEVICE (-9)       /* device status word set (NaN / index guard) */

#define GPAT_PREC_FP64 0    /* FP64 everywhere, reference operation order      */
#define GPAT_PREC_MIXED 1   /* FP32 fields/kappa/drift, compensated sums       */

#define GPAT_NOISE_UNIFORM 0  /* (2u-1)*sqrt(3), the reference's increment    */
#define GPAT_NOISE_GAUSS 1    /* Box-Muller Gaussian increments               */

#define GPAT_COUNT_FLAG_INBOX 1
#define GPAT_COUNT_FLAG_OTHERS 0

/* mhd_configuration: same fields, order and binary layout (13 doubles then
 * 13 int32, 156 bytes) as mhd_config.dat; src/modules/mhd_config.f90:16-27. */
typedef struct gpat_mhd_config {
    double dx, dy, dz, xmin, ymin, zmin, xmax, ymax, zmax, lx, ly, lz, dt_out;
    int32_t nx, ny, nz, nxs, nys, nzs, topox, topoy, topoz, nvar, bcx, bcy, bcz;
} gpat_mhd_config_t;

/* Run parameters on the mover path.  The first block mirrors conf.dat as read
 * by read_particle_params (particle_module.f90:2778-2878) plus the drift,
 * boundary and diagnostics settings (set_drift_parameters :318-328,
 * read_particle_boundary_conditions simulation_setup.f90:104-150,
 * read_diagnostics_params diagnostics.f90:2049-2100). */
typedef struct gpat_params {
    double b0, p0, pmin, pmax;
    double gamma_turb, pindex, kpara0, kret, dt_min_rel, dt_max_rel;
    double acc_region[6];
    double drift1, drift2;
    int32_t momentum_dependency, mag_dependency, acc_region_flag, charge;
    int32_t check_drift_2d, ndim, pbcx, pbcy, pbcz, npp_global;
    uint64_t seed;
    int32_t noise;              /* GPAT_NOISE_*                                */
    int32_t precision;          /* GPAT_PREC_*                                 */
    int64_t nptl_max;           /* particle capacity (init_particles)          */
    int32_t time_interp;        /* 1: two field frames, linear in time         */
    /* dpp_wave / dpp_shear: momentum diffusion by wave scattering and flow
     * shear (set_dpp_params, particle_module.f90:255-272); deltab_flag /
     * correlation_flag: spatially dependent turbulence variance and
     * correlation length (set_flags_params :285-300, inputs through
     * gpat_read_magnetic_fluctuation / gpat_read_correlation_length);
     * spherical_coord / nonuniform_grid: the grid type of set_mhd_grid_type
     * (mhd_config.f90:179-186; x = r, y = theta, z = phi in spherical
     * coordinates; node positions through gpat_read_grid_positions or
     * gpat_set_grid_positions when non-uniform); include_3rd_dim: a 2D
     * run whose particles also move along z with the 3D diffusion tensor
     * (push_particle_2d_include_3rd / _ft, particle_module.f90:3979-4610;
     * ndim must be 2).  These seven need GPAT_PREC_FP64, and so does
     * ndim = 1 (push_particle_1d / _1d_ft, particle_module.f90:2993-3357;
     * fields shaped (nx + 4, 1, 1)). */
    int32_t dpp_wave, dpp_shear, deltab_flag, correlation_flag, include_3rd_dim;
    int32_t spherical_coord, nonuniform_grid;
    /* Split-precision mover only: pushes per particle between re-binnings of
     * the particle set by cell inside one gpat_particle_mover call (0: engine
     * default of 128; negative: bin once per call).  It changes memory
     * locality; results agree statistically for any value (a paused particle
     * resumes from its FP64 record, not from the FP32 working state). */
    int32_t bin_interval;
    int32_t weak_scattering;    /* flow-shear Dpp in the weak-scattering regime */
    /* Focused transport: pitch-angle diffusion coefficient at p0 (duu_init of
     * the reference CLI, stochastic-mhd.f90:935-937, default 10). */
    double duu0;
    double tau0;                /* scattering time at p0 (tau0_scattering, default 1) */
} gpat_params_t;

/* particle_type (particle_module.f90:38-50) as structure-of-arrays.  rng_ctr
 * is the per-particle Philox push counter that replaces the MT19937 state. */
typedef struct gpat_particles {
    double *x, *y, *z, *p, *v, *mu, *weight, *t, *dt;
    int8_t *split_times, *count_flag;
    int32_t *origin, *nsteps_tracked, *nsteps_pushed, *tag_injected, *tag_splitted;
    uint32_t *rng_ctr;
} gpat_particles_t;

/* Module-level state of particle_module (:65-79) plus engine statistics. */
typedef struct gpat_counters {
    int64_t nptl_current, nptl_split, nptl_escaped, tag_max;
    double leak, leak_negp;                     /* exact sums, rounded once   */
    uint64_t leak_hi, leak_lo, leak_negp_hi, leak_negp_lo;  /* raw fixed point */
    uint64_t steps;                             /* particle pushes, cumulative */
    double last_mover_ms;                       /* device time of last mover  */
    uint64_t last_mover_steps;
    int64_t last_mover_launches;                /* mover kernel launches used */
} gpat_counters_t;

typedef struct gpat_handle gpat_handle_t;

const char *gpat_version(void);

/* conf.dat reader.  Replaces read_particle_params (particle_module.f90:
 * 2778-2878) + read_config.f90:20-44: keys are searched forward from the
 * previous match without rewinding, by substring; a key that is not found
 * reads as -1.  pindex = 3 - gamma_turb.  Also reads pbcx/pbcy/pbcz
 * (simulation_setup.f90:104-150, from the start of the file) and
 * npp_global (diagnostics.f90:2049-2100).  Fields it does not read keep
 * the values already in *params. */
int gpat_read_particle_params(const char *conf_path, gpat_params_t *params);
/* get_variable (read_config.f90:20-44) for a single key from the file start. */
int gpat_get_variable(const char *conf_path, const char *key, double *value);
/* load_mhd_config (mhd_config.f90:139-148): 156-byte raw record. */
int gpat_load_mhd_config(const char *path, gpat_mhd_config_t *cfg);

/* init_particles + init_field_data + init_particle_distributions
 * (particle_module.f90:177-258, mhd_data_parallel.f90:66-105,
 * diagnostics.f90:178-226): allocates all device state on `device`. */
int gpat_create(const gpat_params_t *params, const gpat_mhd_config_t *cfg, int device,
                gpat_handle_t **out);
/* free_particles + free_field_data. */
int gpat_destroy(gpat_handle_t *h);
const char *gpat_last_error(const gpat_handle_t *h);

/* tstamps_mhd: load_tstamps_mhd / calc_tstamps_mhd (mhd_config.f90:218-271).
 * tstamps[0] is the reference's tstamps_mhd(1). */
int gpat_set_tstamps(gpat_handle_t *h, const double *tstamps, int n);
int gpat_calc_tstamps_mhd(gpat_handle_t *h, int t_start, int t_end);
/* load_tstamps_mhd (mhd_config.f90:221-255), for a varying MHD output
 * interval: <dir_mhd_data>time_stamps.dat holds the first frame as int32
 * (in an 8-byte slot), then one float64 per frame from the second slot on;
 * frames past tmax_mhd continue with the last interval. */
int gpat_load_tstamps_mhd(gpat_handle_t *h, int t_start, int t_end, int tmax_mhd,
                          const char *dir_mhd_data);

/* read_field_data_parallel (mhd_data_parallel.f90:224-300) from memory:
 * farray is the Fortran-order (nvar, nxg, nyg, nzg) single-precision array,
 * nvar = 8 (raw file layout vx vy vz rho bx by bz |B|) or 32 (with the 24
 * gradients).  var_flag 0 fills farray1, otherwise farray2. */
int gpat_set_fields(gpat_handle_t *h, int var_flag, const float *farray, int nvar);
/* read_field_data_parallel from a raw mhd_data_XXXX file (8 vars). */
int gpat_read_field_data(gpat_handle_t *h, const char *filename, int var_flag);
/* calc_fields_gradients (mhd_data_parallel.f90:504-610) on the device. */
/* Turbulence variance and correlation length (deltab_flag /
 * correlation_flag runs): read_magnetic_fluctuation and
 * read_correlation_length (mhd_data_parallel.f90:306-497) read a file of two
 * FP32 arrays over every ghost-padded node (slab, then 2D component); the
 * gradients are computed as calc_grad_sigma2_* / calc_grad_lc_*
 * (:771-1604).  gpat_set_fluctuations takes the four arrays from host
 * memory (NULL keeps a component; every component starts at 1, as the
 * reference initialises them).  gpat_get_fluctuations returns the 16-float
 * records {db2_slab, db2_2d, lc_slab, lc_2d} x {value, d/dx, d/dy, d/dz}. */
int gpat_set_fluctuations(gpat_handle_t *h, int var_flag, const float *db2_slab,
                          const float *db2_2d, const float *lc_slab, const float *lc_2d);
int gpat_read_magnetic_fluctuation(gpat_handle_t *h, const char *filename, int var_flag);
int gpat_read_correlation_length(gpat_handle_t *h, const char *filename, int var_flag);
int gpat_get_fluctuations(gpat_handle_t *h, int var_flag, float *aux);

int gpat_calc_fields_gradients(gpat_handle_t *h, int var_flag);
/* Node positions of a non-uniform grid (nonuniform_grid = 1), ghost nodes
 * included: nxg x values, nyg y values (2D, 3D) and nzg z values (3D), each
 * increasing (xpos_global of read_global_grid_positions,
 * mhd_data_parallel.f90:2087-2126, which gpat_read_grid_positions restates
 * on <dir>xpos.dat, ypos.dat, zpos.dat).  They replace the uniform
 * positions dx (i - 2) + xmin the handle starts with and are used by the
 * gradients (calc_fields_gradients_nonuniform :612-764 with idxh_grid
 * :2172-2189), the interpolation, the pushes' cell sizes, the boundary
 * extension, the large-quantity counts and the local distributions.  Set
 * them before gpat_calc_fields_gradients.  gpat_get_grid_positions copies
 * them out (spherical or non-uniform grids). */
int gpat_set_grid_positions(gpat_handle_t *h, const double *xpos, const double *ypos,
                            const double *zpos);
int gpat_read_grid_positions(gpat_handle_t *h, const char *dir_mhd_data);
int gpat_get_grid_positions(gpat_handle_t *h, double *xpos, double *ypos, double *zpos);
/* Surfaces separating the acceleration region of 3D runs (acc_by_surface;
 * init_acc_surface / read_acc_surface / interp_acc_surface /
 * check_above_acc_surface, acc_region_surface.f90:27-383).  norm1/norm2:
 * "+x" .. "-z", the normal axis and the side of the region ("+": above);
 * norm2 NULL for one surface; is_intersection: both conditions (1) or
 * either (0).  Heights are doubles over the ghost-padded plane normal to
 * the axis, (nyg, nzg), (nxg, nzg) or (nxg, nyg) with the first index
 * fastest, all 0 until set; var_flag 0 is frame 1, otherwise frame 2
 * (copied to frame 1 by gpat_copy_fields).  With acc_region_flag = 1 a
 * push then changes p only inside the box region and on the region's side
 * of the surfaces, interpolated at the push's start.  3D and
 * GPAT_PREC_FP64 only. */
int gpat_init_acc_surface(gpat_handle_t *h, const char *norm1, const char *norm2,
                          int is_intersection);
int gpat_set_acc_surface(gpat_handle_t *h, int var_flag, const double *surface1,
                         const double *surface2);
int gpat_read_acc_surface(gpat_handle_t *h, int var_flag, const char *filename1,
                          const char *filename2);
/* copy_fields (mhd_data_parallel.f90:1920-1926): farray1 = farray2. */
int gpat_copy_fields(gpat_handle_t *h);
/* Copies a device field array (32 vars per cell, Fortran order) to the host. */
int gpat_get_fields(gpat_handle_t *h, int var_flag, float *farray);

/* inject_particles_spatial_uniform + inject_one_particle
 * (particle_module.f90:385-530), one rank: part_box = {xmin, ymin, zmin,
 * xmax, ymax, zmax}; t = tstamps(ct_mhd) + U * (tstamps(ct_mhd+1) -
 * tstamps(ct_mhd)).  Adds min(nptl, nptl_max - nptl_current) particles and
 * returns GPAT_ERR_CAPACITY when it had to stop at the cap. */
int gpat_inject_particles_spatial_uniform(gpat_handle_t *h, int64_t nptl, double dt,
                                          int dist_flag, double particle_v0, int ct_mhd,
                                          const double part_box[6], double power_index);
/* Injection on the plane x = xpos at t = tstamps(ct_mhd), with the draw order
 * of inject_particles_at_shock (particle_module.f90:542-633).  It replaces
 * the reference's shock locator (interp_shock_location), whose weights use
 * dpy for both ry and rz (:580-581). */
int gpat_inject_particles_at_x(gpat_handle_t *h, int64_t nptl, double xpos, double dt,
                               int dist_flag, double particle_v0, int ct_mhd,
                               double power_index);

/* Quantities of inject_particles_at_large_jz / _absj / _divv / _rho / _db2
 * (particle_module.f90:785-1468). */
#define GPAT_LARGE_JZ 0    /* |dBy/dx - dBx/dy|                        */
#define GPAT_LARGE_ABSJ 1  /* |curl B|                                 */
#define GPAT_LARGE_DIVV 2  /* -div v (compression)                     */
#define GPAT_LARGE_RHO 3   /* rho                                      */
#define GPAT_LARGE_DB2 4   /* db2_slab (needs deltab_flag and its arrays) */
/* get_ncells_large_jz / _absj / _divv / _rho (mhd_data_parallel.f90:
 * 2211-2498): grid nodes of frame slot 0 strictly inside part_box whose
 * quantity is > qmin, evaluated in single precision from the stored
 * gradients as the reference does.  The divv count reads the node two
 * cells lower in x, y (and z in 3D): the reference assigns the whole
 * ghost-padded gradient array to a node-sized allocatable, which is
 * re-allocated with lower bound 1. */
/* locate_shock_xpos (mhd_data_parallel.f90:1988-2006) on frame 1: for each
 * row of the ghost-padded grid (nyg * nzg rows, y fastest) the first 1-based
 * x index of the largest |dvx/dx|; shock_ix may be NULL. */
int gpat_locate_shock_xpos(gpat_handle_t *h, int32_t *shock_ix);
/* inject_particles_at_shock (particle_module.f90:542-633): nptl particles
 * with y (and z) uniform over the box, at the shock of locate_shock_xpos
 * interpolated linearly between the rows either side, x = xmin + (index - 3)
 * dx, t = the frame's time stamp; momenta, mu and tags as
 * gpat_inject_particles_at_x.  The reference's interpolation weights, row
 * offset and index-to-x mapping are not usable as written (rz from dpy,
 * weights that do not sum to 1, uninitialised sums, frame 2 read at rt = 0);
 * this is the interpolation they describe.  Uniform Cartesian grids. */
int gpat_inject_particles_at_shock(gpat_handle_t *h, int64_t nptl, double dt, int dist_flag,
                                   double particle_v0, int ct_mhd, double power_index);
int gpat_count_cells_large(gpat_handle_t *h, int quantity, double qmin,
                           const double part_box[6], int64_t *ncells);
/* inject_particles_at_large_*: nptl_inject = nptl when inject_same_nptl
 * (one rank), else int(nptl * ncells / ncells_norm); each particle is
 * drawn uniformly over the box until it lies in part_box (inclusive) with
 * the interpolated quantity >= qmin, then mu, p and t as
 * inject_particles_spatial_uniform.  *ninjected receives nptl_inject. */
int gpat_inject_particles_at_large(gpat_handle_t *h, int quantity, int64_t nptl, double dt,
                                   int dist_flag, double particle_v0, int ct_mhd,
                                   int inject_same_nptl, double qmin, int64_t ncells_norm,
                                   const double part_box[6], double power_index,
                                   int64_t *ninjected);

/* Particle exchange with the host (e.g. restart files, the Fortran ptls
 * array).  put replaces the whole particle set and raises the injection
 * counter (tag_max) past the largest tag_injected it receives. */
int gpat_put_particles(gpat_handle_t *h, const gpat_particles_t *src, int64_t n);
int gpat_get_particles(gpat_handle_t *h, gpat_particles_t *dst, int64_t capacity,
                       int64_t *n);

/* particle_mover (particle_module.f90:1846-1974) on one rank:
 * mover cycle (:1481-1833), remove_particles, boundary pass on the exact
 * box, remove_particles.  focused_transport selects push_particle_*_ft
 * (mu and v become state; gpat_params_t.duu0 sets D_mumu), nlgc selects
 * calc_spatial_diffusion_coefficients_nlgc with kperp_kpara (both
 * precisions); focused transport needs GPAT_PREC_FP64.  mhd_tframe indexes
 * tstamps (t0 = tstamps(mhd_tframe)). */
int gpat_particle_mover(gpat_handle_t *h, int focused_transport, int nlgc,
                        double kperp_kpara, int nsteps_interval, int mhd_tframe,
                        int num_fine_steps, int dump_escaped_dist);
/* No counterpart in the reference, whose particles read field arrays in host
 * memory.  Selects how the split-precision mover (GPAT_PREC_MIXED, 2D and 3D)
 * of gpat_particle_mover reads the fields: bx = 0 gathers the packed field
 * records from device memory through the caches; bx > 0 cuts the grid into
 * bricks of bx x by x bz cells (bz, hz ignored in 2D), keeps the particle set
 * binned brick-major, and has each CTA copy the records of one brick plus a
 * halo of hx, hy, hz cells on every side into shared memory (TMA) and move
 * that brick's particles for a chunk of bin_interval pushes; a particle that
 * walks out of the staged region finishes its chunk with global gathers.
 * threads: per CTA, 256 or 512 (0: 512); items: particles a CTA takes per
 * brick visit (0: 4096).  The staged records ((sx+1)(sy+1)(sz+1) nodes,
 * s = b + 2h, x 64 or 96 bytes, twice with time_interp) must fit in one CTA's
 * shared memory (GPAT_ERR_ARG otherwise); a brick larger than the grid is cut
 * to it.  Both forms give the same trajectories to FP32 rounding (the same
 * increments for the same push; paused particles are rebuilt from their FP64
 * record at other pushes), not bit for bit. */
int gpat_set_mover_tiles(gpat_handle_t *h, int bx, int by, int bz, int hx, int hy, int hz,
                         int threads, int items);
/* out[8] = {bx, by, bz, hx, hy, hz, threads, items} as set (bx = 0: no bricks). */
int gpat_get_mover_tiles(const gpat_handle_t *h, int *out);
/* split_particle (particle_module.f90:5430-5480): children appended in
 * parent order; stops at nptl_max like the reference. */
int gpat_split_particle(gpat_handle_t *h, double split_ratio, double pmin_split,
                        int nsteps_interval);
/* No counterpart in the reference.  split_particle for callers that cannot
 * call cudaMalloc, e.g. a driver whose particle arrays already live in device
 * memory it manages itself (CUDA Fortran, OpenACC, an application memory
 * pool) and that may not allocate inside its time loop.  `dev` holds DEVICE
 * pointers to caller-owned arrays of `capacity` entries, the first n of which
 * are particles; children are appended after them as gpat_split_particle
 * does.  No handle, and no device memory is allocated or freed: the scan
 * scratch and counters are fixed file-scope device arrays (about 1 MiB on
 * every GPU that loads the library, held until exit), sized for at most
 * 2^26 = 67,108,864 parents; larger n returns GPAT_ERR_ARG.  The first call
 * on a device looks up those arrays' device addresses; with CUDA's lazy
 * module loading (the default) that first call also makes the driver load
 * the library's device code and reserve the arrays.  So make one warm-up
 * call with n = 0 (valid dev and n_out) on each device before the time loop
 * and before any stream capture.  All calls share the arrays, so calls whose
 * work overlaps on the GPU (other streams, other threads) race; serialise
 * them.  Particle tracking is not supported here: pass no tracked particles
 * (tag_splitted < 0); the handle's gpat_split_particle tracks them.
 * Work is enqueued on `stream` (a cudaStream_t, NULL for the default
 * stream), which is synchronised before return.  *n_out is the new particle
 * count, *n_split (may be NULL) the children created; GPAT_ERR_CAPACITY when
 * capacity stopped the splitting. */
int gpat_split_particle_noalloc(const gpat_particles_t *dev, int64_t n, int64_t capacity,
                                double split_ratio, double pmin_split, double p0, double pmax,
                                void *stream, int64_t *n_out, int64_t *n_split);
/* Global f(p) of calc_particle_distributions (diagnostics.f90:738-780):
 * fglobal[npp_global] weighted counts (may be NULL) and counts[npp_global]
 * particle numbers (may be NULL).  Bins are exact. */
int gpat_calc_particle_distributions(gpat_handle_t *h, double *fglobal, uint64_t *counts);
/* One set of local distribution parameters (conf.dat pmin1 pmax1 npbins1
 * nmu1 rx1 ry1 rz1 ..., read_diagnostics_params diagnostics.f90:2100-2200). */
typedef struct gpat_local_dist {
    double pmin, pmax;
    int32_t npbins, nmu, rx, ry, rz, reserved;
} gpat_local_dist_t;
/* Shape of flocal for a parameter set: {nmu, npbins, nrx, nry, nrz} with
 * nrx = (nx + rx - 1) / rx (init_local_particle_distributions :231-330). */
int gpat_local_distribution_dims(gpat_handle_t *h, const gpat_local_dist_t *spec, int32_t dims[5]);
/* A local distribution of calc_particle_distributions (diagnostics.f90:
 * 782-878): flocal(imu, ip, ix, iy, iz) in Fortran order (imu fastest),
 * ix = floor((x - xmin) / (lx / nrx)) + 1, and, as in the reference, only
 * 0 < ip < npbins (the last p bin stays empty).  Weighted sums are exact;
 * counts (may be NULL) are particle numbers. */
int gpat_calc_local_distribution(gpat_handle_t *h, const gpat_local_dist_t *spec, double *flocal,
                                 uint64_t *counts);
/* Global distribution of the particles removed through an open boundary
 * since the last reset (calc_escaped_distributions, diagnostics.f90:913-960):
 * fescaped(npp_global, 2 * ndim) in Fortran order, column ibc = |count_flag|
 * (1 low x, 2 high x, 3 low y, 4 high y, 5 low z, 6 high z). */
int gpat_calc_escaped_distributions(gpat_handle_t *h, double *fescaped, uint64_t *counts);
/* The global distribution with pitch-angle bins (calc_particle_distributions,
 * diagnostics.f90:773-779; nmu_global bins for focused transport):
 * fglobal(nmu, npp_global) in Fortran order over pmin < p <= pmax and
 * -1 <= mu <= 1, imu = floor((mu + 1) / dmu) + 1 with dmu = 2.0 / nmu in
 * single precision as the reference computes it; the particle's own weight. */
int gpat_calc_particle_distributions_mu(gpat_handle_t *h, int32_t nmu, double *fglobal,
                                        uint64_t *counts);
/* fescaped(nmu, npp_global, 2 * ndim) of calc_escaped_distributions
 * (:949-957) over the escaped particles kept by mover calls with
 * dump_escaped_dist = 1 since the last reset, column |count_flag|. */
int gpat_calc_escaped_distributions_mu(gpat_handle_t *h, int32_t nmu, double *fescaped,
                                       uint64_t *counts);
/* Local escaped distributions of one parameter set (calc_escaped_
 * distributions :958-1230) over the same escaped particles, binned like the
 * local distributions: fx(nmu, npbins, nry, nrz, 2) for the low / high x
 * faces, fy(nmu, npbins, nrx, nrz, 2) (ndim > 1), fz(nmu, npbins, nrx, nry,
 * 2) (ndim 3); Fortran order; a NULL pair skips a face. */
int gpat_calc_local_escaped_distribution(gpat_handle_t *h, const gpat_local_dist_t *spec,
                                         double *fx, double *fy, double *fz, uint64_t *cx,
                                         uint64_t *cy, uint64_t *cz);
/* escaped_ptls: the particles removed through an open boundary by
 * gpat_particle_mover calls made with dump_escaped_dist = 1 since the last
 * reset (remove_particles, particle_module.f90:5365-5403, as written by
 * dump_escaped_particles, diagnostics.f90:1896-1978), in removal order;
 * count_flag holds the boundary face (-1 .. -6).  *n gets their number;
 * GPAT_ERR_CAPACITY when it exceeds capacity. */
int gpat_get_escaped_particles(gpat_handle_t *h, gpat_particles_t *dst, int64_t capacity,
                               int64_t *n);
/* reset_escaped_particles: clears the escaped distribution and the escaped
 * particles. */
int gpat_reset_escaped_particles(gpat_handle_t *h);
/* Particle tracking (track_particle_flag, GPAT_PREC_FP64 only).
 * init_particle_tracking (particle_module.f90:5825-5877): tags is
 * tags_tracking(nrows, nptl_tracking) in Fortran order, column j = tracked
 * particle j: {origin, tag_injected, tag_splitted after 1 .. nrows - 2
 * splits}; particles_tracked(nsteps_tracking_max, nptl_tracking) is
 * allocated and zeroed, nsteps_tracking_max = ceiling((1 / dt_min_rel) /
 * nsteps_interval) + 1.  From then on, injection selects listed particles
 * (negated tags, first record; :434-440), gpat_particle_mover records a
 * tracked particle every nsteps_interval pushes (:1697-1722, :1806-1812) and
 * gpat_split_particle follows the tracking branch of split_particle
 * (:5452-5474).  Records past nsteps_tracking_max are dropped and counted.
 * A second call replaces the table and clears the records. */
int gpat_init_particle_tracking(gpat_handle_t *h, const int32_t *tags, int32_t nrows,
                                int32_t nptl_tracking, int32_t nsteps_interval);
/* The same from a raw file: int32 nrows, int32 nptl_tracking, then the
 * table in Fortran order (the "tags" dataset of the reference's tags file). */
int gpat_read_particle_tracking(gpat_handle_t *h, const char *particle_tags_file,
                                int32_t nsteps_interval);
/* nsteps_tracking_max, nptl_tracking and the dropped-record count (each
 * pointer may be NULL). */
int gpat_tracking_dims(gpat_handle_t *h, int64_t *nsteps_tracking_max, int32_t *nptl_tracking,
                       int64_t *dropped);
/* sync_tracked_particles + the data of dump_tracked_particles (:5994-6030,
 * :6235-6299) on one rank: each column keeps its records with
 * tag_splitted < 0, in order, the rest zeroed (this persists, as in the
 * reference); then every field (NULL: skipped) gets nsteps_tracking_max *
 * nptl_tracking values, particles_tracked(step, particle) in Fortran order. */
int gpat_get_tracked_particles(gpat_handle_t *h, gpat_particles_t *dst);
/* free_particle_tracking (:5905-5911). */
int gpat_free_particle_tracking(gpat_handle_t *h);
/* get_pmax_global (diagnostics.f90:1691-1721): the largest particle momentum
 * (0 without particles). */
int gpat_get_pmax_global(gpat_handle_t *h, double *pmax);
/* pbins_edges_global (diagnostics.f90:194-204): npp_global + 1 values. */
int gpat_pbins_edges(gpat_handle_t *h, double *edges);
/* quick_check (diagnostics.f90:116-170) for one rank: out = {nptl_current,
 * nptl_split, sum of weights, leak, leak_negp, pdt_min, pdt_max, pdt_avg}. */
int gpat_quick_check(gpat_handle_t *h, double out[8]);
int gpat_get_counters(gpat_handle_t *h, gpat_counters_t *out);
/* Restores module state after a restart (save/read_particle_module_state). */
int gpat_set_counters(gpat_handle_t *h, const gpat_counters_t *in);

/* The handle's CUDA stream (a cudaStream_t) for callers that time or
 * order work around the engine. */
void *gpat_stream(gpat_handle_t *h);

/* ------------------------------------------------------------------------ */
/* Batched runs.  No counterpart in the reference, whose independent runs    */
/* are separate jobs.  A batch groups up to 64 runs (handles on one device,  */
/* GPAT_PREC_MIXED, one ndim) so that their particle_mover calls become one   */
/* persistent launch per chunk of bin_interval pushes: blocks take           */
/* 128-particle tiles from one counter across all runs, then every run's     */
/* particles are binned by cell and removed, with the counts kept on the     */
/* device, and that chunk is replayed as a CUDA graph until no particle has  */
/* pushes left.  Each run's result is the one gpat_particle_mover gives on   */
/* that handle alone; while a call runs, the runs' handles must not be used. */
/* ------------------------------------------------------------------------ */
typedef struct gpat_batch gpat_batch_t;
/* Launch shape picked by gpat_batch_autotune: minb = resident 128-thread
 * blocks per SM of the kernel variant (its register target), grab = tiles a
 * block takes per scheduler step; pushes_per_s = the measured rate;
 * chunk_pushes = pushes per particle between re-binnings for every run (0:
 * each run's own bin_interval).  minb and grab do not change results;
 * chunk_pushes moves the pause points, so results agree statistically.
 * default_pushes_per_s: gpat_batch_autotune's measured rate of the untuned
 * launch (the single-run kernel's register target, one tile per grab, the
 * first run's own chunk length); 0 where not measured. */
typedef struct gpat_batch_tuning {
    int32_t minb, grab;
    double pushes_per_s;
    int32_t chunk_pushes, reserved;
    double default_pushes_per_s;
} gpat_batch_tuning_t;
int gpat_batch_create(gpat_handle_t *const *runs, int nruns, gpat_batch_t **out);
int gpat_batch_destroy(gpat_batch_t *b);
const char *gpat_batch_last_error(const gpat_batch_t *b);
/* particle_mover for every run; mhd_tframe holds one frame index per run. */
int gpat_batch_particle_mover(gpat_batch_t *b, const int *mhd_tframe, int nlgc,
                              double kperp_kpara, int nsteps_interval, int num_fine_steps);
/* Times one chunk of every candidate (register-target variant x tile grab x
 * chunk length 64 / 128 / 256) from a snapshot of the runs (restored
 * afterwards, so the runs are unchanged) and keeps the fastest for later
 * calls. */
int gpat_batch_autotune(gpat_batch_t *b, const int *mhd_tframe, int nlgc, double kperp_kpara,
                        int nsteps_interval, int num_fine_steps, gpat_batch_tuning_t *best);
int gpat_batch_get_tuning(const gpat_batch_t *b, gpat_batch_tuning_t *t);
int gpat_batch_set_tuning(gpat_batch_t *b, const gpat_batch_tuning_t *t);
/* Device time, pushes and graph launches of the last batched mover call. */
int gpat_batch_stats(const gpat_batch_t *b, double *ms, uint64_t *pushes, int64_t *graph_launches);

/* ------------------------------------------------------------------------ */
/* Learned splitting.  No counterpart in the reference (its split_particle   */
/* uses fixed momentum thresholds).  An MLP importance map -- inputs x, y, z */
/* (box-normalised), log10(p/p0), div v, |B|, |grad B| and normalised time,  */
/* 3 hidden layers of 64 SiLU units, BF16 weights with FP32 accumulation --  */
/* predicts the log-odds that a particle's future momentum exceeds a        */
/* threshold.  It is trained on the GPU (hand-written forward, backward and */
/* Adam kernels) from records of plain runs, and drives weighted splitting  */
/* and Russian roulette with a weight window; both keep the expected weight. */
/* ------------------------------------------------------------------------ */
#define GPAT_MLP_FEATURES 8
#define GPAT_MLP_PARAMS 8961   /* W1[64][8] b1 W2[64][64] b2 W3[64][64] b3 W4[64] b4 */
typedef struct gpat_mlp gpat_mlp_t;
/* record_capacity: training records kept on the device (0: inference only). */
int gpat_mlp_create(int device, uint64_t seed, int64_t record_capacity, gpat_mlp_t **out);
int gpat_mlp_destroy(gpat_mlp_t *m);
const char *gpat_mlp_last_error(const gpat_mlp_t *m);
/* FP32 master parameters (GPAT_MLP_PARAMS) and the feature standardisation
 * norm = {mean[8], 1/std[8]}; either may be NULL. */
int gpat_mlp_set_params(gpat_mlp_t *m, const float *params, const float *norm);
int gpat_mlp_get_params(gpat_mlp_t *m, float *params, float *norm);
/* Output (log-odds) for n host feature rows. */
int gpat_mlp_forward(gpat_mlp_t *m, const float *x, int64_t n, float *z);
/* Mean binary cross-entropy of n host rows with labels y, and its gradient
 * with respect to the parameters (the BF16-rounded weights' gradient). */
int gpat_mlp_loss_grad(gpat_mlp_t *m, const float *x, const float *y, int64_t n, float *loss,
                       float *grad);
/* Training records: gpat_mlp_record appends the features (time t_norm) and
 * injection tag of every live particle of a run; gpat_mlp_label labels each
 * record 1 when its particle's momentum at the run's current state exceeds
 * p_threshold (plain runs: one particle per tag). */
int gpat_mlp_clear_records(gpat_mlp_t *m);
/* Replaces the records with n host rows of features and labels. */
int gpat_mlp_set_records(gpat_mlp_t *m, const float *x, const float *labels, int64_t n);
int gpat_mlp_record(gpat_mlp_t *m, gpat_handle_t *h, double t_norm, int64_t *nrec);
int gpat_mlp_label(gpat_mlp_t *m, gpat_handle_t *h, double p_threshold, int64_t *npos,
                   int64_t *nrec);
/* Adam on all positives and a neg_keep fraction of negatives (the output
 * bias is corrected by log(neg_keep) afterwards). */
int gpat_mlp_train(gpat_mlp_t *m, int epochs, int64_t batch, double lr, double neg_keep,
                   uint64_t seed, double *final_loss);
/* Over a run's live particles at time t_norm: the mean output,
 * L = log(sum_i w_i exp(z_i)) and log(sum_i w_i).  Defensive importance
 * (a fraction alpha of the weighted mean importance added to every
 * particle's): z_floor = log(alpha) + L - log(sum w) and
 * z_ref = L + log(1 + alpha) - log(N); with w_ref = 1 gpat_weighted_split
 * then aims the population at N particles (sum_i w_i / w_t,i = N) and no
 * roulette survivor weighs more than about (1 + alpha) / alpha times the
 * mean weight per target particle. */
int gpat_mlp_score(gpat_mlp_t *m, gpat_handle_t *h, double t_norm, double *mean_z,
                   double *log_sum_wexpz, double *log_sum_w);
/* Weighted split / roulette of a run's particles: floored log-importance
 * z' = log(exp(z) + exp(z_floor)) (z_floor = -INFINITY: none), target
 * weight w_t = w_ref exp(z_ref - z'), window [w_t / sqrt(window_ratio),
 * w_t sqrt(window_ratio)]; above it a particle splits into 2^j copies
 * (j <= max_level, children appended up to nptl_max), below it survives
 * with probability w / w_t at weight w_t (roulette draws are Philox,
 * keyed by the particle's tags and push counter).  Both keep the expected
 * weight of every particle.  Copies split past the 30 binary levels of the
 * int32 tag take tag_splitted = -id from a per-handle counter (ids past the
 * most negative tag a gpat_put_particles set holds). */
int gpat_weighted_split(gpat_handle_t *h, gpat_mlp_t *m, double t_norm, double w_ref, double z_ref,
                        double z_floor, double window_ratio, int max_level, int64_t *nsplit,
                        int64_t *nkilled);
/* No counterpart in the reference.  Learned splitting inside the mover:
 * while set, gpat_particle_mover's split-precision chunk launches score every
 * particle that finishes the interval in the box with the network m (tensor
 * cores, in the same launch) at features of normalised time t_norm, and apply
 * gpat_weighted_split's weight window (same z_ref, z_floor, window_ratio,
 * max_level): children are appended after the set (up to nptl_max), roulette
 * losers are removed.  The brick mover is not used while this is set.
 * m = NULL turns it off.  The network must outlive the setting. */
int gpat_set_mover_learned(gpat_handle_t *h, gpat_mlp_t *m, double t_norm, double w_ref,
                           double z_ref, double z_floor, double window_ratio, int max_level);
/* After a mover call with learned splitting, over the judged particles
 * (before their split): log of the sum of w exp(z) and log of the sum of w
 * (the next call's z_ref and z_floor follow from them as for
 * gpat_mlp_score's), their number, children created and particles removed
 * by roulette. */
int gpat_get_mover_learned(const gpat_handle_t *h, double *log_sum_wexpz, double *log_sum_w,
                           int64_t *judged, int64_t *nsplit, int64_t *nkilled);
/* Count, sum of weights and of squared weights of live particles with
 * p > p_threshold: (sum w)^2 / sum w^2 is their effective sample size. */
int gpat_tail_weights(gpat_handle_t *h, double p_threshold, int64_t *count, double *wsum,
                      double *w2sum);

#ifdef __cplusplus
}
#endif
#endif
