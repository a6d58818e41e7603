/*
 * gpat_oracle.h -- CPU oracle for the GPAT Parker-transport particle mover.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference's CPU algorithm (xiaocanli/stochastic-parker, Fortran), used as
 * the checker for the CUDA engine and as the timed CPU baseline.  Nothing in
 * the product links or calls it; only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it.
 *
 * Parity status: UNPINNED by the reference's own tests.  The reference ships
 * no tests, golden vectors or fixtures, and it cannot be built here (Fortran +
 * MPI + HDF5 + FLAP + mt_stream; no gfortran).  The restatement is pinned
 * instead by analytic known answers (drift-only advection, pure-diffusion
 * variance, DSA spectral index) in tests/test_oracle_*.py and by the golden
 * vectors it generated (tests/golden/make_golden.py).
 *
 * Arithmetic follows the Fortran evaluation order of each cited routine,
 * left to right, with single-precision literals (0.1, 1.0/(3*charge)) kept
 * single, and is compiled with -ffp-contract=off so every +,-,*,/,sqrt is one
 * IEEE-rounded operation.  pow/log10/exp come from the host libm.
 *
 * The reference's MT19937 streams are replaced by Philox-4x32-10 (Salmon et
 * al., SC'11) keyed per particle, so results do not depend on the thread
 * count or schedule.
 */
#ifndef GPAT_ORACLE_H
#define GPAT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* mhd_configuration record, same field order and binary layout as the
 * reference's mhd_config.dat (src/modules/mhd_config.f90:16-27). */
typedef struct orc_mhd_config {
    double dx, dy, dz, xmin, ymin, zmin, xmax, ymax, zmax, lx, ly, lz, dt_out;
    int32_t nx, ny, nz, nxs, nys, nzs, topox, topoy, topoz, nvar, bcx, bcy, bcz;
} orc_mhd_config;

/* Parameters on the path: conf.dat keys read by read_particle_params
 * (particle_module.f90:2778-2878), the drift / flag setters (:269-328) and
 * the boundary flags (simulation_setup.f90:104-150). */
typedef struct orc_params {
    double b0, p0, pmin, pmax;
    double gamma_turb, pindex, kpara0, kret, dt_min_rel, dt_max_rel;
    double acc_region[6];
    double drift1, drift2;
    int32_t momentum_dependency, mag_dependency, acc_region_flag, charge;
    int32_t check_drift_2d, ndim, pbcx, pbcy, pbcz, npp_global;
    uint64_t seed;
    int32_t noise;      /* 0: (2u-1)*sqrt(3) as the reference; 1: Gaussian */
    int32_t focused_transport;  /* particle_mover's focused_transport          */
    int32_t nlgc;               /* particle_mover's nlgc                       */
    int32_t dpp_wave;           /* set_dpp_params (:255-272)                   */
    double duu0;                /* set_duu_params (:279-283)                   */
    double kperp_kpara;         /* particle_mover's kperp_kpara                */
    int32_t dpp_shear, weak_scattering;
    double tau0;
    int32_t deltab_flag, correlation_flag;   /* set_flags_params (:285-300) */
    /* set_mhd_grid_type (mhd_config.f90:179-186); with either set, the node
     * positions come from orc_set_grid_positions. */
    int32_t spherical_coord, nonuniform_grid;
    /* set_flags_params' include_3rd_dim (:294-306): a 2D run whose
     * particles also move along z, pushed by push_particle_2d_include_3rd
     * (_ft) (:3979-4610) */
    int32_t include_3rd_dim;
} orc_params;

/* particle_type (particle_module.f90:38-50) as structure-of-arrays, plus the
 * per-particle Philox push counter that replaces the MT19937 state. */
typedef struct orc_particles {
    double *x, *y, *z, *p, *v, *mu, *weight, *t, *dt;
    int8_t *split_times, *count_flag;
    int32_t *origin, *nsteps_tracked, *nsteps_pushed, *tag_injected, *tag_splitted;
    uint32_t *rng_ctr;
} orc_particles;

/* Module-level counters (particle_module.f90:65-79).  leak and leak_negp are
 * kept as unsigned 128-bit fixed point with 64 fraction bits so the sums are
 * exact for dyadic weights and independent of summation order. */
typedef struct orc_counters {
    uint64_t leak_hi, leak_lo, leak_negp_hi, leak_negp_lo;
    uint64_t steps;          /* pushes, landing redo pushes included */
    int64_t nptl_escaped;    /* removed with count_flag < 0 */
    int64_t nptl_split;
    int64_t tag_max;
} orc_counters;

#define ORC_COUNT_FLAG_INBOX 1
#define ORC_COUNT_FLAG_OTHERS 0

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double orc_u01(uint32_t a, uint32_t b);
void orc_fixed_add(uint64_t *hi, uint64_t *lo, double w);
double orc_fixed_to_double(uint64_t hi, uint64_t lo);

void orc_calc_fields_gradients(float *farray, int ndim, int nxg, int nyg, int nzg,
                               double dx, double dy, double dz);

/* Node positions of the ghost-padded grid (xpos_global on one rank,
 * mhd_data_parallel.f90:2051-2190): nxg x positions, nyg y positions (2D and
 * 3D) and nzg z positions (3D); y and z may be NULL in fewer dimensions.
 * The oracle keeps copies; they serve every routine below while
 * spherical_coord or nonuniform_grid is set. */
void orc_set_grid_positions(const double *xpos, const double *ypos, const double *zpos,
                            int nxg, int nyg, int nzg);
/* calc_global_grid_positions (:2131-2148): pos[j] = d * (j - 2) + xmin. */
void orc_uniform_grid_positions(int n, double d, double xmin, double *pos);
/* binarySearch_R (particle_module.f90:680-698): the 1-based index of the
 * last node <= v, i.e. the number of nodes <= v. */
int orc_binary_search(const double *a, int n, double v);
/* calc_fields_gradients_nonuniform (mhd_data_parallel.f90:612-764) and the
 * fluctuation-record variants (:880-1008 and siblings) with the inverse
 * spans idxh_grid of set_local_grid_positions (:2153-2190). */
void orc_calc_fields_gradients_nonuniform(float *farray, int ndim, int nxg, int nyg, int nzg);
void orc_calc_aux_gradients_nonuniform(float *aux, int ndim, int nxg, int nyg, int nzg);
/* Interpolation corner (pos, Fortran convention as orc_get_interp_paramters)
 * and weights for a position under the grid type of pr:
 * get_interp_paramters_spherical (particle_module.f90:705-775) in spherical
 * coordinates; on a non-uniform Cartesian grid the cell found by
 * binarySearch_R with the fractional offset of :1620-1625. */
void orc_grid_interp_paramters(const orc_params *pr, const orc_mhd_config *cfg, double x,
                               double y, double z, int32_t pos[3], double weights[8]);
void orc_get_interp_paramters(int ndim, double px, double py, double pz,
                              int32_t pos[3], double weights[8]);
void orc_interp_fields(const float *f1, const float *f2, int time_interp, int ndim,
                       int nxg, int nyg, const int32_t pos[3], const double weights[8],
                       double rt, double fields[32]);
void orc_calc_spatial_diffusion_coefficients(const orc_params *pr, double p, double mu,
                                             const double fields[32], const double *aux,
                                             double kappa[22]);
void orc_calc_aux_gradients(float *aux, int ndim, int nxg, int nyg, int nzg,
                            double dx, double dy, double dz);
void orc_interp_aux(const float *a1, const float *a2, int time_interp, int ndim, int nxg,
                    int nyg, const int32_t pos[3], const double w[8], double rt, double out[16]);

/* aux1 / aux2: 16-float fluctuation records of the two frames, or NULL
 * (read when deltab_flag / correlation_flag are on). */
int64_t orc_particle_mover(const orc_params *pr, const orc_mhd_config *cfg,
                           const float *f1, const float *f2, const float *aux1,
                           const float *aux2, int time_interp,
                           orc_particles *ptl, int64_t n, double t0, double dtf,
                           int nsteps_interval, int num_fine_steps, int nthreads,
                           orc_counters *cnt);
int64_t orc_remove_particles(orc_particles *ptl, int64_t n, orc_counters *cnt);
int64_t orc_split_particle(const orc_params *pr, orc_particles *ptl, int64_t n,
                           int64_t nptl_max, double split_ratio, double pmin_split,
                           orc_counters *cnt);
void orc_pbins_edges(const orc_params *pr, double *edges);
void orc_calc_particle_distributions(const orc_params *pr, const orc_particles *ptl,
                                     int64_t n, uint64_t *counts, uint64_t *whi,
                                     uint64_t *wlo, double *fglobal);
int64_t orc_inject_spatial_uniform(const orc_params *pr, orc_particles *ptl, int64_t n,
                                   int64_t nptl_max, int64_t nptl, double dt,
                                   int dist_flag, double particle_v0, double t_frame,
                                   double dt_mhd, const double part_box[6],
                                   double power_index, orc_counters *cnt);
/* get_ncells_large_* and inject_particles_at_large_* (quantity 0 jz,
 * 1 absj, 2 divv, 3 rho, 4 db2); full is frame 1 with gradients, aux its
 * fluctuation records (quantity 4 only). */
int64_t orc_count_cells_large(const orc_params *pr, const orc_mhd_config *cfg, const float *full,
                              const float *aux, int quantity, double qmin,
                              const double part_box[6]);
int64_t orc_inject_at_large(const orc_params *pr, const orc_mhd_config *cfg, const float *full,
                            const float *aux, orc_particles *ptl, int64_t n, int64_t nptl_max,
                            int64_t nptl,
                            double dt, int dist_flag, double particle_v0, double t_frame,
                            double dt_mhd, int quantity, double qmin,
                            const double part_box[6], double power_index, orc_counters *cnt);
void orc_locate_shock_xpos(const float *full, int nxg, int nyg, int nzg, int32_t *S);
int64_t orc_inject_at_shock(const orc_params *pr, const orc_mhd_config *cfg, const int32_t *S,
                            int nyg, int nzg, orc_particles *ptl, int64_t n, int64_t nptl_max,
                            int64_t nptl, double dt, int dist_flag, double particle_v0,
                            double t_frame, double power_index, orc_counters *cnt);
int64_t orc_inject_at_x(const orc_params *pr, const orc_mhd_config *cfg,
                        orc_particles *ptl, int64_t n, int64_t nptl_max,
                        int64_t nptl, double xpos, double dt, int dist_flag,
                        double particle_v0, double t_frame, double power_index,
                        orc_counters *cnt);
void orc_quick_check(const orc_particles *ptl, int64_t n, double out[4]);
/* Attaches a store for the escaped particles remove_particles drops
 * (escaped_ptls); store NULL detaches it. */
void orc_set_escaped_store(orc_particles *store, int64_t cap, int64_t *n);
void orc_set_escaped_histogram(int npp, double pmin, double pmax, uint64_t *counts,
                               uint64_t *whi, uint64_t *wlo);
/* init_acc_surface / read_acc_surface for 3D runs
 * (acc_region_surface.f90:27-249): surface k has normal axis axisk
 * (0 x, 1 y, 2 z) and sign +1 when the acceleration region lies above it;
 * arrays are ghost-padded (nyg, nzg), (nxg, nzg) or (nxg, nyg), the first
 * index fastest, for frame 1 (s11, s21) and frame 2 (s12, s22, NULL: the
 * same).  s11 NULL turns the surfaces off. */
void orc_set_acc_surface(int axis1, int sign1, int axis2, int sign2, int has2, int intersection,
                         const double *s11, const double *s12, const double *s21,
                         const double *s22, int nxg, int nyg, int nzg);
/* Particle tracking (init_particle_tracking): tags_tracking(nrows, n) and
 * the records particles_tracked(nsteps_max, n), Fortran order, owned by the
 * caller; tags NULL turns tracking off.  With tracking on, injection, the
 * mover and split_particle select and record as the reference does. */
void orc_set_tracking(const int32_t *tags, int nrows, int n, int64_t nsteps_max,
                      const orc_particles *rec);
int64_t orc_tracking_dropped(void);
int64_t orc_nsteps_tracking_max(double dt_min_rel, int nsteps_interval);
/* sync_tracked_particles on one rank. */
void orc_sync_tracked(void);
void orc_calc_local_escaped_distribution(const orc_mhd_config *cfg, int ndim, int spherical,
                                         int nonuniform, double pmin, double pmax, int npbins,
                                         int nmu, int rx, int ry, int rz,
                                         const orc_particles *ptl, int64_t n,
                                         uint64_t *cx, uint64_t *hx, uint64_t *lx,
                                         uint64_t *cy, uint64_t *hy, uint64_t *ly,
                                         uint64_t *cz, uint64_t *hz, uint64_t *lz);
void orc_calc_distribution_mu(const orc_params *pr, const orc_particles *ptl, int64_t n, int nmu,
                              int by_face, int nfaces, uint64_t *counts, uint64_t *whi,
                              uint64_t *wlo);
void orc_calc_local_distribution(const orc_mhd_config *cfg, int ndim, int spherical,
                                 int nonuniform, double pmin, double pmax,
                                 int npbins, int nmu, int rx, int ry, int rz,
                                 const orc_particles *ptl, int64_t n, uint64_t *counts,
                                 uint64_t *whi, uint64_t *wlo, double *flocal);

#ifdef __cplusplus
}
#endif
#endif
