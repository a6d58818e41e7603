// Internal declarations shared by the engine's host code and CUDA kernels.
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "gpat_engine.h"

namespace gpat {

// Device status word bits (DevCounters::status).  Kernels never trap: they
// record the condition, skip the access and let the host turn it into
// GPAT_ERR_DEVICE.
enum : unsigned int {
    kStatusIndexGuard = 1u,   // interpolation cell outside the ghost range
    kStatusNonFinite = 2u,    // NaN/Inf position, momentum or time
    kStatusStepLimit = 4u,    // per-interval push limit reached
    kStatusTileTimeout = 8u,  // a brick copy into shared memory did not complete in time
    kStatusTileMiss = 16u,    // a particle outside the staged region of the brick it is binned in
};

// particle_type as SoA device arrays (capacity entries each).
struct DevParticles {
    double *x, *y, *z, *p, *v, *mu, *weight, *t, *dt;
    int8_t *split_times, *count_flag;
    int32_t *origin, *nsteps_tracked, *nsteps_pushed, *tag_injected, *tag_splitted;
    uint32_t *rng_ctr;
};

// Device-side accumulators.  Fixed-point sums are 128-bit (hi, lo) with 64
// fraction bits.
struct DevCounters {
    unsigned long long leak_hi, leak_lo, negp_hi, negp_lo;
    unsigned long long steps;
    unsigned long long nescaped;
    unsigned long long nkept;
    unsigned long long nsplit;
    unsigned long long wsum_hi, wsum_lo, dtsum_hi, dtsum_lo;
    unsigned long long nactive;   // particles a chunked mover launch left mid-interval
    unsigned long long ncells;    // get_ncells_large_* result
    unsigned long long nkilled;   // particles removed by roulette
    unsigned long long nselected; // escaped particles copied by launch_select_escaped
    double dt_min, dt_max;
    unsigned int status;
    unsigned int pad;
    unsigned long long bad_value;
    unsigned long long trk_dropped;  // tracked records past nsteps_tracking_max
    unsigned long long pmax_bits;    // get_pmax_global: bits of the largest p >= 0
};

// Packed per-cell field records read by the movers.  2D: 16 floats,
// 3D: 24 floats (see fields.cu for the slot order).
constexpr int kRec2D = 16;
constexpr int kRec3D = 24;

// Particle tracking (track_particle_flag, particle_module.f90:144-150):
// tags_tracking(nrows, n) and particles_tracked(nsteps_max, n), both in
// Fortran order (column j of the table is tracked particle j).  tags ==
// nullptr: tracking off.
struct TrackArgs {
    const int32_t *tags;
    int nrows, n;            // split_times_max + 2, nptl_tracking
    int64_t nsteps_max;      // nsteps_tracking_max
    DevParticles rec;
};

// Everything the mover kernels need, passed by value.
struct MoverArgs {
    DevParticles P;
    int64_t n;
    const float *rec1, *rec2;  // packed records, frame 1 and frame 2
    int time_interp, ndim, nxg, nyg, nzg;
    int nsteps_interval, num_fine_steps;
    double dx, dy, dz, idx, idy, idz;
    double xmin, ymin, zmin, xmax, ymax, zmax;          // exact box
    double xmin1, xmax1, ymin1, ymax1, zmin1, zmax1;    // half-cell extended
    double cfg_xmin, cfg_ymin, cfg_zmin, cfg_lx, cfg_ly, cfg_lz;
    double dt_min, dt_max, t0, dtf, dt_fine, limit;
    double p0, pindex, gamma_turb, kpara0, kret, drift1, drift2;
    double acc_region[6];
    int charge, momentum_dependency, mag_dependency, acc_region_flag;
    int check_drift_2d, pbcx, pbcy, pbcz, noise;
    uint32_t key0, key1;
    uint32_t max_pushes;        // per particle per call, guards runaway loops
    uint8_t *pause;             // split-precision chunk launches: paused (1) / finished (0) per index
    uint32_t chunk_pushes;      // split-precision mover: stop a particle after this many
                                // pushes (between pushes) so the set can be re-binned; 0 = off
    // particle_mover's focused_transport / nlgc / kperp_kpara and duu0.
    // Focused transport interpolates all 32 variables from full1/full2.
    int focused_transport, nlgc;
    double kperp_kpara, duu0;
    // Momentum diffusion (set_dpp_params); the FP64 mover then reads the full
    // 32-variable records too.
    int dpp_wave, dpp_shear, weak_scattering;
    double tau0;
    // Spatially dependent turbulence (set_flags_params): fluctuation records
    // of both frames, read by the FP64 mover when a flag is on.
    int deltab_flag, correlation_flag;
    const float *aux1, *aux2;
    const float *full1, *full2;
    // Grid type (set_mhd_grid_type): spherical coordinates (x = r,
    // y = theta, z = phi) and/or non-uniform node positions; the node
    // positions (ghost nodes included) are read by the FP64 mover whenever
    // either is set.
    int spherical, nonuniform;
    const double *xpos, *ypos, *zpos;
    int include_3rd;   // 2D run with transport along z (FP64 mover)
    // Acceleration-region surfaces of 3D runs (acc_by_surface): heights over
    // the plane normal to surf_axis[k] (0 x, 1 y, 2 z), ghost-padded with
    // leading dimension surf_ld[k], for frame 1 and frame 2; surf_sign[k]
    // +1 when the region lies above surface k.
    int surf_on, surf_has2, surf_inter;
    int surf_axis[2], surf_sign[2], surf_ld[2];
    const double *surf[2][2];   // [surface][frame]
    TrackArgs trk;              // FP64 mover only
    DevCounters *cnt;
};

// Single-precision constants of the split-precision mover, derived on the
// host once per call so they live in the kernel's parameter space rather
// than in registers.  Positions are measured in cells from the box minimum.
struct MixedConsts {
    float idx, idy, idz;               // 1 / cell size
    float dxf, dyf, dzf;               // cell sizes
    int nx, ny, nz;                    // cells in the exact box
    float dt_min, dt_max, dtf, inv_dtf;
    float ip0, pindex, gm2, kpara0, kret;
    float kperp0, gm2_3, pindex_perp;  // NLGC: kpara0 kperp_kpara, (gamma-2)/3, (5-gamma)/3
    float vdq;                         // single-precision 1 / (3 charge)
    float d1p0, d2p0sq;                // drift1 p0, drift2 p0^2
    float pfloor;                      // 0.25 p0
    float acc[6];                      // acceleration region, box fractions
    float acc_off[3], acc_scale[3];    // cell -> box fraction: (c + off) * scale
};

// What the split-precision mover reads besides MixedConsts and the particle
// arrays: the part of MoverArgs used on the device, small enough that a
// table of kMaxBatchRuns runs fits in constant memory.
struct MixedRunArgs {
    const float *rec1, *rec2;
    DevCounters *cnt;
    double dx, dy, dz, xmin, ymin, zmin, t0, dtf, dt_fine, limit;
    int nxg, nyg, nzg, time_interp, nsteps_interval, acc_region_flag, mag_dependency;
    int momentum_dependency, check_drift_2d, pbcx, pbcy, pbcz, noise;
    uint32_t key0, key1, max_pushes, chunk_pushes;
    // Chunked launches: one byte per particle index set to 1 when the particle
    // paused with pushes left in the interval, 0 when it finished (null: not
    // recorded).  The next binning moves finished particles out of the way.
    uint8_t *pause;
};

// One run of a batched launch: its arguments, constants and both particle
// buffers (the launch's parity picks the source).
constexpr int kMaxBatchRuns = 64;
struct BatchRun {
    MixedRunArgs a;
    MixedConsts k;
    DevParticles P[2];
};

// Learned splitting (learned.cu).
constexpr int kMlpFeatures = 8;
constexpr int kMlpHidden = 64;
constexpr int kMlpParams = kMlpHidden * kMlpFeatures + kMlpHidden + 2 * (kMlpHidden * kMlpHidden +
                                                                          kMlpHidden) +
                           kMlpHidden + 1;
// Particle features: interpolation from the packed records plus the box.
struct FeatureArgs {
    const float *rec;
    double xmin, ymin, zmin, idx, idy, idz, ilx, ily, ilz, ip0;
    int nxg, nyg, nzg;
    float t_norm;
};
// Importance exp(z') with z' = log(exp(z) + exp(z_floor)): the floor (a
// fraction of the weighted mean importance, -inf for none) bounds the
// weights roulette can create.
struct WSplitArgs {
    double w_ref, z_ref, z_floor, sqrt_ratio;
    int max_level;
    uint32_t key0, key1;
    // lineage ids handed to copies split past the int32 tag's 30 binary
    // levels (their tag_splitted is minus the id); null: no split there
    unsigned long long *fresh;
};
// Learned splitting inside the split-precision mover: particles that finish
// the interval in the box are scored by the network and split or played
// roulette in the same launch.
struct FusedLearn {
    const __nv_bfloat16 *w16;
    const float *norm;
    FeatureArgs f;
    WSplitArgs s;
    int64_t cap;
    unsigned long long *count;   // particles including children (starts at the launch's total)
    unsigned long long *zsum;    // {judged, sum of w exp(z - z_shift) as hi, lo, sum of w as hi, lo}
    double z_shift;
};
// Per-minibatch activations ([64][b] except h0: [b][8]) and output deltas.
struct MlpTrainBuffers {
    float *h0, *a1, *a2, *a3, *h1, *h2, *h3, *dz;
};

// Launchers (defined in the .cu files).  All enqueue on `s`.
cudaError_t launch_scatter_raw_fields(const float *raw, int nvar, float *full, size_t ncells,
                                      cudaStream_t s);
// ih: per-axis inverse spans of a non-uniform grid (3 device pointers), or
// null for the uniform 0.5 / d.
cudaError_t launch_calc_fields_gradients(float *full, int ndim, int nxg, int nyg, int nzg,
                                         double dx, double dy, double dz, cudaStream_t s,
                                         const double *const *ih = nullptr);
cudaError_t launch_pack_records(const float *full, float *rec, int ndim, size_t ncells,
                                cudaStream_t s);
// Chunk-planar copy of packed records (R / 4 planes of float4, one per
// 16-byte chunk of the record) for the tile mover.
cudaError_t launch_planarize_records(const float *rec, float *planes, int ndim, size_t ncells,
                                     cudaStream_t s);
// Fluctuation records: 16 floats per node, {db2_slab, db2_2d, lc_slab,
// lc_2d} x {value, d/dx, d/dy, d/dz}.
cudaError_t launch_calc_aux_gradients(float *aux, int ndim, int nxg, int nyg, int nzg, double dx,
                                      double dy, double dz, cudaStream_t s,
                                      const double *const *ih = nullptr);
cudaError_t launch_scatter_aux(const float *src, float *aux, int comp, size_t ncells,
                               cudaStream_t s);
cudaError_t launch_fill(float *a, float v, size_t n, cudaStream_t s);
cudaError_t launch_mover_fp64(const MoverArgs &a, int sm_count, cudaStream_t s);
cudaError_t launch_mover_mixed(const MoverArgs &a, const MixedConsts &c, int sm_count,
                               cudaStream_t s);
MixedConsts make_mixed_consts(const MoverArgs &a);
// The global-gather chunk launch with learned splitting of finished particles.
cudaError_t launch_mover_learned(const MoverArgs &a, const MixedConsts &c, const FusedLearn &L,
                                 cudaStream_t s);
MixedRunArgs mixed_run_args(const MoverArgs &a);
// Batched split-precision mover (see mover_mixed.cu).
cudaError_t upload_batch_runs(const BatchRun *runs, int nruns, cudaStream_t s);
cudaError_t launch_batch_prefix(int nruns, const unsigned long long *run_n, long long *tile_prefix,
                                unsigned long long *tile_counter,
                                unsigned long long *nactive_total, cudaStream_t s);
int batch_minb_variants(int ndim, int *out);
// launch_cell_sort with the particle count in device memory (*n_dev, updated
// to the kept count), grids sized by the capacity: capturable in a graph.
struct CellGrid;
struct EscHist;
cudaError_t launch_cell_sort_dev(const DevParticles &src, const DevParticles &dst,
                                 unsigned long long *n_dev, int64_t cap, const CellGrid &g,
                                 void *scratch, DevCounters *cnt, const EscHist &esc,
                                 cudaStream_t s);
cudaError_t launch_mover_mixed_batch(int ndim, bool nlgc, int minb, int parity, int nruns,
                                     int sm_count, int grab, const long long *tile_prefix,
                                     const unsigned long long *run_n,
                                     unsigned long long *tile_counter,
                                     unsigned long long *nactive_total, cudaStream_t s);

// Split-precision mover with bricks of field records staged in shared memory
// (mover_tile.cu).  The particle set must be binned brick-major with the same
// brick shape (CellGrid::tile); incl is the sort's per-bin inclusive prefix.
struct TileSched {
    int bx, by, bz;                  // cells per brick and axis (bz = 1 in 2D)
    int hx, hy, hz;                  // halo: staged cells beyond the brick on each side
    int nbx, nby, nbz;               // bricks per axis
    long long nbricks;
    int cpb;                         // cells per brick
    int items;                       // particles per work item at most
    const unsigned int *incl;
    const long long *item_prefix;    // nbricks + 1 entries, written by the launch
    unsigned long long *item_counter;
    uint32_t tile_bytes;             // one frame's staged records
    uint32_t tile2_off;              // frame 2's staged records, in float4 from the start
    uint32_t nodes;                  // staged nodes: one chunk plane, in float4
    // Particles that left the staged region mid-chunk: their indices and the
    // pushes they had made, finished by the global-gather overflow kernel.
    long long *ovf_idx;
    unsigned int *ovf_done;
    unsigned long long *ovf_count;
};
// Dynamic shared memory of one CTA for a staged region of (s + 1) nodes per
// axis, s = brick cells + 2 halo cells, and the layout values TileSched needs.
size_t tile_smem_bytes(int ndim, int sx, int sy, int sz, int time_interp, uint32_t *tile_bytes,
                       uint32_t *tile2_off);
// TMA tensor map over a frame's chunk-planar records (launch_planarize_records)
// with a {4, sx+1, sy+1(, sz+1), R/4} box: every chunk plane of the staged
// region in one copy.
cudaError_t encode_brick_map(CUtensorMap *m, const float *planes, int ndim, int nxg, int nyg,
                             int nzg, int sx, int sy, int sz);
// Work items of the current binning, one persistent tile mover launch
// (threads per CTA: 256 or 512), then the overflow kernel (its count is
// zeroed by the caller before).
cudaError_t launch_mover_tile(const MoverArgs &a, const MixedConsts &c, const TileSched &s,
                              const CUtensorMap &tm1, const CUtensorMap &tm2, int threads,
                              int sm_count, cudaStream_t st);

// Quantities of inject_particles_at_large_* (GPAT_LARGE_*).
struct LargeArgs {
    int quantity;          // GPAT_LARGE_JZ / ABSJ / DIVV / RHO
    double qmin;
    double dom[6];         // sampling domain (the exact box): xmin ymin zmin xmax ymax zmax
    const float *full;     // frame 1, 32 variables per node (ghost layout)
    const float *aux;      // frame 1 fluctuation records (GPAT_LARGE_DB2), or null
    int nx, ny, nz, nxg, nyg;
    double dx, dy, dz, gxmin, gymin, gzmin;
    int spherical, nonuniform;              // grid type, as MoverArgs
    const double *xpos, *ypos, *zpos;       // node positions when either is set
    int nzg;
};

struct InjectArgs {
    DevParticles P;
    int64_t base, count;
    int32_t tag0;
    int mode;         // 0: spatial uniform, 1: plane x = xpos, 2: where a quantity is large,
                      // 3: at the shock located per row (shock_ix)
    int dist_flag, ndim;
    double box[6];    // xmin ymin zmin xmax ymax zmax
    double xpos, dt, particle_v0, t_frame, dt_mhd, power_index;
    double p0, pmin, pmax;
    uint32_t key0, key1;
    LargeArgs lg;     // mode 2
    // mode 3: 1-based x index of the shock per (y, z) row of the ghost-padded
    // grid (nyg x nzg rows), and the grid origin and spacing
    const int32_t *shock_ix;
    int nyg, nzg;
    double gxmin, gymin, gzmin, dx, dy, dz;
};
// Status bits (kStatusStepLimit on a runaway rejection loop) go to *status.
cudaError_t launch_inject(const InjectArgs &a, unsigned int *status, cudaStream_t s);
// locate_shock_xpos (mhd_data_parallel.f90:1988-2006) on frame 1: per row of
// the ghost-padded grid, the first 1-based x index of the largest |dvx/dx|.
cudaError_t launch_locate_shock(const float *full, int nxg, int nrows, int32_t *shock_ix,
                                cudaStream_t s);
// get_ncells_large_*: adds the count of grid nodes inside box (strict) whose
// quantity exceeds lg.qmin to *ncells.
cudaError_t launch_count_large(const LargeArgs &lg, int ndim, const double box[6],
                               unsigned long long *ncells, cudaStream_t s);

// Distribution of removed escaped particles by boundary face
// (calc_escaped_distributions): bins[(face * npp + ip) * 3 + {0: count,
// 1: weight hi, 2: weight lo}], face = |count_flag| - 1.
struct EscHist {
    unsigned long long *bins;
    int npp;
    double pmin, pmax, pmin_log, dp_log;
};

// Stable compaction of particles with count_flag == INBOX from src to dst.
// scratch must hold compaction_scratch_bytes(n) bytes.
size_t compaction_scratch_bytes(int64_t n);
cudaError_t launch_remove_particles(const DevParticles &src, const DevParticles &dst, int64_t n,
                                    void *scratch, DevCounters *cnt, const EscHist &esc,
                                    cudaStream_t s);

// Copies the particles of src with count_flag < 0 (escaped through an open
// boundary) to dst[base ..] in order; cnt->nselected gets their number.
// scratch as for launch_remove_particles.
cudaError_t launch_select_escaped(const DevParticles &src, int64_t n, const DevParticles &dst,
                                  int64_t base, void *scratch, DevCounters *cnt, cudaStream_t s);

// One local distribution (flocal of calc_particle_distributions).
struct LocalDistArgs {
    double xmin, ymin, zmin, dxd, dyd, dzd, pmin_log, dp_log, dmu;
    int nmu, npb, nrx, nry, nrz;
    // spherical: weights divided by r^2 sin(theta); nonuniform: spatial bins
    // (binarySearch_R(pos, x) - 1) / r + 1 on the node positions.
    int ndim, spherical, nonuniform, rx, ry, rz, nxg, nyg, nzg;
    const double *xpos, *ypos, *zpos;
};
// bins: (count, whi, wlo) per flocal element, zeroed here.
cudaError_t launch_local_dist(const DevParticles &P, int64_t n, const LocalDistArgs &a,
                              unsigned long long *bins, size_t nbins, cudaStream_t s);
// Local escaped distributions into the per-face (count, whi, wlo) arrays
// fx, fy, fz (zeroed by the caller; nullptr skips a face).
cudaError_t launch_local_escaped(const DevParticles &P, int64_t n, const LocalDistArgs &a,
                                 unsigned long long *fx, unsigned long long *fy,
                                 unsigned long long *fz, cudaStream_t s);
// Global (or, with by_face, escaped) distribution with pitch-angle bins.
struct MuDistArgs {
    double pmin, pmax, pmin_log, dp_log, dmu;
    int npp, nmu, by_face;
};
cudaError_t launch_mu_dist(const DevParticles &P, int64_t n, const MuDistArgs &a,
                           unsigned long long *bins, size_t nbins, cudaStream_t s);
// Splitting: children appended after n in parent order, at most cap - n.
// With tracking on, tracked parents follow split_particle's tracking branch.
cudaError_t launch_split_particles(const DevParticles &P, int64_t n, int64_t cap,
                                   double split_ratio, double pmin_split, double p0,
                                   double pmax, void *scratch, DevCounters *cnt,
                                   cudaStream_t s, const TrackArgs *trk = nullptr);
// Tracking of particles injected in [first, n): inject_one_particle's
// selection (particle_module.f90:434-440).
cudaError_t launch_track_injected(const DevParticles &P, int64_t first, int64_t n,
                                  const TrackArgs &trk, DevCounters *cnt, cudaStream_t s);
// sync_tracked_particles on one rank (particle_module.f90:5994-6030): each
// column keeps its records with tag_splitted < 0 in order, the rest zeroed.
cudaError_t launch_sync_tracked(const TrackArgs &trk, cudaStream_t s);
// get_pmax_global (diagnostics.f90:1691-1721): the largest p over the
// particles, from 0, as the bits of a non-negative double in *bits (zeroed
// by the caller).
cudaError_t launch_pmax(const DevParticles &P, int64_t n, unsigned long long *bits,
                        cudaStream_t s);
// Grid geometry for spatial binning of particles (one bin per field cell).
// tile != 0 orders the bins brick-major for the tile mover: bricks of
// bx x by x bz cells (nbx x nby x nbz of them, the last ones padded), cells
// x-fastest inside a brick, and the cell taken with cell_of() from dx, dy, dz
// exactly as the mover takes it.
struct CellGrid {
    double xmin, ymin, zmin, idx, idy, idz;
    int nxg, nyg, nzg;
    int tile;
    double dx, dy, dz;
    int bx, by, bz, nbx, nby, nbz;
    // done_bin: one more bin after the spatial ones collects the in-box
    // particles that finished the interval, so the next chunk launch covers
    // the paused ones only.  A particle is binned spatially when every
    // particle is (*nactive == 0 after the launch, or all_active), or when it
    // was moved by the launch (index below n_moved) and paused (pause[i]).
    int done_bin, all_active;
    const uint8_t *pause;
    int64_t n_moved;
    const unsigned long long *nactive;
};
// Bins of a grid: cells, or bricks x cells per brick; plus the done bin.
__host__ __device__ int64_t cell_grid_bins(const CellGrid &g);
// The per-bin counts inside the sort scratch; after a sort they hold the
// inclusive prefix (the end of every bin's particle range).
const unsigned int *cell_sort_counts(const void *scratch, int64_t nbins);
// Counting sort of the in-box particles of src into dst by cell; drops the
// rest (remove_particles) and counts escapes.  cnt->nkept gets the new count.
size_t cell_sort_scratch_bytes(int64_t cap, int64_t nbins);
cudaError_t launch_cell_sort(const DevParticles &src, const DevParticles &dst, int64_t n,
                             const CellGrid &g, void *scratch, DevCounters *cnt,
                             const EscHist &esc, cudaStream_t s);
// Global f(p) histogram into (count, whi, wlo) triples per bin (zeroed here).
cudaError_t launch_histogram(const DevParticles &P, int64_t n, int npp, double pmin,
                             double pmax, unsigned long long *bins, cudaStream_t s);
// quick_check reductions into cnt (wsum, dtsum, dt_min, dt_max).
cudaError_t launch_quick_check(const DevParticles &P, int64_t n, DevCounters *cnt,
                               cudaStream_t s);

// Learned splitting launchers (learned.cu).
size_t mlp_shared_bytes();
cudaError_t mlp_set_kernel_attributes();
cudaError_t launch_to_bf16(const float *master, __nv_bfloat16 *w16, cudaStream_t s);
cudaError_t launch_mlp_infer(const __nv_bfloat16 *w16, const float *norm, const float *x, int64_t n,
                             float *z, cudaStream_t s);
cudaError_t launch_mlp_train_step(const MlpTrainBuffers &t, const __nv_bfloat16 *w16,
                                  const float *norm, const float *x, const float *y,
                                  const int64_t *index, int64_t b, float *grad, float *loss,
                                  cudaStream_t s);
cudaError_t launch_adam(float *master, float *m1, float *m2, float *grad, __nv_bfloat16 *w16,
                        float lr, int step, cudaStream_t s);
cudaError_t launch_record_features(const FeatureArgs &g, int ndim, const DevParticles &P, int64_t n,
                                   float *feat, int32_t *tags, unsigned long long *count,
                                   int64_t cap, cudaStream_t s);
cudaError_t launch_label_records(const DevParticles &P, int64_t n, const int32_t *tags,
                                 int64_t nrec, float *p_by_tag, int64_t ntags, float threshold,
                                 float *labels, unsigned long long *npos, cudaStream_t s);
cudaError_t launch_weighted_split(const __nv_bfloat16 *w16, const float *norm,
                                  const FeatureArgs &g, int ndim, const DevParticles &P,
                                  int64_t n, int64_t cap, const WSplitArgs &a,
                                  unsigned long long *count, DevCounters *cnt, cudaStream_t s);
cudaError_t launch_tail(const DevParticles &P, int64_t n, double pthr, unsigned long long *out,
                        cudaStream_t s);
// z of every live particle (index-aligned), its maximum (order-preserving
// int key), and exact sums out = {count, sum(z + 64) hi/lo, sum(w exp(z - zmax)) hi/lo}.
cudaError_t launch_score(const __nv_bfloat16 *w16, const float *norm, const FeatureArgs &g,
                         int ndim, const DevParticles &P, int64_t n, float *z, int *zmax_key,
                         unsigned long long *out, cudaStream_t s);

}  // namespace gpat
