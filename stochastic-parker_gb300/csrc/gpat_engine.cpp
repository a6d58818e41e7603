// Host side of the engine: the C ABI declared in include/gpat_engine.h.
// Owns the device state of one GPAT rank (particles, fields, counters) and
// sequences the kernels in the order the reference's module procedures run.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <new>
#include <vector>

#include "gpat_internal.h"

using namespace gpat;

struct gpat_handle {
    gpat_params_t prm{};
    gpat_mhd_config_t cfg{};
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::string err;
    // fields
    int nxg = 0, nyg = 0, nzg = 0;
    size_t ncells = 0;
    int nslots = 1;
    float *full[2] = {nullptr, nullptr};
    float *rec[2] = {nullptr, nullptr};
    float *staging = nullptr;
    float *aux[2] = {nullptr, nullptr};   // fluctuation records (deltab / correlation runs)
    // Node positions of spherical / non-uniform grids (ghost nodes included)
    // and their inverse spans for the non-uniform gradients, per axis.
    bool grid = false;
    std::vector<double> gpos[3];
    double *dpos[3] = {nullptr, nullptr, nullptr};
    double *dih[3] = {nullptr, nullptr, nullptr};
    // Acceleration-region surfaces (init_acc_surface): [surface][slot].
    bool surf_on = false, surf_has2 = false, surf_inter = true;
    int surf_axis[2] = {0, 0}, surf_sign[2] = {1, 1};
    size_t surf_n[2] = {0, 0}, surf_ld[2] = {0, 0};
    double *dsurf[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    bool fields_set[2] = {false, false};
    bool rec_ready[2] = {false, false};
    // particles (double-buffered SoA)
    int64_t cap = 0, n = 0;
    int cur = 0;
    void *pmem[2] = {nullptr, nullptr};
    DevParticles P[2]{};
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // split-precision path: particles kept binned by cell
    void *sort_scratch = nullptr;
    int64_t sort_bins = 0;   // bins the sort scratch is sized for
    bool unsorted = true;   // particles appended since the last binning
    // Split-precision mover with field bricks in shared memory (mover_tile.cu):
    // brick cells per axis (tile_b[0] = 0: the global-gather mover), threads
    // per CTA, particles per work item; binned_tiles: the last binning was
    // brick-major with this shape.
    int tile_b[3] = {0, 0, 0};
    int tile_h[3] = {0, 0, 0};       // halo cells staged around a brick
    int tile_threads = 512;
    int tile_items = 4096;
    bool binned_tiles = false;
    // chunked split-precision launches: paused flag per index, the particles
    // the last binning put in spatial bins (the rest finished the interval)
    // and the bins of that binning
    uint8_t *pause = nullptr;
    int64_t pause_cap = 0;
    // learned splitting inside the mover (gpat_set_mover_learned): the
    // launch arguments, and on the device the particle count with children,
    // the judged count and the fixed-point sum of w exp(z - z_shift)
    bool learn_on = false;
    FusedLearn learn{};
    unsigned long long *learn_dev = nullptr;
    unsigned long long learn_host[6] = {};
    // weighted splitting's next fresh lineage id (device), and the floor a
    // received particle set puts under it (the most negative tag_splitted)
    unsigned long long *fresh_dev = nullptr;
    unsigned long long fresh_floor = 0;
    int64_t learn_split = 0, learn_killed = 0;
    int64_t n_active = 0;
    int64_t last_sort_bins = 0;
    unsigned int n_spatial_host = 0;
    long long *tile_dev = nullptr;   // item prefix (nbricks + 1) and the item counter
    int64_t tile_dev_n = 0;
    void *tile_ovf = nullptr;        // overflow list: indices, pushes done, count
    int64_t tile_ovf_cap = 0;
    // Chunk-planar copies of the packed records the tile mover stages, per
    // frame slot; rec_gen counts writes of rec[s], plane_gen the copy's source.
    float *planes[2] = {nullptr, nullptr};
    uint64_t rec_gen[2] = {1, 1}, plane_gen[2] = {0, 0};
    DevCounters *dcnt = nullptr;
    DevCounters hcnt{};
    unsigned long long *dbins = nullptr;
    unsigned long long *desc = nullptr;   // escaped distribution, 6 faces x npp x 3
    // escaped_ptls: particles removed through an open boundary while the
    // mover is called with dump_escaped_dist (grown like
    // resize_escaped_particles, particle_module.f90:5329-5358).
    void *emem = nullptr;
    DevParticles E{};
    int64_t ecap = 0, ne = 0;
    // particle tracking (init_particle_tracking, particle_module.f90:5825-5877):
    // tags_tracking(trk_rows, trk_n) and particles_tracked(trk_steps, trk_n)
    int32_t *dtags = nullptr;
    void *tmem = nullptr;
    int32_t *dshock = nullptr;   // shock x index per (y, z) row (locate_shock_xpos)
    DevParticles T{};
    int trk_rows = 0, trk_n = 0;
    int64_t trk_steps = 0;
    // module state kept on the host
    std::vector<double> tstamps;
    int64_t tag_max = 0;
    int64_t nptl_split = 0;
    double last_mover_ms = 0.0;
    uint64_t last_mover_steps = 0;
    int64_t last_mover_launches = 0;
};

namespace {

int fail(gpat_handle_t *h, int code, const std::string &msg) {
    if (h) h->err = msg;
    return code;
}

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return fail(h, GPAT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

double fixed_to_double(unsigned long long hi, unsigned long long lo) {
    return (double)hi + (double)lo * (1.0 / 18446744073709551616.0);
}

// Particle arrays carved out of one allocation, 256-byte aligned each.
size_t particle_bytes(int64_t cap) {
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t c = (size_t)cap;
    return 9 * al(8 * c) + 2 * al(c) + 6 * al(4 * c);
}

DevParticles carve(void *base, int64_t cap) {
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    char *q = static_cast<char *>(base);
    const size_t c = (size_t)cap;
    DevParticles P{};
    double **d[9] = {&P.x, &P.y, &P.z, &P.p, &P.v, &P.mu, &P.weight, &P.t, &P.dt};
    for (auto *pp : d) { *pp = reinterpret_cast<double *>(q); q += al(8 * c); }
    P.split_times = reinterpret_cast<int8_t *>(q); q += al(c);
    P.count_flag = reinterpret_cast<int8_t *>(q); q += al(c);
    int32_t **i4[5] = {&P.origin, &P.nsteps_tracked, &P.nsteps_pushed, &P.tag_injected,
                       &P.tag_splitted};
    for (auto *pp : i4) { *pp = reinterpret_cast<int32_t *>(q); q += al(4 * c); }
    P.rng_ctr = reinterpret_cast<uint32_t *>(q);
    return P;
}

TrackArgs track_args(const gpat_handle_t *h) {
    TrackArgs t{};
    if (!h->dtags) return t;
    t.tags = h->dtags;
    t.nrows = h->trk_rows;
    t.n = h->trk_n;
    t.nsteps_max = h->trk_steps;
    t.rec = h->T;
    return t;
}

int check_status(gpat_handle_t *h) {
    if (h->hcnt.status) {
        const unsigned s = h->hcnt.status;
        std::string m = "device status:";
        if (s & kStatusIndexGuard) {
            m += " interpolation index outside the ghost cells;";
            const unsigned long long v = h->hcnt.bad_value;
            if (v && !(s & kStatusTileMiss)) {
                m += " (node " + std::to_string((short)(v & 0xffff)) + ", " +
                     std::to_string((short)((v >> 16) & 0xffff)) + ", " +
                     std::to_string((short)((v >> 32) & 0xffff)) + "; " +
                     (((v >> 48) & 0xff) == 2 ? "brick" : "global") + " gather)";
                CK(cudaMemsetAsync(&h->dcnt->bad_value, 0, sizeof(unsigned long long), h->stream));
            }
        }
        if (s & kStatusNonFinite) m += " non-finite particle state;";
        if (s & kStatusStepLimit) m += " per-call push/iteration limit reached;";
        if (s & kStatusTileTimeout) m += " a field brick copy into shared memory timed out;";
        if (s & kStatusTileMiss) {
            const unsigned long long v = h->hcnt.bad_value;
            m += " a particle outside the staged brick it was binned in (node " +
                 std::to_string(v & 0xffff) + ", " + std::to_string((v >> 16) & 0xffff) +
                 ", region origin " + std::to_string((short)((v >> 32) & 0xffff)) + ", " +
                 std::to_string((short)((v >> 48) & 0xffff)) + ");";
            CK(cudaMemsetAsync(&h->dcnt->bad_value, 0, sizeof(unsigned long long), h->stream));
        }
        CK(cudaMemsetAsync(&h->dcnt->status, 0, sizeof(unsigned int), h->stream));
        h->hcnt.status = 0;
        return fail(h, GPAT_ERR_DEVICE, m);
    }
    return GPAT_OK;
}

int pull_counters(gpat_handle_t *h) {
    CK(cudaMemcpyAsync(&h->hcnt, h->dcnt, sizeof(DevCounters), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

// conf.dat reading with the reference's get_variable semantics
// (read_config.f90:20-44): scan forward line by line from the current
// position for a line containing the key; the value is read list-directed
// after the first delimiter, up to ';' or the end of the line.  A key that
// is not found before EOF reads as -1 and leaves the file at EOF.
struct ConfScanner {
    std::vector<std::string> lines;
    size_t pos = 0;
    bool load(const char *path) {
        FILE *f = std::fopen(path, "r");
        if (!f) return false;
        char buf[4096];
        while (std::fgets(buf, sizeof buf, f)) {
            std::string s(buf);
            while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
            if (s.size() > 150) s.resize(150);   // character(len=150) single_line
            lines.push_back(s);
        }
        std::fclose(f);
        return true;
    }
    double get(const char *key, char delim = '=') {
        while (pos < lines.size()) {
            const std::string &s = lines[pos++];
            if (s.find(key) != std::string::npos) return parse(s, delim);
        }
        return -1.0;
    }
    static double parse(const std::string &line, char delim) {
        std::string s = line;
        while (!s.empty() && (s.back() == ' ' || s.back() == '\t')) s.pop_back();
        size_t end = s.size();
        const size_t semi = s.find(';');
        if (semi != std::string::npos) end = semi;
        const size_t d = s.find(delim);
        if (d == std::string::npos || d + 1 > end) return -1.0;
        std::string v = s.substr(d + 1, end - d - 1);
        for (char &c : v)
            if (c == 'd' || c == 'D') c = 'e';   // Fortran D exponent
        size_t a = v.find_first_not_of(" \t,");
        if (a == std::string::npos) return -1.0;
        char *stop = nullptr;
        const double x = std::strtod(v.c_str() + a, &stop);
        if (stop == v.c_str() + a) return -1.0;
        return x;
    }
};

int to_int_via_real4(double v) { return (int)(float)v; }

int mover_args(gpat_handle_t *h, int mhd_tframe, int nsteps_interval, int num_fine_steps,
               MoverArgs &a) {
    const gpat_params_t &p = h->prm;
    const gpat_mhd_config_t &c = h->cfg;
    if (mhd_tframe < 1 || (size_t)mhd_tframe + 1 > h->tstamps.size())
        return fail(h, GPAT_ERR_ARG, "mhd_tframe outside the time stamps");
    if (nsteps_interval < 1 || num_fine_steps < 1)
        return fail(h, GPAT_ERR_ARG, "nsteps_interval and num_fine_steps must be >= 1");
    if (!h->rec_ready[0] || (p.time_interp && !h->rec_ready[1]))
        return fail(h, GPAT_ERR_STATE, "fields and their gradients are not set");
    std::memset(&a, 0, sizeof a);
    a.P = h->P[h->cur];
    a.n = h->n;
    a.rec1 = h->rec[0];
    a.rec2 = p.time_interp ? h->rec[1] : h->rec[0];
    a.full1 = h->full[0];
    a.full2 = p.time_interp ? h->full[1] : h->full[0];
    a.deltab_flag = p.deltab_flag;
    a.correlation_flag = p.correlation_flag;
    a.aux1 = h->aux[0];
    a.aux2 = p.time_interp ? h->aux[1] : h->aux[0];
    a.duu0 = p.duu0;
    a.dpp_wave = p.dpp_wave;
    a.dpp_shear = p.dpp_shear;
    a.weak_scattering = p.weak_scattering;
    a.tau0 = p.tau0;
    a.time_interp = p.time_interp;
    a.ndim = p.ndim;
    a.nxg = h->nxg; a.nyg = h->nyg; a.nzg = h->nzg;
    a.nsteps_interval = nsteps_interval;
    a.num_fine_steps = num_fine_steps;
    a.dx = c.dx; a.dy = c.dy; a.dz = c.dz;
    a.idx = 1.0 / c.dx; a.idy = 1.0 / c.dy; a.idz = 1.0 / c.dz;
    // set_field_configuration on one rank (simulation_setup.f90:171-253).
    a.xmin = c.xmin; a.xmax = c.xmin + (double)c.nx * c.dx;
    a.ymin = c.ymin; a.ymax = c.ymin + (double)c.ny * c.dy;
    a.zmin = c.zmin;
    a.zmax = (p.ndim == 3) ? c.zmin + (double)c.nz * c.dz : c.zmax;
    a.xmin1 = a.xmin - c.dx * 0.5; a.xmax1 = a.xmax + c.dx * 0.5;
    a.ymin1 = a.ymin - c.dy * 0.5; a.ymax1 = a.ymax + c.dy * 0.5;
    a.zmin1 = a.zmin - c.dz * 0.5; a.zmax1 = a.zmax + c.dz * 0.5;
    a.spherical = p.spherical_coord ? 1 : 0;
    a.nonuniform = p.nonuniform_grid ? 1 : 0;
    a.include_3rd = (p.ndim == 2 && p.include_3rd_dim) ? 1 : 0;
    a.surf_on = h->surf_on ? 1 : 0;
    a.surf_has2 = h->surf_has2 ? 1 : 0;
    a.surf_inter = h->surf_inter ? 1 : 0;
    for (int k = 0; k < 2; ++k) {
        a.surf_axis[k] = h->surf_axis[k];
        a.surf_sign[k] = h->surf_sign[k];
        a.surf_ld[k] = (int)h->surf_ld[k];
        a.surf[k][0] = h->dsurf[k][0];
        a.surf[k][1] = p.time_interp ? h->dsurf[k][1] : h->dsurf[k][0];
    }
    a.xpos = h->dpos[0]; a.ypos = h->dpos[1]; a.zpos = h->dpos[2];
    if (p.nonuniform_grid) {
        // particle_mover_one_cycle (:1535-1546): the half cells beyond the
        // box are those of the first and last cells (xpos_local(i) is node
        // i + 1); the z extension only matters in 3D.
        const std::vector<double> &X = h->gpos[0], &Y = h->gpos[1], &Z = h->gpos[2];
        a.xmin1 = a.xmin - (X[3] - X[2]) * 0.5;
        a.xmax1 = a.xmax + (X[c.nx + 2] - X[c.nx + 1]) * 0.5;
        if (p.ndim > 1) {   // 1D runs keep no y positions
            a.ymin1 = a.ymin - (Y[3] - Y[2]) * 0.5;
            a.ymax1 = a.ymax + (Y[c.ny + 2] - Y[c.ny + 1]) * 0.5;
        }
        if (p.ndim == 3) {
            a.zmin1 = a.zmin - (Z[3] - Z[2]) * 0.5;
            a.zmax1 = a.zmax + (Z[c.nz + 2] - Z[c.nz + 1]) * 0.5;
        }
    }
    a.cfg_xmin = c.xmin; a.cfg_ymin = c.ymin; a.cfg_zmin = c.zmin;
    a.cfg_lx = c.lx; a.cfg_ly = c.ly; a.cfg_lz = c.lz;
    a.t0 = h->tstamps[mhd_tframe - 1];
    a.dtf = h->tstamps[mhd_tframe] - a.t0;
    if (!(a.dtf > 0.0)) return fail(h, GPAT_ERR_ARG, "time stamps must increase");
    // set_dt_min_max (particle_module.f90:5519-5524).
    a.dt_min = p.dt_min_rel * a.dtf;
    a.dt_max = p.dt_max_rel * a.dtf;
    a.dt_fine = a.dtf / num_fine_steps;
    a.limit = a.dtf + a.dt_fine * (double)0.1f;
    const double dt_floor = std::min(a.dt_min, a.dt_max);
    if (!(dt_floor > 0.0)) return fail(h, GPAT_ERR_ARG, "dt_min_rel and dt_max_rel must be > 0");
    const double pushes = std::ceil(a.dtf / dt_floor) + 2.0 * num_fine_steps + 16.0;
    if (pushes > 2.0e9) return fail(h, GPAT_ERR_ARG, "dtf / dt_min exceeds 2e9 pushes");
    a.max_pushes = (uint32_t)pushes;
    a.p0 = p.p0; a.pindex = p.pindex; a.gamma_turb = p.gamma_turb;
    a.kpara0 = p.kpara0; a.kret = p.kret; a.drift1 = p.drift1; a.drift2 = p.drift2;
    for (int i = 0; i < 6; ++i) a.acc_region[i] = p.acc_region[i];
    a.charge = p.charge;
    a.momentum_dependency = p.momentum_dependency;
    a.mag_dependency = p.mag_dependency;
    a.acc_region_flag = p.acc_region_flag;
    a.check_drift_2d = p.check_drift_2d;
    a.pbcx = p.pbcx; a.pbcy = p.pbcy; a.pbcz = p.pbcz;
    a.noise = p.noise;
    a.key0 = (uint32_t)p.seed;
    a.key1 = (uint32_t)(p.seed >> 32);
    a.trk = track_args(h);
    a.cnt = h->dcnt;
    a.pause = nullptr;
    return GPAT_OK;
}

// tiled: bins ordered brick-major with the handle's brick shape (tile mover).
CellGrid cell_grid(const gpat_handle_t *h, bool tiled = false) {
    CellGrid g{};
    g.xmin = h->cfg.xmin; g.ymin = h->cfg.ymin; g.zmin = h->cfg.zmin;
    g.idx = 1.0 / h->cfg.dx; g.idy = 1.0 / h->cfg.dy;
    g.idz = h->prm.ndim == 3 ? 1.0 / h->cfg.dz : 0.0;
    g.nxg = h->nxg; g.nyg = h->nyg; g.nzg = h->nzg;
    if (tiled) {
        g.tile = 1;
        g.dx = h->cfg.dx; g.dy = h->cfg.dy; g.dz = h->cfg.dz;
        g.bx = h->tile_b[0]; g.by = h->tile_b[1];
        g.bz = h->prm.ndim == 3 ? h->tile_b[2] : 1;
        g.nbx = (h->nxg + g.bx - 1) / g.bx;
        g.nby = (h->nyg + g.by - 1) / g.by;
        g.nbz = (h->nzg + g.bz - 1) / g.bz;
    }
    return g;
}

bool tiles_on(const gpat_handle_t *h) {
    return h->tile_b[0] > 0 && h->prm.precision == GPAT_PREC_MIXED;
}

// Bins the current particles by cell into the other buffer (split-precision
// path), dropping particles that are not in the box.
EscHist escaped_hist(const gpat_handle_t *h) {
    EscHist e;
    e.bins = h->desc;
    e.npp = h->prm.npp_global;
    e.pmin = h->prm.pmin;
    e.pmax = h->prm.pmax;
    e.pmin_log = std::log10(h->prm.pmin);
    e.dp_log = (std::log10(h->prm.pmax) - e.pmin_log) / h->prm.npp_global;
    return e;
}

// tiled: brick-major bins for the tile mover (the sort scratch grows to fit).
// n_moved >= 0: the binning after a chunk launch that moved the first n_moved
// particles.  While some are still paused, those that finished the interval
// go to the trailing done bin and h->n_active counts the paused ones, which
// lead the array; once none is paused, every particle is binned spatially
// again for the next interval.  n_moved < 0: every particle spatially.
int bin_particles(gpat_handle_t *h, bool tiled = false, int64_t n_moved = -1) {
    const int nxt = 1 - h->cur;
    CellGrid g = cell_grid(h, tiled);
    if (n_moved >= 0 && h->pause) {
        g.done_bin = 1;
        g.pause = h->pause;
        g.n_moved = n_moved;
        g.nactive = &h->dcnt->nactive;
    }
    const int64_t nbins = cell_grid_bins(g);
    if (nbins > h->sort_bins) {
        CK(cudaStreamSynchronize(h->stream));
        if (h->sort_scratch) CK(cudaFree(h->sort_scratch));
        h->sort_scratch = nullptr;
        h->sort_bins = 0;
        if (cudaMalloc(&h->sort_scratch, cell_sort_scratch_bytes(h->cap, nbins)) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, GPAT_ERR_OOM, "binning scratch");
        }
        h->sort_bins = nbins;
    }
    CK(launch_cell_sort(h->P[h->cur], h->P[nxt], h->n, g, h->sort_scratch, h->dcnt,
                        escaped_hist(h), h->stream));
    if (g.done_bin && h->n > 0)   // particles in spatial bins: the prefix before the done bin
        CK(cudaMemcpyAsync(&h->n_spatial_host, cell_sort_counts(h->sort_scratch, nbins) + nbins - 2,
                           sizeof(unsigned int), cudaMemcpyDeviceToHost, h->stream));
    int rc = pull_counters(h);
    if (rc) return rc;
    h->cur = nxt;
    h->n = (int64_t)h->hcnt.nkept;
    h->n_active = (g.done_bin && h->n > 0) ? (int64_t)h->n_spatial_host : h->n;
    h->last_sort_bins = nbins;
    h->unsorted = false;
    h->binned_tiles = tiled;
    return GPAT_OK;
}

int ensure_pause(gpat_handle_t *h) {
    if (h->pause_cap >= h->cap) return GPAT_OK;
    CK(cudaStreamSynchronize(h->stream));
    if (h->pause) CK(cudaFree(h->pause));
    h->pause = nullptr;
    h->pause_cap = 0;
    if (cudaMalloc(&h->pause, (size_t)h->cap) != cudaSuccess) {
        cudaGetLastError();
        return fail(h, GPAT_ERR_OOM, "pause flags");
    }
    h->pause_cap = h->cap;
    return GPAT_OK;
}

// Copies the node positions to the device with their inverse spans
// idxh_grid (set_local_grid_positions, mhd_data_parallel.f90:2172-2189):
// 1 / (x[i+1] - x[i-1]) inside, the one-sided spans at the two ends.
int upload_grid(gpat_handle_t *h) {
    for (int ax = 0; ax < h->prm.ndim; ++ax) {
        const std::vector<double> &x = h->gpos[ax];
        const size_t n = x.size();
        std::vector<double> ih(n, 0.0);
        if (n >= 3) {
            for (size_t i = 1; i + 1 < n; ++i) ih[i] = 1.0 / (x[i + 1] - x[i - 1]);
            ih[0] = 1.0 / (-(3.0 * x[0]) + 4.0 * x[1] - x[2]);
            ih[n - 1] = 1.0 / (3.0 * x[n - 1] - 4.0 * x[n - 2] + x[n - 3]);
        }
        CK(cudaMemcpyAsync(h->dpos[ax], x.data(), sizeof(double) * n, cudaMemcpyHostToDevice,
                           h->stream));
        CK(cudaMemcpyAsync(h->dih[ax], ih.data(), sizeof(double) * n, cudaMemcpyHostToDevice,
                           h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

// The inverse spans for the non-uniform gradients, or null (uniform 0.5/d).
const double *const *grad_spans(const gpat_handle_t *h) {
    return h->prm.nonuniform_grid ? h->dih : nullptr;
}

// Copies the first n particles of one carved buffer to another.
cudaError_t copy_particles_d2d(const DevParticles &S, const DevParticles &D, int64_t n,
                               cudaStream_t s) {
    const size_t c = (size_t)n;
    const void *src[17] = {S.x, S.y, S.z, S.p, S.v, S.mu, S.weight, S.t, S.dt, S.split_times,
                           S.count_flag, S.origin, S.nsteps_tracked, S.nsteps_pushed,
                           S.tag_injected, S.tag_splitted, S.rng_ctr};
    void *dst[17] = {D.x, D.y, D.z, D.p, D.v, D.mu, D.weight, D.t, D.dt, D.split_times,
                     D.count_flag, D.origin, D.nsteps_tracked, D.nsteps_pushed,
                     D.tag_injected, D.tag_splitted, D.rng_ctr};
    const size_t width[17] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 1, 1, 4, 4, 4, 4, 4, 4};
    for (int k = 0; k < 17; ++k) {
        const cudaError_t e = cudaMemcpyAsync(dst[k], src[k], width[k] * c,
                                              cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// remove_particles' copy of the escaped particles (particle_module.f90:
// 5368-5392): before the current set drops them, particles with
// count_flag < 0 are appended to the escaped store in set order.
int collect_escaped(gpat_handle_t *h) {
    if (h->n <= 0) return GPAT_OK;
    if (h->ne + h->n > h->ecap) {
        const int64_t ncap = std::max((int64_t)(1.25 * (double)h->ecap), h->ne + h->n);
        void *mem = nullptr;
        CK(cudaMalloc(&mem, particle_bytes(ncap)));
        const DevParticles N = carve(mem, ncap);
        if (h->ne > 0) CK(copy_particles_d2d(h->E, N, h->ne, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (h->emem) CK(cudaFree(h->emem));
        h->emem = mem;
        h->E = N;
        h->ecap = ncap;
    }
    CK(launch_select_escaped(h->P[h->cur], h->n, h->E, h->ne, h->scratch, h->dcnt, h->stream));
    const int rc = pull_counters(h);
    if (rc) return rc;
    h->ne += (int64_t)h->hcnt.nselected;
    return GPAT_OK;
}

int ensure_scratch(gpat_handle_t *h, int64_t n) {
    const size_t need = compaction_scratch_bytes(n);
    if (need <= h->scratch_bytes) return GPAT_OK;
    if (h->scratch) CK(cudaFree(h->scratch));
    h->scratch = nullptr;
    CK(cudaMalloc(&h->scratch, need));
    h->scratch_bytes = need;
    return GPAT_OK;
}

}  // namespace

extern "C" {

const char *gpat_version(void) { return "gpat-gb300 0.1 (sm_103a)"; }

const char *gpat_last_error(const gpat_handle_t *h) { return h ? h->err.c_str() : "null handle"; }

int gpat_get_variable(const char *conf_path, const char *key, double *value) {
    if (!conf_path || !key || !value) return GPAT_ERR_ARG;
    ConfScanner sc;
    if (!sc.load(conf_path)) return GPAT_ERR_IO;
    *value = sc.get(key);
    return GPAT_OK;
}

int gpat_read_particle_params(const char *conf_path, gpat_params_t *p) {
    if (!conf_path || !p) return GPAT_ERR_ARG;
    ConfScanner sc;
    if (!sc.load(conf_path)) return GPAT_ERR_IO;
    // read_particle_params key order (particle_module.f90:2790-2815).
    p->b0 = sc.get("b0");
    p->p0 = sc.get("p0");
    p->pmin = sc.get("pmin");
    p->pmax = sc.get("pmax");
    p->momentum_dependency = to_int_via_real4(sc.get("momentum_dependency"));
    p->gamma_turb = sc.get("gamma_turb");
    p->pindex = 3.0 - p->gamma_turb;
    p->mag_dependency = to_int_via_real4(sc.get("mag_dependency"));
    p->kpara0 = sc.get("kpara0");
    p->kret = sc.get("kret");
    p->dt_min_rel = sc.get("dt_min_rel");
    p->dt_max_rel = sc.get("dt_max_rel");
    p->acc_region_flag = to_int_via_real4(sc.get("acc_region_flag"));
    double acc[6];
    const char *acc_keys[6] = {"acc_xmin", "acc_xmax", "acc_ymin", "acc_ymax", "acc_zmin", "acc_zmax"};
    for (int i = 0; i < 6; ++i) acc[i] = sc.get(acc_keys[i]);
    if (p->acc_region_flag == 1) {
        for (int i = 0; i < 6; ++i) p->acc_region[i] = acc[i];
    } else {
        const double dflt[6] = {0.0, 1.0, 0.0, 1.0, 0.0, 1.0};
        for (int i = 0; i < 6; ++i) p->acc_region[i] = dflt[i];
    }
    // read_particle_boundary_conditions (simulation_setup.f90:104-150).
    ConfScanner sb;
    sb.load(conf_path);
    p->pbcx = to_int_via_real4(sb.get("pbcx"));
    p->pbcy = to_int_via_real4(sb.get("pbcy"));
    p->pbcz = to_int_via_real4(sb.get("pbcz"));
    // read_diagnostics_params (diagnostics.f90:2049-2100): npp_global first.
    ConfScanner sd;
    sd.load(conf_path);
    const double npp = sd.get("npp_global");
    if (npp > 0) p->npp_global = (int)npp;
    return GPAT_OK;
}

int gpat_load_mhd_config(const char *path, gpat_mhd_config_t *cfg) {
    // The file holds the 156 bytes of the record without trailing padding.
    constexpr size_t kRecord = 13 * 8 + 13 * 4;
    static_assert(offsetof(gpat_mhd_config_t, bcz) + 4 == kRecord, "mhd_config layout");
    if (!path || !cfg) return GPAT_ERR_ARG;
    FILE *f = std::fopen(path, "rb");
    if (!f) return GPAT_ERR_IO;
    std::memset(cfg, 0, sizeof(*cfg));
    const size_t got = std::fread(cfg, 1, kRecord, f);
    std::fclose(f);
    return got == kRecord ? GPAT_OK : GPAT_ERR_IO;
}

int gpat_create(const gpat_params_t *params, const gpat_mhd_config_t *cfg, int device,
                gpat_handle_t **out) {
    if (!params || !cfg || !out) return GPAT_ERR_ARG;
    *out = nullptr;
    const gpat_params_t &p = *params;
    if (p.ndim < 1 || p.ndim > 3) return GPAT_ERR_UNSUPPORTED;
    if (p.include_3rd_dim && p.ndim != 2) return GPAT_ERR_ARG;
    if ((p.dpp_wave || p.dpp_shear || p.deltab_flag || p.correlation_flag || p.spherical_coord ||
         p.nonuniform_grid || p.include_3rd_dim || p.ndim == 1) &&
        p.precision != GPAT_PREC_FP64)
        return GPAT_ERR_UNSUPPORTED;
    if (p.precision != GPAT_PREC_FP64 && p.precision != GPAT_PREC_MIXED) return GPAT_ERR_ARG;
    if (p.noise != GPAT_NOISE_UNIFORM && p.noise != GPAT_NOISE_GAUSS) return GPAT_ERR_ARG;
    if (p.nptl_max < 1 || p.nptl_max > (int64_t)2000000000) return GPAT_ERR_ARG;
    // The histogram keeps 3 x 8 bytes per bin in shared memory (48 KB max).
    if (p.npp_global < 1 || p.npp_global > 2048) return GPAT_ERR_ARG;
    if (!(p.p0 > 0.0) || !(p.pmin > 0.0) || !(p.pmax > p.pmin)) return GPAT_ERR_ARG;
    if (cfg->nx < 1 || cfg->ny < 1 || (p.ndim == 3 && cfg->nz < 1)) return GPAT_ERR_ARG;
    if (!(cfg->dx > 0.0) || !(cfg->dy > 0.0) || (p.ndim == 3 && !(cfg->dz > 0.0))) return GPAT_ERR_ARG;

    gpat_handle_t *h = new gpat_handle_t();
    h->prm = p;
    h->cfg = *cfg;
    h->device = device;
    auto bail = [&](int code) {
        gpat_destroy(h);
        return code;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail(GPAT_ERR_CUDA);
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return bail(GPAT_ERR_CUDA);
    h->sm_count = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
        return bail(GPAT_ERR_CUDA);
    // init_field_data (mhd_data_parallel.f90:66-105): ghost cells on each
    // resolved side; the z extent of a 2D run is nz (one plane).
    h->nxg = cfg->nx + 4;
    // 1D arrays are (-1:nx+2, 1, 1) (init_field_data :80-81)
    h->nyg = (p.ndim == 1) ? 1 : cfg->ny + 4;
    h->nzg = (p.ndim == 3) ? cfg->nz + 4 : std::max(1, cfg->nz);
    if (p.ndim == 1) h->nzg = 1;
    if (p.ndim == 2 && h->nzg != 1) return bail(GPAT_ERR_UNSUPPORTED);
    h->ncells = (size_t)h->nxg * h->nyg * h->nzg;
    h->nslots = p.time_interp ? 2 : 1;
    const int R = (p.ndim == 2) ? kRec2D : kRec3D;
    for (int s = 0; s < h->nslots; ++s) {
        if (cudaMalloc(&h->full[s], 32 * sizeof(float) * h->ncells) != cudaSuccess ||
            cudaMalloc(&h->rec[s], (size_t)R * sizeof(float) * h->ncells) != cudaSuccess)
            return bail(GPAT_ERR_OOM);
        cudaMemsetAsync(h->full[s], 0, 32 * sizeof(float) * h->ncells, h->stream);
        // init_magnetic_fluctuation / init_correlation_length
        // (mhd_data_parallel.f90:107-182): every component starts at 1
        if (p.deltab_flag || p.correlation_flag) {
            if (cudaMalloc(&h->aux[s], 16 * sizeof(float) * h->ncells) != cudaSuccess)
                return bail(GPAT_ERR_OOM);
            if (launch_fill(h->aux[s], 1.0f, 16 * h->ncells, h->stream) != cudaSuccess)
                return bail(GPAT_ERR_CUDA);
        }
    }
    // Grid positions (init_grid_positions / set_local_grid_positions,
    // mhd_data_parallel.f90:2051-2190): the uniform positions until
    // gpat_set_grid_positions or gpat_read_grid_positions replaces them.
    if (p.spherical_coord || p.nonuniform_grid) {
        h->grid = true;
        const int ng[3] = {h->nxg, h->nyg, h->nzg};
        const double d[3] = {cfg->dx, cfg->dy, cfg->dz};
        const double o[3] = {cfg->xmin, cfg->ymin, cfg->zmin};
        for (int ax = 0; ax < p.ndim; ++ax) {
            h->gpos[ax].resize(ng[ax]);
            for (int j = 0; j < ng[ax]; ++j) h->gpos[ax][j] = d[ax] * (double)(j - 2) + o[ax];
            if (cudaMalloc(&h->dpos[ax], sizeof(double) * ng[ax]) != cudaSuccess ||
                cudaMalloc(&h->dih[ax], sizeof(double) * ng[ax]) != cudaSuccess)
                return bail(GPAT_ERR_OOM);
        }
        if (upload_grid(h) != GPAT_OK) return bail(GPAT_ERR_CUDA);
    }
    // init_particles (particle_module.f90:177-258), double-buffered.
    h->cap = p.nptl_max;
    for (int b = 0; b < 2; ++b) {
        if (cudaMalloc(&h->pmem[b], particle_bytes(h->cap)) != cudaSuccess) return bail(GPAT_ERR_OOM);
        cudaMemsetAsync(h->pmem[b], 0, particle_bytes(h->cap), h->stream);
        h->P[b] = carve(h->pmem[b], h->cap);
    }
    if (p.precision == GPAT_PREC_MIXED) {
        if (cudaMalloc(&h->sort_scratch, cell_sort_scratch_bytes(h->cap, (int64_t)h->ncells)) !=
            cudaSuccess)
            return bail(GPAT_ERR_OOM);
        h->sort_bins = (int64_t)h->ncells;
    }
    if (cudaMalloc(&h->dcnt, sizeof(DevCounters)) != cudaSuccess) return bail(GPAT_ERR_OOM);
    cudaMemsetAsync(h->dcnt, 0, sizeof(DevCounters), h->stream);
    if (cudaMalloc(&h->dbins, sizeof(unsigned long long) * 3 * (size_t)p.npp_global) != cudaSuccess)
        return bail(GPAT_ERR_OOM);
    const size_t esc_bytes = sizeof(unsigned long long) * 3 * 6 * (size_t)p.npp_global;
    if (cudaMalloc(&h->desc, esc_bytes) != cudaSuccess) return bail(GPAT_ERR_OOM);
    cudaMemsetAsync(h->desc, 0, esc_bytes, h->stream);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(GPAT_ERR_CUDA);
    *out = h;
    return GPAT_OK;
}

int gpat_destroy(gpat_handle_t *h) {
    if (!h) return GPAT_ERR_ARG;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (int s = 0; s < 2; ++s) {
        if (h->full[s]) cudaFree(h->full[s]);
        if (h->rec[s]) cudaFree(h->rec[s]);
        if (h->aux[s]) cudaFree(h->aux[s]);
    }
    for (int ax = 0; ax < 3; ++ax) {
        if (h->dpos[ax]) cudaFree(h->dpos[ax]);
        if (h->dih[ax]) cudaFree(h->dih[ax]);
    }
    for (int k = 0; k < 2; ++k)
        for (int t = 0; t < 2; ++t)
            if (h->dsurf[k][t]) cudaFree(h->dsurf[k][t]);
    for (int s = 0; s < 2; ++s) {
        if (h->pmem[s]) cudaFree(h->pmem[s]);
    }
    if (h->staging) cudaFree(h->staging);
    if (h->emem) cudaFree(h->emem);
    if (h->tmem) cudaFree(h->tmem);
    if (h->dtags) cudaFree(h->dtags);
    if (h->dshock) cudaFree(h->dshock);
    if (h->scratch) cudaFree(h->scratch);
    if (h->sort_scratch) cudaFree(h->sort_scratch);
    if (h->tile_dev) cudaFree(h->tile_dev);
    if (h->pause) cudaFree(h->pause);
    if (h->learn_dev) cudaFree(h->learn_dev);
    if (h->fresh_dev) cudaFree(h->fresh_dev);
    if (h->tile_ovf) cudaFree(h->tile_ovf);
    for (int s = 0; s < 2; ++s)
        if (h->planes[s]) cudaFree(h->planes[s]);
    if (h->dcnt) cudaFree(h->dcnt);
    if (h->dbins) cudaFree(h->dbins);
    if (h->desc) cudaFree(h->desc);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return GPAT_OK;
}

int gpat_set_tstamps(gpat_handle_t *h, const double *ts, int n) {
    if (!h || !ts || n < 2) return fail(h, GPAT_ERR_ARG, "need at least two time stamps");
    h->tstamps.assign(ts, ts + n);
    return GPAT_OK;
}

int gpat_calc_tstamps_mhd(gpat_handle_t *h, int t_start, int t_end) {
    if (!h || t_end <= t_start) return fail(h, GPAT_ERR_ARG, "t_end must exceed t_start");
    // calc_tstamps_mhd (mhd_config.f90:263-271): tstamps(i) = i * dt_out.
    h->tstamps.clear();
    for (int i = t_start; i <= t_end; ++i) h->tstamps.push_back(i * h->cfg.dt_out);
    return GPAT_OK;
}

int gpat_load_tstamps_mhd(gpat_handle_t *h, int t_start, int t_end, int tmax_mhd,
                          const char *dir_mhd_data) {
    if (!h || !dir_mhd_data) return GPAT_ERR_ARG;
    if (t_end <= t_start) return fail(h, GPAT_ERR_ARG, "t_end must exceed t_start");
    // load_tstamps_mhd (mhd_config.f90:221-255): int32 first frame ts_mhd at
    // byte 0, the stamp of frame i in 8-byte slot i - ts_mhd + 2; frames past
    // tmax_mhd continue with the last interval.
    const std::string path = std::string(dir_mhd_data) + "time_stamps.dat";
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return fail(h, GPAT_ERR_IO, "cannot open " + path);
    int32_t ts_mhd = 0;
    const int n = t_end - t_start + 1;
    const int nread = std::min(tmax_mhd, t_end) - t_start + 1;
    std::vector<double> ts((size_t)n, 0.0);
    bool ok = std::fread(&ts_mhd, sizeof ts_mhd, 1, f) == 1 && t_start >= ts_mhd && nread >= 1;
    if (ok) ok = std::fseek(f, (long)(t_start - ts_mhd + 2) * 8, SEEK_SET) == 0;
    if (ok) ok = std::fread(ts.data(), sizeof(double), (size_t)nread, f) == (size_t)nread;
    std::fclose(f);
    if (!ok) return fail(h, GPAT_ERR_IO, "time_stamps.dat does not cover t_start .. tmax_mhd");
    if (nread < n) {
        if (nread < 2) return fail(h, GPAT_ERR_ARG, "tmax_mhd leaves fewer than two stamps");
        const double dt_last = ts[nread - 1] - ts[nread - 2];
        for (int i = nread; i < n; ++i) ts[i] = ts[i - 1] + dt_last;
    }
    h->tstamps = ts;
    return GPAT_OK;
}

int gpat_set_fields(gpat_handle_t *h, int var_flag, const float *farray, int nvar) {
    if (!h || !farray || (nvar != 8 && nvar != 32)) return fail(h, GPAT_ERR_ARG, "nvar must be 8 or 32");
    const int slot = var_flag == 0 ? 0 : 1;
    if (slot >= h->nslots) return fail(h, GPAT_ERR_STATE, "farray2 needs time_interp = 1");
    CK(cudaSetDevice(h->device));
    if (nvar == 32) {
        CK(cudaMemcpyAsync(h->full[slot], farray, 32 * sizeof(float) * h->ncells,
                           cudaMemcpyHostToDevice, h->stream));
        CK(launch_pack_records(h->full[slot], h->rec[slot], h->prm.ndim, h->ncells, h->stream));
        h->rec_ready[slot] = true;
        ++h->rec_gen[slot];
    } else {
        if (!h->staging) CK(cudaMalloc(&h->staging, 8 * sizeof(float) * h->ncells));
        CK(cudaMemcpyAsync(h->staging, farray, 8 * sizeof(float) * h->ncells,
                           cudaMemcpyHostToDevice, h->stream));
        CK(launch_scatter_raw_fields(h->staging, 8, h->full[slot], h->ncells, h->stream));
        h->rec_ready[slot] = false;
    }
    CK(cudaStreamSynchronize(h->stream));
    h->fields_set[slot] = true;
    return GPAT_OK;
}

int gpat_set_fluctuations(gpat_handle_t *h, int var_flag, const float *db2_slab,
                          const float *db2_2d, const float *lc_slab, const float *lc_2d) {
    if (!h) return GPAT_ERR_ARG;
    const int slot = var_flag == 0 ? 0 : 1;
    if (slot >= h->nslots) return fail(h, GPAT_ERR_STATE, "slot 1 needs time_interp = 1");
    if (!h->aux[slot])
        return fail(h, GPAT_ERR_STATE, "fluctuation arrays need deltab_flag or correlation_flag");
    CK(cudaSetDevice(h->device));
    if (!h->staging) CK(cudaMalloc(&h->staging, 8 * sizeof(float) * h->ncells));
    const float *src[4] = {db2_slab, db2_2d, lc_slab, lc_2d};
    for (int g = 0; g < 4; ++g) {
        if (!src[g]) continue;
        CK(cudaMemcpyAsync(h->staging, src[g], sizeof(float) * h->ncells, cudaMemcpyHostToDevice,
                           h->stream));
        CK(launch_scatter_aux(h->staging, h->aux[slot], 4 * g, h->ncells, h->stream));
        CK(cudaStreamSynchronize(h->stream));   // staging is reused
    }
    const gpat_mhd_config_t &c = h->cfg;
    CK(launch_calc_aux_gradients(h->aux[slot], h->prm.ndim, h->nxg, h->nyg, h->nzg, c.dx, c.dy,
                                 c.dz, h->stream, grad_spans(h)));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

namespace {
// Two consecutive FP32 arrays of every (ghost-padded) node, as
// read_magnetic_fluctuation / read_correlation_length read them
// (mhd_data_parallel.f90:306-497).
int read_pair(gpat_handle_t *h, const char *filename, std::vector<float> &a,
              std::vector<float> &b) {
    FILE *f = std::fopen(filename, "rb");
    if (!f) return fail(h, GPAT_ERR_IO, std::string("cannot open ") + filename);
    a.resize(h->ncells);
    b.resize(h->ncells);
    const size_t ga = std::fread(a.data(), sizeof(float), a.size(), f);
    const size_t gb = std::fread(b.data(), sizeof(float), b.size(), f);
    std::fclose(f);
    if (ga != a.size() || gb != b.size())
        return fail(h, GPAT_ERR_IO, std::string("short fluctuation file ") + filename);
    return GPAT_OK;
}
}  // namespace

int gpat_read_magnetic_fluctuation(gpat_handle_t *h, const char *filename, int var_flag) {
    if (!h || !filename) return GPAT_ERR_ARG;
    std::vector<float> a, b;
    int rc = read_pair(h, filename, a, b);
    if (rc) return rc;
    return gpat_set_fluctuations(h, var_flag, a.data(), b.data(), nullptr, nullptr);
}

int gpat_read_correlation_length(gpat_handle_t *h, const char *filename, int var_flag) {
    if (!h || !filename) return GPAT_ERR_ARG;
    std::vector<float> a, b;
    int rc = read_pair(h, filename, a, b);
    if (rc) return rc;
    return gpat_set_fluctuations(h, var_flag, nullptr, nullptr, a.data(), b.data());
}

int gpat_get_fluctuations(gpat_handle_t *h, int var_flag, float *aux) {
    if (!h || !aux) return GPAT_ERR_ARG;
    const int slot = var_flag == 0 ? 0 : 1;
    if (slot >= h->nslots || !h->aux[slot]) return fail(h, GPAT_ERR_STATE, "no fluctuation arrays");
    CK(cudaSetDevice(h->device));
    CK(cudaMemcpy(aux, h->aux[slot], 16 * sizeof(float) * h->ncells, cudaMemcpyDeviceToHost));
    return GPAT_OK;
}

int gpat_set_grid_positions(gpat_handle_t *h, const double *xpos, const double *ypos,
                            const double *zpos) {
    if (!h) return GPAT_ERR_ARG;
    if (!h->prm.nonuniform_grid)
        return fail(h, GPAT_ERR_STATE, "grid positions are set only when nonuniform_grid is on");
    const double *src[3] = {xpos, ypos, zpos};
    for (int ax = 0; ax < h->prm.ndim; ++ax) {
        if (!src[ax]) return fail(h, GPAT_ERR_ARG, "missing grid positions");
        const size_t n = h->gpos[ax].size();
        for (size_t i = 1; i < n; ++i)
            if (!(src[ax][i] > src[ax][i - 1]))
                return fail(h, GPAT_ERR_ARG, "grid positions must increase");
    }
    for (int ax = 0; ax < h->prm.ndim; ++ax)
        h->gpos[ax].assign(src[ax], src[ax] + h->gpos[ax].size());
    CK(cudaSetDevice(h->device));
    return upload_grid(h);
}

int gpat_read_grid_positions(gpat_handle_t *h, const char *dir_mhd_data) {
    if (!h || !dir_mhd_data) return GPAT_ERR_ARG;
    if (!h->prm.nonuniform_grid)
        return fail(h, GPAT_ERR_STATE, "grid positions are read only when nonuniform_grid is on");
    // read_global_grid_positions (mhd_data_parallel.f90:2087-2126): raw
    // doubles, xpos.dat, ypos.dat (2D and 3D), zpos.dat (3D).
    const char *names[3] = {"xpos.dat", "ypos.dat", "zpos.dat"};
    std::vector<double> v[3];
    for (int ax = 0; ax < h->prm.ndim; ++ax) {
        const std::string path = std::string(dir_mhd_data) + names[ax];
        FILE *f = std::fopen(path.c_str(), "rb");
        if (!f) return fail(h, GPAT_ERR_IO, "cannot open " + path);
        v[ax].resize(h->gpos[ax].size());
        const size_t got = std::fread(v[ax].data(), sizeof(double), v[ax].size(), f);
        std::fclose(f);
        if (got != v[ax].size()) return fail(h, GPAT_ERR_IO, "short grid file " + path);
    }
    return gpat_set_grid_positions(h, v[0].data(), h->prm.ndim > 1 ? v[1].data() : nullptr,
                                   h->prm.ndim == 3 ? v[2].data() : nullptr);
}

int gpat_get_grid_positions(gpat_handle_t *h, double *xpos, double *ypos, double *zpos) {
    if (!h) return GPAT_ERR_ARG;
    if (!h->grid) return fail(h, GPAT_ERR_STATE, "uniform Cartesian grid: no node positions kept");
    double *dst[3] = {xpos, ypos, zpos};
    for (int ax = 0; ax < h->prm.ndim; ++ax)
        if (dst[ax]) std::copy(h->gpos[ax].begin(), h->gpos[ax].end(), dst[ax]);
    return GPAT_OK;
}

namespace {
// "+x" ... "-z": sign and normal axis of a surface (surface_norm1/2).
bool parse_norm(const char *n, int &sign, int &axis) {
    if (!n || (n[0] != '+' && n[0] != '-') || n[1] < 'x' || n[1] > 'z' || n[2] != '\0')
        return false;
    sign = n[0] == '+' ? 1 : -1;
    axis = n[1] - 'x';
    return true;
}
}  // namespace

int gpat_init_acc_surface(gpat_handle_t *h, const char *norm1, const char *norm2,
                          int is_intersection) {
    if (!h) return GPAT_ERR_ARG;
    if (h->prm.ndim != 3) return fail(h, GPAT_ERR_UNSUPPORTED, "acceleration surfaces are 3D only");
    if (h->prm.precision != GPAT_PREC_FP64)
        return fail(h, GPAT_ERR_UNSUPPORTED, "acceleration surfaces need GPAT_PREC_FP64");
    if (h->surf_on) return fail(h, GPAT_ERR_STATE, "acceleration surfaces already set up");
    int sg[2], ax[2];
    if (!parse_norm(norm1, sg[0], ax[0]) || (norm2 && !parse_norm(norm2, sg[1], ax[1])))
        return fail(h, GPAT_ERR_ARG, "surface norms are +x, -x, +y, -y, +z or -z");
    if (!norm2) { sg[1] = sg[0]; ax[1] = ax[0]; }
    CK(cudaSetDevice(h->device));
    const int ng[3] = {h->nxg, h->nyg, h->nzg};
    for (int k = 0; k < (norm2 ? 2 : 1); ++k) {
        // (nyg, nzg) for x, (nxg, nzg) for y, (nxg, nyg) for z (:38-89)
        h->surf_ld[k] = (size_t)(ax[k] == 0 ? ng[1] : ng[0]);
        h->surf_n[k] = h->surf_ld[k] * (size_t)(ax[k] == 2 ? ng[1] : ng[2]);
        for (int t = 0; t < h->nslots; ++t) {
            CK(cudaMalloc(&h->dsurf[k][t], sizeof(double) * h->surf_n[k]));
            CK(cudaMemsetAsync(h->dsurf[k][t], 0, sizeof(double) * h->surf_n[k], h->stream));
        }
    }
    CK(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 2; ++k) { h->surf_sign[k] = sg[k]; h->surf_axis[k] = ax[k]; }
    h->surf_has2 = norm2 != nullptr;
    h->surf_inter = is_intersection != 0;
    h->surf_on = true;
    return GPAT_OK;
}

int gpat_set_acc_surface(gpat_handle_t *h, int var_flag, const double *surface1,
                         const double *surface2) {
    if (!h || !surface1) return GPAT_ERR_ARG;
    if (!h->surf_on) return fail(h, GPAT_ERR_STATE, "gpat_init_acc_surface first");
    if (h->surf_has2 && !surface2) return fail(h, GPAT_ERR_ARG, "surface 2 is missing");
    const int slot = var_flag == 0 ? 0 : 1;
    if (slot >= h->nslots) return fail(h, GPAT_ERR_STATE, "slot 1 needs time_interp = 1");
    CK(cudaSetDevice(h->device));
    const double *src[2] = {surface1, surface2};
    for (int k = 0; k < (h->surf_has2 ? 2 : 1); ++k)
        CK(cudaMemcpyAsync(h->dsurf[k][slot], src[k], sizeof(double) * h->surf_n[k],
                           cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

int gpat_read_acc_surface(gpat_handle_t *h, int var_flag, const char *filename1,
                          const char *filename2) {
    if (!h || !filename1) return GPAT_ERR_ARG;
    if (!h->surf_on) return fail(h, GPAT_ERR_STATE, "gpat_init_acc_surface first");
    const char *names[2] = {filename1, filename2};
    std::vector<double> v[2];
    for (int k = 0; k < (h->surf_has2 ? 2 : 1); ++k) {
        if (!names[k]) return fail(h, GPAT_ERR_ARG, "surface 2 file is missing");
        FILE *f = std::fopen(names[k], "rb");
        if (!f) return fail(h, GPAT_ERR_IO, std::string("cannot open ") + names[k]);
        v[k].resize(h->surf_n[k]);
        const size_t got = std::fread(v[k].data(), sizeof(double), v[k].size(), f);
        std::fclose(f);
        if (got != v[k].size())
            return fail(h, GPAT_ERR_IO, std::string("short surface file ") + names[k]);
    }
    return gpat_set_acc_surface(h, var_flag, v[0].data(), h->surf_has2 ? v[1].data() : nullptr);
}

int gpat_read_field_data(gpat_handle_t *h, const char *filename, int var_flag) {
    if (!h || !filename) return GPAT_ERR_ARG;
    FILE *f = std::fopen(filename, "rb");
    if (!f) return fail(h, GPAT_ERR_IO, std::string("cannot open ") + filename);
    std::vector<float> buf(8 * h->ncells);
    const size_t got = std::fread(buf.data(), sizeof(float), buf.size(), f);
    std::fclose(f);
    if (got != buf.size()) return fail(h, GPAT_ERR_IO, std::string("short field file ") + filename);
    return gpat_set_fields(h, var_flag, buf.data(), 8);
}

int gpat_calc_fields_gradients(gpat_handle_t *h, int var_flag) {
    if (!h) return GPAT_ERR_ARG;
    const int slot = var_flag == 0 ? 0 : 1;
    if (slot >= h->nslots || !h->fields_set[slot]) return fail(h, GPAT_ERR_STATE, "fields not set");
    CK(cudaSetDevice(h->device));
    const gpat_mhd_config_t &c = h->cfg;
    CK(launch_calc_fields_gradients(h->full[slot], h->prm.ndim, h->nxg, h->nyg, h->nzg, c.dx, c.dy,
                                    c.dz, h->stream, grad_spans(h)));
    CK(launch_pack_records(h->full[slot], h->rec[slot], h->prm.ndim, h->ncells, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->rec_ready[slot] = true;
    ++h->rec_gen[slot];
    return GPAT_OK;
}

int gpat_copy_fields(gpat_handle_t *h) {
    if (!h) return GPAT_ERR_ARG;
    if (h->nslots < 2) return fail(h, GPAT_ERR_STATE, "copy_fields needs time_interp = 1");
    CK(cudaSetDevice(h->device));
    const int R = (h->prm.ndim == 2) ? kRec2D : kRec3D;
    CK(cudaMemcpyAsync(h->full[0], h->full[1], 32 * sizeof(float) * h->ncells,
                       cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->rec[0], h->rec[1], (size_t)R * sizeof(float) * h->ncells,
                       cudaMemcpyDeviceToDevice, h->stream));
    if (h->aux[0] && h->aux[1])   // copy_magnetic_fluctuation / copy_correlation_length
        CK(cudaMemcpyAsync(h->aux[0], h->aux[1], 16 * sizeof(float) * h->ncells,
                           cudaMemcpyDeviceToDevice, h->stream));
    for (int k = 0; k < 2; ++k)   // copy_acc_surface
        if (h->dsurf[k][0] && h->dsurf[k][1])
            CK(cudaMemcpyAsync(h->dsurf[k][0], h->dsurf[k][1], sizeof(double) * h->surf_n[k],
                               cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->fields_set[0] = h->fields_set[1];
    h->rec_ready[0] = h->rec_ready[1];
    ++h->rec_gen[0];
    return GPAT_OK;
}

int gpat_get_fields(gpat_handle_t *h, int var_flag, float *farray) {
    if (!h || !farray) return GPAT_ERR_ARG;
    const int slot = var_flag == 0 ? 0 : 1;
    if (slot >= h->nslots) return fail(h, GPAT_ERR_STATE, "no farray2");
    CK(cudaSetDevice(h->device));
    CK(cudaMemcpyAsync(farray, h->full[slot], 32 * sizeof(float) * h->ncells,
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

// Field access for the large-quantity injection and cell counts: frame slot
// 0 with its gradients, and the exact box as the sampling domain.
static LargeArgs large_args(const gpat_handle_t *h, int quantity, double qmin) {
    const gpat_mhd_config_t &c = h->cfg;
    LargeArgs g{};
    g.quantity = quantity;
    g.qmin = qmin;
    g.dom[0] = c.xmin; g.dom[3] = c.xmin + (double)c.nx * c.dx;
    g.dom[1] = c.ymin; g.dom[4] = c.ymin + (double)c.ny * c.dy;
    g.dom[2] = c.zmin;
    g.dom[5] = (h->prm.ndim == 3) ? c.zmin + (double)c.nz * c.dz : c.zmax;
    g.full = h->full[0];
    g.aux = h->aux[0];
    g.nx = c.nx; g.ny = c.ny; g.nz = (h->prm.ndim == 3) ? c.nz : 1;
    g.nxg = h->nxg; g.nyg = h->nyg;
    g.dx = c.dx; g.dy = c.dy; g.dz = c.dz;
    g.gxmin = c.xmin; g.gymin = c.ymin; g.gzmin = c.zmin;
    g.spherical = h->prm.spherical_coord ? 1 : 0;
    g.nonuniform = h->prm.nonuniform_grid ? 1 : 0;
    g.xpos = h->dpos[0]; g.ypos = h->dpos[1]; g.zpos = h->dpos[2];
    g.nzg = h->nzg;
    return g;
}

// locate_shock_xpos on frame 1 into h->dshock (nyg * nzg rows).
static int locate_shock(gpat_handle_t *h) {
    if (!h->rec_ready[0]) return fail(h, GPAT_ERR_STATE, "fields and their gradients are not set");
    const int nrows = h->nyg * h->nzg;
    if (!h->dshock) {
        if (cudaMalloc(&h->dshock, sizeof(int32_t) * (size_t)nrows) != cudaSuccess) {
            cudaGetLastError();
            h->dshock = nullptr;
            return fail(h, GPAT_ERR_OOM, "shock table");
        }
    }
    CK(launch_locate_shock(h->full[0], h->nxg, nrows, h->dshock, h->stream));
    return GPAT_OK;
}

static int inject_common(gpat_handle_t *h, int mode, int64_t nptl, double xpos, double dt,
                         int dist_flag, double particle_v0, int ct_mhd, const double *box,
                         double power_index, const LargeArgs *lg = nullptr) {
    if (nptl < 0) return fail(h, GPAT_ERR_ARG, "nptl < 0");
    if (dist_flag < 0 || dist_flag > 2) return fail(h, GPAT_ERR_ARG, "dist_flag must be 0, 1 or 2");
    if (ct_mhd < 1 || (size_t)ct_mhd + 1 > h->tstamps.size())
        return fail(h, GPAT_ERR_ARG, "ct_mhd outside the time stamps");
    CK(cudaSetDevice(h->device));
    const int64_t room = h->cap - h->n;
    const int64_t count = std::min(nptl, room);
    InjectArgs a{};
    a.P = h->P[h->cur];
    a.base = h->n;
    a.count = count;
    a.tag0 = (int32_t)h->tag_max;
    a.mode = mode;
    a.dist_flag = dist_flag;
    a.ndim = h->prm.ndim;
    const gpat_mhd_config_t &c = h->cfg;
    if (mode == 0 || mode == 2) {
        for (int i = 0; i < 6; ++i) a.box[i] = box[i];
        if (mode == 2) a.lg = *lg;
    } else {
        a.box[0] = c.xmin; a.box[3] = c.xmin + (double)c.nx * c.dx;
        a.box[1] = c.ymin; a.box[4] = c.ymin + (double)c.ny * c.dy;
        a.box[2] = c.zmin;
        a.box[5] = (h->prm.ndim == 3) ? c.zmin + (double)c.nz * c.dz : c.zmax;
    }
    a.xpos = xpos;
    if (mode == 3) {
        a.shock_ix = h->dshock;
        a.nyg = h->nyg; a.nzg = h->nzg;
        a.gxmin = c.xmin; a.gymin = c.ymin; a.gzmin = c.zmin;
        a.dx = c.dx; a.dy = c.dy; a.dz = c.dz;
    }
    a.dt = dt;
    a.particle_v0 = particle_v0;
    a.t_frame = h->tstamps[ct_mhd - 1];
    a.dt_mhd = h->tstamps[ct_mhd] - h->tstamps[ct_mhd - 1];
    a.power_index = power_index;
    a.p0 = h->prm.p0; a.pmin = h->prm.pmin; a.pmax = h->prm.pmax;
    a.key0 = (uint32_t)h->prm.seed;
    a.key1 = (uint32_t)(h->prm.seed >> 32);
    CK(launch_inject(a, &h->dcnt->status, h->stream));
    CK(launch_track_injected(a.P, h->n, h->n + count, track_args(h), h->dcnt, h->stream));
    int rc = pull_counters(h);
    if (rc) return rc;
    h->n += count;
    if (count > 0) h->unsorted = true;
    h->tag_max += count;
    rc = check_status(h);
    if (rc) return rc;
    if (count < nptl) return fail(h, GPAT_ERR_CAPACITY, "nptl_max reached while injecting");
    return GPAT_OK;
}

int gpat_inject_particles_spatial_uniform(gpat_handle_t *h, int64_t nptl, double dt, int dist_flag,
                                          double particle_v0, int ct_mhd, const double part_box[6],
                                          double power_index) {
    if (!h || !part_box) return GPAT_ERR_ARG;
    return inject_common(h, 0, nptl, 0.0, dt, dist_flag, particle_v0, ct_mhd, part_box, power_index);
}

int gpat_inject_particles_at_x(gpat_handle_t *h, int64_t nptl, double xpos, double dt, int dist_flag,
                               double particle_v0, int ct_mhd, double power_index) {
    if (!h) return GPAT_ERR_ARG;
    return inject_common(h, 1, nptl, xpos, dt, dist_flag, particle_v0, ct_mhd, nullptr, power_index);
}

int gpat_locate_shock_xpos(gpat_handle_t *h, int32_t *shock_ix) {
    if (!h) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc = locate_shock(h);
    if (rc) return rc;
    if (shock_ix)
        CK(cudaMemcpyAsync(shock_ix, h->dshock, sizeof(int32_t) * (size_t)(h->nyg * h->nzg),
                           cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

int gpat_inject_particles_at_shock(gpat_handle_t *h, int64_t nptl, double dt, int dist_flag,
                                   double particle_v0, int ct_mhd, double power_index) {
    if (!h) return GPAT_ERR_ARG;
    if (h->prm.spherical_coord || h->prm.nonuniform_grid)
        return fail(h, GPAT_ERR_UNSUPPORTED, "shock injection needs a uniform Cartesian grid");
    CK(cudaSetDevice(h->device));
    const int rc = locate_shock(h);
    if (rc) return rc;
    return inject_common(h, 3, nptl, 0.0, dt, dist_flag, particle_v0, ct_mhd, nullptr, power_index);
}

int gpat_count_cells_large(gpat_handle_t *h, int quantity, double qmin, const double part_box[6],
                           int64_t *ncells) {
    if (!h || !part_box || !ncells) return GPAT_ERR_ARG;
    if (h->prm.ndim == 1)
        return fail(h, GPAT_ERR_UNSUPPORTED, "large-quantity injection is 2D and 3D only");
    if (quantity < GPAT_LARGE_JZ || quantity > GPAT_LARGE_DB2)
        return fail(h, GPAT_ERR_ARG, "quantity must be one of GPAT_LARGE_*");
    if (quantity == GPAT_LARGE_DB2 && !h->aux[0])
        return fail(h, GPAT_ERR_STATE, "db2 injection needs deltab_flag and the fluctuation arrays");
    if (!h->rec_ready[0]) return fail(h, GPAT_ERR_STATE, "fields and their gradients are not set");
    CK(cudaSetDevice(h->device));
    const LargeArgs g = large_args(h, quantity, qmin);
    CK(cudaMemsetAsync(&h->dcnt->ncells, 0, sizeof(unsigned long long), h->stream));
    CK(launch_count_large(g, h->prm.ndim, part_box, &h->dcnt->ncells, h->stream));
    int rc = pull_counters(h);
    if (rc) return rc;
    *ncells = (int64_t)h->hcnt.ncells;
    return GPAT_OK;
}

int gpat_inject_particles_at_large(gpat_handle_t *h, int quantity, int64_t nptl, double dt,
                                   int dist_flag, double particle_v0, int ct_mhd,
                                   int inject_same_nptl, double qmin, int64_t ncells_norm,
                                   const double part_box[6], double power_index,
                                   int64_t *ninjected) {
    if (!h || !part_box) return GPAT_ERR_ARG;
    if (h->prm.ndim == 1)
        return fail(h, GPAT_ERR_UNSUPPORTED, "large-quantity injection is 2D and 3D only");
    if (nptl < 0) return fail(h, GPAT_ERR_ARG, "nptl < 0");
    if (!inject_same_nptl && ncells_norm <= 0)
        return fail(h, GPAT_ERR_ARG, "ncells_norm must be > 0");
    int64_t ncells = 0;
    int rc = gpat_count_cells_large(h, quantity, qmin, part_box, &ncells);
    if (rc) return rc;
    // nptl * mpi_sub_size * (ncells / ncells_g or ncells_norm) on one rank;
    // 0 / 0 (no cell above qmin) injects nothing.
    int64_t n = 0;
    if (inject_same_nptl) n = ncells > 0 ? nptl : 0;
    else n = (int64_t)((double)nptl * ((double)ncells / (double)ncells_norm));
    if (ninjected) *ninjected = n;
    const LargeArgs g = large_args(h, quantity, qmin);
    return inject_common(h, 2, n, 0.0, dt, dist_flag, particle_v0, ct_mhd, part_box, power_index,
                         &g);
}

int gpat_put_particles(gpat_handle_t *h, const gpat_particles_t *src, int64_t n) {
    if (!h || !src || n < 0) return GPAT_ERR_ARG;
    if (n > h->cap) return fail(h, GPAT_ERR_CAPACITY, "more particles than nptl_max");
    CK(cudaSetDevice(h->device));
    const DevParticles &D = h->P[h->cur];
    const size_t c = (size_t)n;
    auto cp = [&](void *dst, const void *s, size_t bytes) -> cudaError_t {
        if (!bytes) return cudaSuccess;
        if (!s) return cudaErrorInvalidValue;
        return cudaMemcpyAsync(dst, s, bytes, cudaMemcpyHostToDevice, h->stream);
    };
    CK(cp(D.x, src->x, 8 * c)); CK(cp(D.y, src->y, 8 * c)); CK(cp(D.z, src->z, 8 * c));
    CK(cp(D.p, src->p, 8 * c)); CK(cp(D.v, src->v, 8 * c)); CK(cp(D.mu, src->mu, 8 * c));
    CK(cp(D.weight, src->weight, 8 * c)); CK(cp(D.t, src->t, 8 * c)); CK(cp(D.dt, src->dt, 8 * c));
    CK(cp(D.split_times, src->split_times, c)); CK(cp(D.count_flag, src->count_flag, c));
    CK(cp(D.origin, src->origin, 4 * c)); CK(cp(D.nsteps_tracked, src->nsteps_tracked, 4 * c));
    CK(cp(D.nsteps_pushed, src->nsteps_pushed, 4 * c));
    CK(cp(D.tag_injected, src->tag_injected, 4 * c));
    CK(cp(D.tag_splitted, src->tag_splitted, 4 * c));
    CK(cp(D.rng_ctr, src->rng_ctr, 4 * c));
    CK(cudaStreamSynchronize(h->stream));
    h->n = n;
    h->unsorted = true;
    // the injection counter moves past every tag received, so later
    // injections do not repeat a tag and per-tag tables (labels of learned
    // splitting) cover them
    int64_t top = -1, low = 0;
    for (int64_t i = 0; i < n; ++i) {
        top = std::max<int64_t>(top, src->tag_injected[i]);
        low = std::min<int64_t>(low, src->tag_splitted[i]);
    }
    h->tag_max = std::max<int64_t>(h->tag_max, top + 1);
    // weighted splitting hands out lineage ids past the most negative tag
    h->fresh_floor = std::max<unsigned long long>(h->fresh_floor, (unsigned long long)(-low));
    return GPAT_OK;
}

int gpat_get_particles(gpat_handle_t *h, gpat_particles_t *dst, int64_t capacity, int64_t *n) {
    if (!h || !dst || !n) return GPAT_ERR_ARG;
    *n = h->n;
    if (h->n > capacity) return fail(h, GPAT_ERR_CAPACITY, "destination too small");
    CK(cudaSetDevice(h->device));
    const DevParticles &S = h->P[h->cur];
    const size_t c = (size_t)h->n;
    auto cp = [&](void *d, const void *s, size_t bytes) -> cudaError_t {
        if (!bytes || !d) return cudaSuccess;   // NULL destination: field skipped
        return cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToHost, h->stream);
    };
    CK(cp(dst->x, S.x, 8 * c)); CK(cp(dst->y, S.y, 8 * c)); CK(cp(dst->z, S.z, 8 * c));
    CK(cp(dst->p, S.p, 8 * c)); CK(cp(dst->v, S.v, 8 * c)); CK(cp(dst->mu, S.mu, 8 * c));
    CK(cp(dst->weight, S.weight, 8 * c)); CK(cp(dst->t, S.t, 8 * c)); CK(cp(dst->dt, S.dt, 8 * c));
    CK(cp(dst->split_times, S.split_times, c)); CK(cp(dst->count_flag, S.count_flag, c));
    CK(cp(dst->origin, S.origin, 4 * c)); CK(cp(dst->nsteps_tracked, S.nsteps_tracked, 4 * c));
    CK(cp(dst->nsteps_pushed, S.nsteps_pushed, 4 * c));
    CK(cp(dst->tag_injected, S.tag_injected, 4 * c));
    CK(cp(dst->tag_splitted, S.tag_splitted, 4 * c));
    CK(cp(dst->rng_ctr, S.rng_ctr, 4 * c));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

int gpat_get_escaped_particles(gpat_handle_t *h, gpat_particles_t *dst, int64_t capacity,
                               int64_t *n) {
    if (!h || !dst || !n) return GPAT_ERR_ARG;
    *n = h->ne;
    if (h->ne > capacity) return fail(h, GPAT_ERR_CAPACITY, "destination too small");
    if (h->ne == 0) return GPAT_OK;
    CK(cudaSetDevice(h->device));
    const DevParticles &S = h->E;
    const size_t c = (size_t)h->ne;
    auto cp = [&](void *d, const void *s, size_t bytes) -> cudaError_t {
        if (!bytes || !d) return cudaSuccess;
        return cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToHost, h->stream);
    };
    CK(cp(dst->x, S.x, 8 * c)); CK(cp(dst->y, S.y, 8 * c)); CK(cp(dst->z, S.z, 8 * c));
    CK(cp(dst->p, S.p, 8 * c)); CK(cp(dst->v, S.v, 8 * c)); CK(cp(dst->mu, S.mu, 8 * c));
    CK(cp(dst->weight, S.weight, 8 * c)); CK(cp(dst->t, S.t, 8 * c)); CK(cp(dst->dt, S.dt, 8 * c));
    CK(cp(dst->split_times, S.split_times, c)); CK(cp(dst->count_flag, S.count_flag, c));
    CK(cp(dst->origin, S.origin, 4 * c)); CK(cp(dst->nsteps_tracked, S.nsteps_tracked, 4 * c));
    CK(cp(dst->nsteps_pushed, S.nsteps_pushed, 4 * c));
    CK(cp(dst->tag_injected, S.tag_injected, 4 * c));
    CK(cp(dst->tag_splitted, S.tag_splitted, 4 * c));
    CK(cp(dst->rng_ctr, S.rng_ctr, 4 * c));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

int gpat_set_mover_tiles(gpat_handle_t *h, int bx, int by, int bz, int hx, int hy, int hz,
                         int threads, int items) {
    if (!h) return GPAT_ERR_ARG;
    if (bx == 0) {
        h->tile_b[0] = h->tile_b[1] = h->tile_b[2] = 0;
        h->tile_h[0] = h->tile_h[1] = h->tile_h[2] = 0;
        return GPAT_OK;
    }
    if (h->prm.precision != GPAT_PREC_MIXED || h->prm.ndim < 2)
        return fail(h, GPAT_ERR_UNSUPPORTED, "field bricks need the split-precision 2D/3D mover");
    if (h->prm.ndim == 2) { bz = 1; hz = 0; }
    if (bx < 2 || by < 2 || (h->prm.ndim == 3 && bz < 2))
        return fail(h, GPAT_ERR_ARG, "bricks need at least 2 cells per axis");
    if (hx < 0 || hy < 0 || hz < 0 || hx > 64 || hy > 64 || hz > 64)
        return fail(h, GPAT_ERR_ARG, "halo cells must be in [0, 64]");
    if (threads == 0) threads = 512;
    if (threads != 256 && threads != 512) return fail(h, GPAT_ERR_ARG, "threads must be 256 or 512");
    if (items == 0) items = 4096;
    if (items < 32 || items > (1 << 24)) return fail(h, GPAT_ERR_ARG, "items out of range");
    // a brick larger than the grid is the grid; TMA boxes hold at most 256 nodes per axis
    bx = std::min(bx, h->nxg - 1);
    by = std::min(by, h->nyg - 1);
    if (h->prm.ndim == 3) bz = std::min(bz, h->nzg - 1);
    const int sx = bx + 2 * hx, sy = by + 2 * hy, sz = bz + 2 * hz;   // staged cells
    if (sx + 1 > 256 || sy + 1 > 256 || sz + 1 > 256)
        return fail(h, GPAT_ERR_ARG, "at most 255 staged cells per axis");
    int smem_max = 0;
    CK(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
    const size_t need = tile_smem_bytes(h->prm.ndim, sx, sy, sz, h->prm.time_interp, nullptr, nullptr);
    if (need + 1024 > (size_t)smem_max)
        return fail(h, GPAT_ERR_ARG, "staged records exceed the shared memory of one CTA (" +
                                         std::to_string(need) + " bytes)");
    if (bx != h->tile_b[0] || by != h->tile_b[1] || bz != h->tile_b[2]) h->binned_tiles = false;
    h->tile_b[0] = bx; h->tile_b[1] = by; h->tile_b[2] = bz;
    h->tile_h[0] = hx; h->tile_h[1] = hy; h->tile_h[2] = hz;
    h->tile_threads = threads;
    h->tile_items = items;
    return GPAT_OK;
}

int gpat_get_mover_tiles(const gpat_handle_t *h, int *out) {
    if (!h || !out) return GPAT_ERR_ARG;
    out[0] = h->tile_b[0]; out[1] = h->tile_b[1]; out[2] = h->tile_b[2];
    out[3] = h->tile_h[0]; out[4] = h->tile_h[1]; out[5] = h->tile_h[2];
    out[6] = h->tile_threads; out[7] = h->tile_items;
    return GPAT_OK;
}

int gpat_particle_mover(gpat_handle_t *h, int focused_transport, int nlgc, double kperp_kpara,
                        int nsteps_interval, int mhd_tframe, int num_fine_steps,
                        int dump_escaped_dist) {
    if (!h) return GPAT_ERR_ARG;
    // The escaped distribution is always accumulated; dump_escaped_dist also
    // keeps the escaped particles themselves (escaped_ptls).
    const bool keep_escaped = dump_escaped_dist != 0;
    const bool mixed = h->prm.precision == GPAT_PREC_MIXED;
    if (focused_transport && mixed)
        return fail(h, GPAT_ERR_UNSUPPORTED, "focused transport runs in FP64 precision");
    MoverArgs a;
    int rc = mover_args(h, mhd_tframe, nsteps_interval, num_fine_steps, a);
    if (rc) return rc;
    a.focused_transport = focused_transport ? 1 : 0;
    a.nlgc = nlgc ? 1 : 0;
    a.kperp_kpara = kperp_kpara;
    CK(cudaSetDevice(h->device));
    rc = ensure_scratch(h, h->n);
    if (rc) return rc;
    const bool learned = mixed && h->learn_on;
    const bool tiled = mixed && tiles_on(h) && !learned;
    if (mixed) {
        rc = ensure_pause(h);
        if (rc) return rc;
        a.pause = h->pause;
    }
    if (mixed && (h->unsorted || (tiled && !h->binned_tiles) || h->n_active != h->n)) {
        // New particles since the last binning (or a binning for another
        // brick shape): bin them before moving.
        rc = bin_particles(h, tiled);
        if (rc) return rc;
        a.P = h->P[h->cur];
        a.n = h->n;
    }
    const unsigned long long steps_before = h->hcnt.steps;
    double mover_ms = 0.0;
    int64_t launches = 0;
    if (tiled) {
        // Field bricks in shared memory: a particle pauses after bin_interval
        // pushes; one that walks out of its staged region on the way finishes
        // those pushes in the overflow kernel.  Between launches the set is
        // binned brick-major again (removal included).  Every launch pushes
        // each paused particle at least once, so the launches are bounded by
        // the push limit.
        const int bi = h->prm.bin_interval;
        a.chunk_pushes = bi == 0 ? 128u : (bi > 0 ? (uint32_t)bi : 0u);
        const MixedConsts k = make_mixed_consts(a);
        TileSched s{};
        const CellGrid g = cell_grid(h, true);
        s.bx = g.bx; s.by = g.by; s.bz = g.bz;
        s.hx = h->tile_h[0]; s.hy = h->tile_h[1]; s.hz = h->prm.ndim == 3 ? h->tile_h[2] : 0;
        s.nbx = g.nbx; s.nby = g.nby; s.nbz = g.nbz;
        s.nbricks = (long long)g.nbx * g.nby * g.nbz;
        s.cpb = g.bx * g.by * g.bz;
        s.items = h->tile_items;
        const int sx = s.bx + 2 * s.hx, sy = s.by + 2 * s.hy, sz = s.bz + 2 * s.hz;
        tile_smem_bytes(h->prm.ndim, sx, sy, sz, a.time_interp, &s.tile_bytes, &s.tile2_off);
        if (h->tile_ovf_cap < h->cap) {
            CK(cudaStreamSynchronize(h->stream));
            if (h->tile_ovf) CK(cudaFree(h->tile_ovf));
            h->tile_ovf = nullptr;
            h->tile_ovf_cap = 0;
            if (cudaMalloc(&h->tile_ovf, (size_t)h->cap * 12 + 256) != cudaSuccess) {
                cudaGetLastError();
                return fail(h, GPAT_ERR_OOM, "tile overflow list");
            }
            h->tile_ovf_cap = h->cap;
        }
        s.ovf_idx = static_cast<long long *>(h->tile_ovf);
        s.ovf_done = reinterpret_cast<unsigned int *>(s.ovf_idx + h->cap);
        s.ovf_count = reinterpret_cast<unsigned long long *>(
            (reinterpret_cast<uintptr_t>(s.ovf_done + h->cap) + 15) & ~(uintptr_t)15);
        if (h->tile_dev_n < s.nbricks + 2) {
            CK(cudaStreamSynchronize(h->stream));
            if (h->tile_dev) CK(cudaFree(h->tile_dev));
            h->tile_dev = nullptr;
            h->tile_dev_n = 0;
            if (cudaMalloc(&h->tile_dev, sizeof(long long) * (size_t)(s.nbricks + 2)) != cudaSuccess) {
                cudaGetLastError();
                return fail(h, GPAT_ERR_OOM, "tile work items");
            }
            h->tile_dev_n = s.nbricks + 2;
        }
        s.item_prefix = h->tile_dev;
        s.item_counter = reinterpret_cast<unsigned long long *>(h->tile_dev + s.nbricks + 1);
        s.nodes = (uint32_t)((sx + 1) * (sy + 1) * (h->prm.ndim == 3 ? sz + 1 : 1));
        // chunk-planar copies of the frames' records, rebuilt when the records changed
        const int R = (h->prm.ndim == 2) ? kRec2D : kRec3D;
        for (int slot = 0; slot < (a.time_interp ? 2 : 1); ++slot) {
            if (!h->planes[slot]) {
                if (cudaMalloc(&h->planes[slot], (size_t)R * sizeof(float) * h->ncells) !=
                    cudaSuccess) {
                    cudaGetLastError();
                    return fail(h, GPAT_ERR_OOM, "chunk-planar field records");
                }
                h->plane_gen[slot] = 0;
            }
            if (h->plane_gen[slot] != h->rec_gen[slot]) {
                CK(launch_planarize_records(h->rec[slot], h->planes[slot], h->prm.ndim, h->ncells,
                                            h->stream));
                h->plane_gen[slot] = h->rec_gen[slot];
            }
        }
        CUtensorMap tm1, tm2;
        CK(encode_brick_map(&tm1, h->planes[0], h->prm.ndim, h->nxg, h->nyg, h->nzg, sx, sy, sz));
        CK(encode_brick_map(&tm2, a.time_interp ? h->planes[1] : h->planes[0], h->prm.ndim, h->nxg,
                            h->nyg, h->nzg, sx, sy, sz));
        const int64_t max_launches = (int64_t)a.max_pushes + 4;
        for (;;) {
            CK(cudaMemsetAsync(&h->dcnt->nactive, 0, sizeof(unsigned long long), h->stream));
            CK(cudaMemsetAsync(s.ovf_count, 0, sizeof(unsigned long long), h->stream));
            a.P = h->P[h->cur];
            a.n = h->n_active;   // paused particles lead the array; finished ones trail
            s.incl = cell_sort_counts(h->sort_scratch, h->last_sort_bins);
            CK(cudaEventRecord(h->ev0, h->stream));
            CK(launch_mover_tile(a, k, s, tm1, tm2, h->tile_threads, h->sm_count, h->stream));
            CK(cudaEventRecord(h->ev1, h->stream));
            ++launches;
            if (keep_escaped) {
                rc = collect_escaped(h);
                if (rc) return rc;
            }
            rc = bin_particles(h, true, a.n);
            if (rc) return rc;
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
            mover_ms += ms;
            if (h->hcnt.status) break;   // reported below
            if (h->hcnt.nactive == 0) break;
            if (launches > max_launches)
                return fail(h, GPAT_ERR_DEVICE, "tile mover launches did not finish the interval");
        }
    } else if (mixed) {
        // Chunks of bin_interval pushes per particle; between chunks the set is
        // binned by cell again (and removal happens), so lanes of a warp keep
        // gathering neighbouring records while the particles spread out.
        const int bi = h->prm.bin_interval;
        a.chunk_pushes = bi == 0 ? 128u : (bi > 0 ? (uint32_t)bi : 0u);
        const MixedConsts k = make_mixed_consts(a);
        const int64_t max_chunks = (int64_t)a.max_pushes / (a.chunk_pushes ? a.chunk_pushes : 1) + 4;
        const unsigned long long split0 = h->hcnt.nsplit, kill0 = h->hcnt.nkilled;
        if (learned)
            CK(cudaMemsetAsync(h->learn_dev + 1, 0, 5 * sizeof(unsigned long long), h->stream));
        for (;;) {
            CK(cudaMemsetAsync(&h->dcnt->nactive, 0, sizeof(unsigned long long), h->stream));
            a.P = h->P[h->cur];
            a.n = h->n_active;   // paused particles lead the array; finished ones trail
            if (learned) {
                // children are appended after every particle of the set
                h->learn_host[0] = (unsigned long long)h->n;
                CK(cudaMemcpyAsync(h->learn_dev, h->learn_host, sizeof(unsigned long long),
                                   cudaMemcpyHostToDevice, h->stream));
                FusedLearn L = h->learn;
                L.cap = h->cap;
                L.count = h->learn_dev;
                L.zsum = h->learn_dev + 1;
                CK(cudaEventRecord(h->ev0, h->stream));
                CK(launch_mover_learned(a, k, L, h->stream));
                CK(cudaEventRecord(h->ev1, h->stream));
                CK(cudaMemcpyAsync(h->learn_host, h->learn_dev, 6 * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, h->stream));
                CK(cudaStreamSynchronize(h->stream));
                h->n = (int64_t)h->learn_host[0];
            } else {
                CK(cudaEventRecord(h->ev0, h->stream));
                CK(launch_mover_mixed(a, k, h->sm_count, h->stream));
                CK(cudaEventRecord(h->ev1, h->stream));
            }
            ++launches;
            if (keep_escaped) {
                rc = collect_escaped(h);
                if (rc) return rc;
            }
            rc = bin_particles(h, false, a.n);   // remove_particles as a binning by cell
            if (rc) return rc;
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
            mover_ms += ms;
            if (h->hcnt.nactive == 0) break;
            if (launches > max_chunks)
                return fail(h, GPAT_ERR_DEVICE, "mover chunks did not finish the interval");
        }
        if (learned) {
            h->learn_split = (int64_t)(h->hcnt.nsplit - split0);
            h->learn_killed = (int64_t)(h->hcnt.nkilled - kill0);
            h->nptl_split += h->learn_split;
        }
    } else {
        CK(cudaEventRecord(h->ev0, h->stream));
        CK(launch_mover_fp64(a, h->sm_count, h->stream));
        CK(cudaEventRecord(h->ev1, h->stream));
        launches = 1;
        if (keep_escaped) {
            rc = collect_escaped(h);
            if (rc) return rc;
        }
        // remove_particles (particle_module.f90:5365-5403), order-preserving.
        const int nxt = 1 - h->cur;
        CK(launch_remove_particles(h->P[h->cur], h->P[nxt], h->n, h->scratch, h->dcnt,
                                   escaped_hist(h), h->stream));
        rc = pull_counters(h);
        if (rc) return rc;
        h->cur = nxt;
        h->n = (int64_t)h->hcnt.nkept;
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
        mover_ms = ms;
    }
    h->last_mover_ms = mover_ms;
    h->last_mover_launches = launches;
    h->last_mover_steps = h->hcnt.steps - steps_before;
    return check_status(h);
}

int gpat_split_particle(gpat_handle_t *h, double split_ratio, double pmin_split, int nsteps_interval) {
    (void)nsteps_interval;
    if (!h) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    int rc = ensure_scratch(h, h->n);
    if (rc) return rc;
    const unsigned long long before = h->hcnt.nsplit;
    const TrackArgs trk = track_args(h);
    CK(launch_split_particles(h->P[h->cur], h->n, h->cap, split_ratio, pmin_split, h->prm.p0,
                              h->prm.pmax, h->scratch, h->dcnt, h->stream, &trk));
    rc = pull_counters(h);
    if (rc) return rc;
    const int64_t created = (int64_t)(h->hcnt.nsplit - before);
    const int64_t wanted = (int64_t)h->hcnt.nkept;
    h->n += created;
    if (created > 0) h->unsorted = true;
    h->nptl_split += created;
    if (created < wanted) return fail(h, GPAT_ERR_CAPACITY, "nptl_max reached while splitting");
    return GPAT_OK;
}

int gpat_calc_particle_distributions(gpat_handle_t *h, double *fglobal, uint64_t *counts) {
    if (!h) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    const int npp = h->prm.npp_global;
    CK(launch_histogram(h->P[h->cur], h->n, npp, h->prm.pmin, h->prm.pmax, h->dbins, h->stream));
    std::vector<unsigned long long> b(3 * (size_t)npp);
    CK(cudaMemcpyAsync(b.data(), h->dbins, sizeof(unsigned long long) * b.size(),
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < npp; ++i) {
        if (counts) counts[i] = b[3 * i];
        if (fglobal) fglobal[i] = fixed_to_double(b[3 * i + 1], b[3 * i + 2]);
    }
    return GPAT_OK;
}

static int local_args(gpat_handle_t *h, const gpat_local_dist_t *sp, LocalDistArgs &a) {
    if (!sp || sp->npbins < 1 || sp->nmu < 1 || sp->rx < 1 || sp->ry < 1 || sp->rz < 1 ||
        !(sp->pmin > 0.0) || !(sp->pmax > sp->pmin))
        return fail(h, GPAT_ERR_ARG, "bad local distribution parameters");
    const gpat_mhd_config_t &c = h->cfg;
    const int nz = h->prm.ndim == 3 ? c.nz : 1;
    // init_local_particle_distributions (diagnostics.f90:262-270) on one rank
    a.nrx = (c.nx + sp->rx - 1) / sp->rx;
    a.nry = (c.ny + sp->ry - 1) / sp->ry;
    a.nrz = (nz + sp->rz - 1) / sp->rz;
    a.dxd = c.lx / a.nrx;
    a.dyd = c.ly / a.nry;
    a.dzd = c.lz / a.nrz;
    a.xmin = c.xmin; a.ymin = c.ymin; a.zmin = c.zmin;
    a.pmin_log = std::log10(sp->pmin);
    a.dp_log = (std::log10(sp->pmax) - a.pmin_log) / sp->npbins;
    a.dmu = (double)(2.0f / (float)sp->nmu);   // 2.0 / nmu1 in single precision (:273)
    a.nmu = sp->nmu;
    a.npb = sp->npbins;
    a.ndim = h->prm.ndim;
    a.spherical = h->prm.spherical_coord ? 1 : 0;
    a.nonuniform = h->prm.nonuniform_grid ? 1 : 0;
    a.rx = sp->rx; a.ry = sp->ry; a.rz = sp->rz;
    a.nxg = h->nxg; a.nyg = h->nyg; a.nzg = h->nzg;
    a.xpos = h->dpos[0]; a.ypos = h->dpos[1]; a.zpos = h->dpos[2];
    return GPAT_OK;
}

int gpat_local_distribution_dims(gpat_handle_t *h, const gpat_local_dist_t *spec, int32_t dims[5]) {
    if (!h || !dims) return GPAT_ERR_ARG;
    LocalDistArgs a;
    const int rc = local_args(h, spec, a);
    if (rc) return rc;
    dims[0] = a.nmu; dims[1] = a.npb; dims[2] = a.nrx; dims[3] = a.nry; dims[4] = a.nrz;
    return GPAT_OK;
}

int gpat_calc_local_distribution(gpat_handle_t *h, const gpat_local_dist_t *spec, double *flocal,
                                 uint64_t *counts) {
    if (!h) return GPAT_ERR_ARG;
    LocalDistArgs a;
    int rc = local_args(h, spec, a);
    if (rc) return rc;
    const size_t nbins = (size_t)a.nmu * a.npb * a.nrx * a.nry * a.nrz;
    if (nbins > ((size_t)1 << 31)) return fail(h, GPAT_ERR_ARG, "local distribution too large");
    CK(cudaSetDevice(h->device));
    unsigned long long *bins = nullptr;
    std::vector<unsigned long long> b;
    try {
        b.resize(3 * nbins);
    } catch (const std::bad_alloc &) {
        return fail(h, GPAT_ERR_OOM, "local distribution does not fit in host memory");
    }
    CK(cudaMallocAsync((void **)&bins, sizeof(unsigned long long) * 3 * nbins, h->stream));
    cudaError_t e = launch_local_dist(h->P[h->cur], h->n, a, bins, nbins, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b.data(), bins, sizeof(unsigned long long) * b.size(),
                            cudaMemcpyDeviceToHost, h->stream);
    cudaFreeAsync(bins, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(h, GPAT_ERR_CUDA, cudaGetErrorString(e));
    for (size_t i = 0; i < nbins; ++i) {
        if (counts) counts[i] = b[3 * i];
        if (flocal) flocal[i] = fixed_to_double(b[3 * i + 1], b[3 * i + 2]);
    }
    return GPAT_OK;
}

int gpat_calc_escaped_distributions(gpat_handle_t *h, double *fescaped, uint64_t *counts) {
    if (!h) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    const size_t npp = (size_t)h->prm.npp_global;
    const size_t ncol = 2 * (size_t)h->prm.ndim;
    std::vector<unsigned long long> b(3 * 6 * npp);
    CK(cudaMemcpyAsync(b.data(), h->desc, sizeof(unsigned long long) * b.size(),
                       cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t f = 0; f < ncol; ++f)
        for (size_t ip = 0; ip < npp; ++ip) {
            const size_t k = f * npp + ip;
            if (counts) counts[k] = b[3 * k];
            if (fescaped) fescaped[k] = fixed_to_double(b[3 * k + 1], b[3 * k + 2]);
        }
    return GPAT_OK;
}

extern "C++" {
// Runs a (count, whi, wlo) binning into a temporary device buffer and
// unpacks it into counts / weights (either may be NULL).
template <class Launch>
static int run_bins(gpat_handle_t *h, size_t nbins, Launch launch, double *f, uint64_t *c) {
    if (nbins > ((size_t)1 << 31)) return fail(h, GPAT_ERR_ARG, "distribution too large");
    CK(cudaSetDevice(h->device));
    unsigned long long *bins = nullptr;
    std::vector<unsigned long long> b;
    try {
        b.resize(3 * nbins);
    } catch (const std::bad_alloc &) {
        return fail(h, GPAT_ERR_OOM, "distribution does not fit in host memory");
    }
    CK(cudaMallocAsync((void **)&bins, sizeof(unsigned long long) * 3 * nbins, h->stream));
    cudaError_t e = cudaMemsetAsync(bins, 0, sizeof(unsigned long long) * 3 * nbins, h->stream);
    if (e == cudaSuccess) e = launch(bins);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b.data(), bins, sizeof(unsigned long long) * b.size(),
                            cudaMemcpyDeviceToHost, h->stream);
    cudaFreeAsync(bins, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(h, GPAT_ERR_CUDA, cudaGetErrorString(e));
    for (size_t i = 0; i < nbins; ++i) {
        if (c) c[i] = b[3 * i];
        if (f) f[i] = fixed_to_double(b[3 * i + 1], b[3 * i + 2]);
    }
    return GPAT_OK;
}

static MuDistArgs mu_args(const gpat_handle_t *h, int nmu, int by_face) {
    MuDistArgs a;
    a.pmin = h->prm.pmin;
    a.pmax = h->prm.pmax;
    a.pmin_log = std::log10(h->prm.pmin);
    a.dp_log = (std::log10(h->prm.pmax) - a.pmin_log) / h->prm.npp_global;
    a.dmu = (double)(2.0f / (float)nmu);   // dmu = 2.0 / nmu_global (diagnostics.f90:206)
    a.npp = h->prm.npp_global;
    a.nmu = nmu;
    a.by_face = by_face;
    return a;
}
}  // extern "C++"

int gpat_calc_particle_distributions_mu(gpat_handle_t *h, int32_t nmu, double *fglobal,
                                        uint64_t *counts) {
    if (!h) return GPAT_ERR_ARG;
    if (nmu < 1) return fail(h, GPAT_ERR_ARG, "nmu must be >= 1");
    const MuDistArgs a = mu_args(h, nmu, 0);
    const size_t nbins = (size_t)nmu * (size_t)a.npp;
    return run_bins(h, nbins, [&](unsigned long long *bins) {
        return launch_mu_dist(h->P[h->cur], h->n, a, bins, nbins, h->stream);
    }, fglobal, counts);
}

int gpat_calc_escaped_distributions_mu(gpat_handle_t *h, int32_t nmu, double *fescaped,
                                       uint64_t *counts) {
    if (!h) return GPAT_ERR_ARG;
    if (nmu < 1) return fail(h, GPAT_ERR_ARG, "nmu must be >= 1");
    const MuDistArgs a = mu_args(h, nmu, 1);
    const size_t nbins = (size_t)nmu * (size_t)a.npp * 2 * (size_t)h->prm.ndim;
    return run_bins(h, nbins, [&](unsigned long long *bins) {
        return launch_mu_dist(h->E, h->ne, a, bins, nbins, h->stream);
    }, fescaped, counts);
}

int gpat_calc_local_escaped_distribution(gpat_handle_t *h, const gpat_local_dist_t *spec,
                                         double *fx, double *fy, double *fz, uint64_t *cx,
                                         uint64_t *cy, uint64_t *cz) {
    if (!h) return GPAT_ERR_ARG;
    LocalDistArgs a;
    int rc = local_args(h, spec, a);
    if (rc) return rc;
    const size_t mp = (size_t)a.nmu * (size_t)a.npb;
    const size_t nx = mp * a.nry * a.nrz * 2, ny = mp * a.nrx * a.nrz * 2;
    const size_t nz = mp * a.nrx * a.nry * 2;
    const size_t sizes[3] = {nx, h->prm.ndim > 1 ? ny : 0, h->prm.ndim > 2 ? nz : 0};
    double *f[3] = {fx, fy, fz};
    uint64_t *c[3] = {cx, cy, cz};
    for (int face = 0; face < 3; ++face) {
        if (!sizes[face] || (!f[face] && !c[face])) continue;
        rc = run_bins(h, sizes[face], [&](unsigned long long *bins) {
            unsigned long long *b[3] = {nullptr, nullptr, nullptr};
            b[face] = bins;
            return launch_local_escaped(h->E, h->ne, a, b[0], b[1], b[2], h->stream);
        }, f[face], c[face]);
        if (rc) return rc;
    }
    return GPAT_OK;
}

int gpat_get_pmax_global(gpat_handle_t *h, double *pmax) {
    if (!h || !pmax) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    CK(cudaMemsetAsync(&h->dcnt->pmax_bits, 0, sizeof(unsigned long long), h->stream));
    CK(launch_pmax(h->P[h->cur], h->n, &h->dcnt->pmax_bits, h->stream));
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, &h->dcnt->pmax_bits, sizeof bits, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::memcpy(pmax, &bits, sizeof bits);
    return GPAT_OK;
}

int gpat_free_particle_tracking(gpat_handle_t *h) {
    if (!h) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->stream));
    if (h->tmem) cudaFree(h->tmem);
    if (h->dtags) cudaFree(h->dtags);
    h->tmem = nullptr;
    h->dtags = nullptr;
    h->T = DevParticles{};
    h->trk_rows = h->trk_n = 0;
    h->trk_steps = 0;
    return GPAT_OK;
}

int gpat_init_particle_tracking(gpat_handle_t *h, const int32_t *tags, int32_t nrows,
                                int32_t nptl_tracking, int32_t nsteps_interval) {
    if (!h || !tags) return GPAT_ERR_ARG;
    if (nrows < 2 || nptl_tracking < 1 || nsteps_interval < 1)
        return fail(h, GPAT_ERR_ARG, "tags_tracking needs >= 2 rows, >= 1 column, nsteps_interval >= 1");
    if (nrows > 2 + 127)   // split_times is an int8
        return fail(h, GPAT_ERR_ARG, "tags_tracking has more split levels than split_times holds");
    if (h->prm.precision != GPAT_PREC_FP64)
        return fail(h, GPAT_ERR_UNSUPPORTED, "particle tracking runs in FP64 precision");
    // nsteps_tracking_max = ceiling((1.0 / dt_min_rel) / nsteps_interval) + 1
    const double steps = std::ceil((1.0 / h->prm.dt_min_rel) / (double)nsteps_interval);
    if (!(steps >= 0.0) || steps > 2.0e9)
        return fail(h, GPAT_ERR_ARG, "dt_min_rel gives no usable nsteps_tracking_max");
    int rc = gpat_free_particle_tracking(h);
    if (rc) return rc;
    const int64_t nsteps_max = (int64_t)steps + 1;
    const int64_t nrec = nsteps_max * (int64_t)nptl_tracking;
    if (nrec > ((int64_t)1 << 36))   // beyond any device, and particle_bytes stays exact
        return fail(h, GPAT_ERR_OOM, "particles_tracked does not fit on the device");
    if (cudaMalloc(&h->tmem, particle_bytes(nrec)) != cudaSuccess) {
        cudaGetLastError();
        h->tmem = nullptr;
        return fail(h, GPAT_ERR_OOM, "particles_tracked does not fit on the device");
    }
    const size_t tbytes = sizeof(int32_t) * (size_t)nrows * (size_t)nptl_tracking;
    if (cudaMalloc(&h->dtags, tbytes) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(h->tmem);
        h->tmem = nullptr;
        h->dtags = nullptr;
        return fail(h, GPAT_ERR_OOM, "tags_tracking does not fit on the device");
    }
    // reset_tracked_particles (:5880-5898): every record zero
    CK(cudaMemsetAsync(h->tmem, 0, particle_bytes(nrec), h->stream));
    CK(cudaMemcpyAsync(h->dtags, tags, tbytes, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(&h->dcnt->trk_dropped, 0, sizeof(unsigned long long), h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->T = carve(h->tmem, nrec);
    h->trk_rows = nrows;
    h->trk_n = nptl_tracking;
    h->trk_steps = nsteps_max;
    return GPAT_OK;
}

int gpat_read_particle_tracking(gpat_handle_t *h, const char *particle_tags_file,
                                int32_t nsteps_interval) {
    if (!h || !particle_tags_file) return GPAT_ERR_ARG;
    FILE *f = std::fopen(particle_tags_file, "rb");
    if (!f) return fail(h, GPAT_ERR_IO, std::string("cannot open ") + particle_tags_file);
    int32_t dims[2] = {0, 0};
    if (std::fread(dims, sizeof(int32_t), 2, f) != 2 || dims[0] < 2 || dims[0] > 2 + 127 ||
        dims[1] < 1) {
        std::fclose(f);
        return fail(h, GPAT_ERR_IO, "tags file: bad dimensions");
    }
    std::vector<int32_t> tags;
    try {
        tags.resize((size_t)dims[0] * (size_t)dims[1]);
    } catch (const std::bad_alloc &) {
        std::fclose(f);
        return fail(h, GPAT_ERR_OOM, "tags file: table does not fit in host memory");
    }
    const size_t got = std::fread(tags.data(), sizeof(int32_t), tags.size(), f);
    std::fclose(f);
    if (got != tags.size()) return fail(h, GPAT_ERR_IO, "tags file: short read");
    return gpat_init_particle_tracking(h, tags.data(), dims[0], dims[1], nsteps_interval);
}

int gpat_tracking_dims(gpat_handle_t *h, int64_t *nsteps_tracking_max, int32_t *nptl_tracking,
                       int64_t *dropped) {
    if (!h) return GPAT_ERR_ARG;
    if (!h->dtags) return fail(h, GPAT_ERR_STATE, "particle tracking is not initialised");
    if (nsteps_tracking_max) *nsteps_tracking_max = h->trk_steps;
    if (nptl_tracking) *nptl_tracking = h->trk_n;
    if (dropped) {
        CK(cudaSetDevice(h->device));
        int rc = pull_counters(h);
        if (rc) return rc;
        *dropped = (int64_t)h->hcnt.trk_dropped;
    }
    return GPAT_OK;
}

int gpat_get_tracked_particles(gpat_handle_t *h, gpat_particles_t *dst) {
    if (!h || !dst) return GPAT_ERR_ARG;
    if (!h->dtags) return fail(h, GPAT_ERR_STATE, "particle tracking is not initialised");
    CK(cudaSetDevice(h->device));
    // sync_tracked_particles (:5994-6030) compacts the records in place
    CK(launch_sync_tracked(track_args(h), h->stream));
    const DevParticles &S = h->T;
    const size_t c = (size_t)(h->trk_steps * (int64_t)h->trk_n);
    auto cp = [&](void *d, const void *s, size_t bytes) -> cudaError_t {
        if (!bytes || !d) return cudaSuccess;   // NULL destination: field skipped
        return cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToHost, h->stream);
    };
    CK(cp(dst->x, S.x, 8 * c)); CK(cp(dst->y, S.y, 8 * c)); CK(cp(dst->z, S.z, 8 * c));
    CK(cp(dst->p, S.p, 8 * c)); CK(cp(dst->v, S.v, 8 * c)); CK(cp(dst->mu, S.mu, 8 * c));
    CK(cp(dst->weight, S.weight, 8 * c)); CK(cp(dst->t, S.t, 8 * c)); CK(cp(dst->dt, S.dt, 8 * c));
    CK(cp(dst->split_times, S.split_times, c)); CK(cp(dst->count_flag, S.count_flag, c));
    CK(cp(dst->origin, S.origin, 4 * c)); CK(cp(dst->nsteps_tracked, S.nsteps_tracked, 4 * c));
    CK(cp(dst->nsteps_pushed, S.nsteps_pushed, 4 * c));
    CK(cp(dst->tag_injected, S.tag_injected, 4 * c));
    CK(cp(dst->tag_splitted, S.tag_splitted, 4 * c));
    CK(cp(dst->rng_ctr, S.rng_ctr, 4 * c));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

int gpat_reset_escaped_particles(gpat_handle_t *h) {
    if (!h) return GPAT_ERR_ARG;
    h->ne = 0;   // nptl_escaped = 0 (diagnostics.f90:2227-2246)
    CK(cudaSetDevice(h->device));
    CK(cudaMemsetAsync(h->desc, 0, sizeof(unsigned long long) * 3 * 6 * (size_t)h->prm.npp_global,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

int gpat_pbins_edges(gpat_handle_t *h, double *edges) {
    if (!h || !edges) return GPAT_ERR_ARG;
    const double lo = std::log10(h->prm.pmin), hi = std::log10(h->prm.pmax);
    const double d = (hi - lo) / h->prm.npp_global;
    for (int i = 0; i <= h->prm.npp_global; ++i) edges[i] = std::pow(10.0, lo + i * d);
    return GPAT_OK;
}

int gpat_quick_check(gpat_handle_t *h, double out[8]) {
    if (!h || !out) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    DevCounters z{};
    z.dt_min = 1.0;
    z.dt_max = 0.0;
    const size_t off = offsetof(DevCounters, wsum_hi);
    const size_t len = offsetof(DevCounters, status) - off;
    CK(cudaMemcpyAsync(reinterpret_cast<char *>(h->dcnt) + off, reinterpret_cast<char *>(&z) + off,
                       len, cudaMemcpyHostToDevice, h->stream));
    CK(launch_quick_check(h->P[h->cur], h->n, h->dcnt, h->stream));
    int rc = pull_counters(h);
    if (rc) return rc;
    const DevCounters &c = h->hcnt;
    out[0] = (double)h->n;
    out[1] = (double)h->nptl_split;
    out[2] = fixed_to_double(c.wsum_hi, c.wsum_lo);
    out[3] = fixed_to_double(c.leak_hi, c.leak_lo);
    out[4] = fixed_to_double(c.negp_hi, c.negp_lo);
    out[5] = c.dt_min;
    out[6] = c.dt_max;
    out[7] = h->n > 0 ? fixed_to_double(c.dtsum_hi, c.dtsum_lo) / (double)h->n : 0.0;
    return GPAT_OK;
}

int gpat_get_counters(gpat_handle_t *h, gpat_counters_t *out) {
    if (!h || !out) return GPAT_ERR_ARG;
    int rc = pull_counters(h);
    if (rc) return rc;
    const DevCounters &c = h->hcnt;
    out->nptl_current = h->n;
    out->nptl_split = h->nptl_split;
    out->nptl_escaped = (int64_t)c.nescaped;
    out->tag_max = h->tag_max;
    out->leak_hi = c.leak_hi; out->leak_lo = c.leak_lo;
    out->leak_negp_hi = c.negp_hi; out->leak_negp_lo = c.negp_lo;
    out->leak = fixed_to_double(c.leak_hi, c.leak_lo);
    out->leak_negp = fixed_to_double(c.negp_hi, c.negp_lo);
    out->steps = c.steps;
    out->last_mover_ms = h->last_mover_ms;
    out->last_mover_steps = h->last_mover_steps;
    out->last_mover_launches = h->last_mover_launches;
    return GPAT_OK;
}

int gpat_set_counters(gpat_handle_t *h, const gpat_counters_t *in) {
    if (!h || !in) return GPAT_ERR_ARG;
    int rc = pull_counters(h);
    if (rc) return rc;
    h->nptl_split = in->nptl_split;
    h->tag_max = in->tag_max;
    h->hcnt.leak_hi = in->leak_hi; h->hcnt.leak_lo = in->leak_lo;
    h->hcnt.negp_hi = in->leak_negp_hi; h->hcnt.negp_lo = in->leak_negp_lo;
    h->hcnt.nescaped = (unsigned long long)in->nptl_escaped;
    h->hcnt.steps = in->steps;
    CK(cudaMemcpyAsync(h->dcnt, &h->hcnt, sizeof(DevCounters), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return GPAT_OK;
}

void *gpat_stream(gpat_handle_t *h) { return h ? (void *)h->stream : nullptr; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched runs: one persistent mover launch per chunk for all runs, the
// chunk (mover + every run's binning) replayed as a CUDA graph.
// ---------------------------------------------------------------------------
struct gpat_batch {
    std::vector<gpat_handle_t *> runs;
    int device = 0, sm_count = 0, ndim = 2;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    unsigned long long *dev = nullptr;     // run_n[nruns], tile_counter, nactive_total
    long long *tile_prefix = nullptr;      // nruns + 1
    unsigned long long *host_ull = nullptr;   // pinned: run_n readback and nactive
    std::vector<BatchRun> desc;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    int graph_key[3] = {-1, -1, -1};       // nlgc, minb, grab of the captured graphs
    std::vector<void *> graph_scratch;     // each run's binning scratch in the graphs
    gpat_batch_tuning_t tuning{};
    std::string err;
    double last_ms = 0.0;
    uint64_t last_steps = 0;
    int64_t last_graph_launches = 0;
};

namespace {

int bfail(gpat_batch_t *b, int code, const std::string &msg) {
    if (b) b->err = msg;
    return code;
}

#define BCK(call)                                                                     \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return bfail(b, GPAT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

unsigned long long *run_n_dev(gpat_batch_t *b) { return b->dev; }
unsigned long long *tile_counter_dev(gpat_batch_t *b) { return b->dev + b->runs.size(); }
unsigned long long *nactive_dev(gpat_batch_t *b) { return b->dev + b->runs.size() + 1; }

void destroy_graphs(gpat_batch_t *b) {
    for (auto &e : b->exec) {
        if (e) cudaGraphExecDestroy(e);
        e = nullptr;
    }
    b->graph_key[0] = b->graph_key[1] = b->graph_key[2] = -1;
}

// Captures the chunk graph for both buffer parities: scheduler prefix, the
// persistent batched mover, and each run's binning (removal included) from
// buffer `parity` into the other one.
int capture_graphs(gpat_batch_t *b, int nlgc, int minb, int grab) {
    destroy_graphs(b);
    const int nr = (int)b->runs.size();
    for (int parity = 0; parity < 2; ++parity) {
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = launch_batch_prefix(nr, run_n_dev(b), b->tile_prefix, tile_counter_dev(b),
                                            nactive_dev(b), b->stream);
        if (e == cudaSuccess)
            e = launch_mover_mixed_batch(b->ndim, nlgc != 0, minb, parity, nr, b->sm_count, grab,
                                         b->tile_prefix, run_n_dev(b), tile_counter_dev(b),
                                         nactive_dev(b), b->stream);
        for (int r = 0; r < nr && e == cudaSuccess; ++r) {
            gpat_handle_t *h = b->runs[r];
            e = launch_cell_sort_dev(h->P[parity], h->P[1 - parity], run_n_dev(b) + r, h->cap,
                                     cell_grid(h), h->sort_scratch, h->dcnt, escaped_hist(h),
                                     b->stream);
        }
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess || ee != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return bfail(b, GPAT_ERR_CUDA, std::string("batch graph capture: ") +
                                               cudaGetErrorString(e != cudaSuccess ? e : ee));
        }
        const cudaError_t ie = cudaGraphInstantiate(&b->exec[parity], g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess)
            return bfail(b, GPAT_ERR_CUDA, std::string("cudaGraphInstantiate: ") +
                                               cudaGetErrorString(ie));
    }
    b->graph_key[0] = nlgc;
    b->graph_key[1] = minb;
    b->graph_key[2] = grab;
    b->graph_scratch.clear();
    for (gpat_handle_t *h : b->runs) b->graph_scratch.push_back(h->sort_scratch);
    return GPAT_OK;
}

// Brings every run to binned particles in buffer 0, builds and uploads the
// run table and the device particle counts.
int batch_prepare(gpat_batch_t *b, const int *tframes, int nlgc, double kperp_kpara,
                  int nsteps_interval, int num_fine_steps) {
    const int nr = (int)b->runs.size();
    b->desc.resize(nr);
    for (int r = 0; r < nr; ++r) {
        gpat_handle_t *h = b->runs[r];
        MoverArgs a;
        int rc = mover_args(h, tframes[r], nsteps_interval, num_fine_steps, a);
        if (rc) return bfail(b, rc, "run " + std::to_string(r) + ": " + h->err);
        a.nlgc = nlgc ? 1 : 0;
        a.kperp_kpara = kperp_kpara;
        const int bi = h->prm.bin_interval;
        a.chunk_pushes = bi == 0 ? 128u : (bi > 0 ? (uint32_t)bi : 0u);
        if (b->tuning.chunk_pushes > 0) a.chunk_pushes = (uint32_t)b->tuning.chunk_pushes;
        for (int k = 0; k < 2 && (h->unsorted || h->cur != 0); ++k) {
            rc = bin_particles(h);
            if (rc) return bfail(b, rc, "run " + std::to_string(r) + ": " + h->err);
        }
        if (h->cur != 0) return bfail(b, GPAT_ERR_STATE, "run could not be brought to buffer 0");
        if (cudaStreamSynchronize(h->stream) != cudaSuccess)
            return bfail(b, GPAT_ERR_CUDA, "run stream synchronize failed");
        BatchRun &d = b->desc[r];
        d.a = mixed_run_args(a);
        d.k = make_mixed_consts(a);
        d.P[0] = h->P[0];
        d.P[1] = h->P[1];
        b->host_ull[r] = (unsigned long long)h->n;
    }
    BCK(upload_batch_runs(b->desc.data(), nr, b->stream));
    BCK(cudaMemcpyAsync(run_n_dev(b), b->host_ull, sizeof(unsigned long long) * (size_t)nr,
                        cudaMemcpyHostToDevice, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    return GPAT_OK;
}

// Replays chunk graphs until no particle paused; returns the final parity.
int batch_run_chunks(gpat_batch_t *b, int max_chunks, int *parity_out, int64_t *launches) {
    const size_t nr = b->runs.size();
    int parity = 0;
    *launches = 0;
    for (;;) {
        BCK(cudaGraphLaunch(b->exec[parity], b->stream));
        ++*launches;
        parity ^= 1;
        BCK(cudaMemcpyAsync(b->host_ull + nr, nactive_dev(b), sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, b->stream));
        BCK(cudaStreamSynchronize(b->stream));
        if (b->host_ull[nr] == 0 || (max_chunks > 0 && *launches >= max_chunks)) break;
        if (*launches > 1000000) return bfail(b, GPAT_ERR_DEVICE, "batch chunks did not finish");
    }
    *parity_out = parity;
    return GPAT_OK;
}

// Reads the runs' counts and counters back into their handles.
int batch_finish(gpat_batch_t *b, int parity, uint64_t *steps_total) {
    const size_t nr = b->runs.size();
    BCK(cudaMemcpyAsync(b->host_ull, run_n_dev(b), sizeof(unsigned long long) * nr,
                        cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    uint64_t total = 0;
    int first_err = GPAT_OK;
    for (size_t r = 0; r < nr; ++r) {
        gpat_handle_t *h = b->runs[r];
        const unsigned long long before = h->hcnt.steps;
        int rc = pull_counters(h);
        if (rc) return bfail(b, rc, h->err);
        h->n = (int64_t)b->host_ull[r];
        h->cur = parity;
        h->unsorted = false;
        h->last_mover_steps = h->hcnt.steps - before;
        total += h->last_mover_steps;
        rc = check_status(h);
        if (rc && first_err == GPAT_OK) {
            first_err = rc;
            b->err = "run " + std::to_string(r) + ": " + h->err;
        }
    }
    *steps_total = total;
    return first_err;
}

}  // namespace

int gpat_batch_create(gpat_handle_t *const *runs, int nruns, gpat_batch_t **out) {
    if (!runs || !out || nruns < 1 || nruns > kMaxBatchRuns) return GPAT_ERR_ARG;
    *out = nullptr;
    const gpat_handle_t *h0 = runs[0];
    for (int r = 0; r < nruns; ++r) {
        const gpat_handle_t *h = runs[r];
        if (!h) return GPAT_ERR_ARG;
        if (h->prm.precision != GPAT_PREC_MIXED || h->device != h0->device ||
            h->prm.ndim != h0->prm.ndim)
            return GPAT_ERR_UNSUPPORTED;
        for (int q = 0; q < r; ++q)
            if (runs[q] == h) return GPAT_ERR_ARG;
    }
    gpat_batch_t *b = new gpat_batch_t;
    b->runs.assign(runs, runs + nruns);
    b->device = h0->device;
    b->sm_count = h0->sm_count;
    b->ndim = h0->prm.ndim;
    int variants[4];
    batch_minb_variants(b->ndim, variants);
    b->tuning.minb = b->ndim == 2 ? 6 : 5;   // the single-run kernel's register target
    b->tuning.grab = 1;
    cudaSetDevice(b->device);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaMalloc(&b->dev, sizeof(unsigned long long) * ((size_t)nruns + 2)) != cudaSuccess ||
        cudaMalloc(&b->tile_prefix, sizeof(long long) * ((size_t)nruns + 1)) != cudaSuccess ||
        cudaMallocHost(&b->host_ull, sizeof(unsigned long long) * ((size_t)nruns + 2)) !=
            cudaSuccess) {
        gpat_batch_destroy(b);
        return GPAT_ERR_OOM;
    }
    *out = b;
    return GPAT_OK;
}

int gpat_batch_destroy(gpat_batch_t *b) {
    if (!b) return GPAT_ERR_ARG;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    destroy_graphs(b);
    if (b->dev) cudaFree(b->dev);
    if (b->tile_prefix) cudaFree(b->tile_prefix);
    if (b->host_ull) cudaFreeHost(b->host_ull);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return GPAT_OK;
}

const char *gpat_batch_last_error(const gpat_batch_t *b) { return b ? b->err.c_str() : "null batch"; }

int gpat_batch_particle_mover(gpat_batch_t *b, const int *mhd_tframe, int nlgc, double kperp_kpara,
                              int nsteps_interval, int num_fine_steps) {
    if (!b || !mhd_tframe) return GPAT_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    int rc = batch_prepare(b, mhd_tframe, nlgc, kperp_kpara, nsteps_interval, num_fine_steps);
    if (rc) return rc;
    bool same_scratch = b->graph_scratch.size() == b->runs.size();
    for (size_t r = 0; same_scratch && r < b->runs.size(); ++r)
        same_scratch = b->graph_scratch[r] == b->runs[r]->sort_scratch;
    if (!b->exec[0] || b->graph_key[0] != (nlgc ? 1 : 0) || b->graph_key[1] != b->tuning.minb ||
        b->graph_key[2] != b->tuning.grab || !same_scratch) {
        rc = capture_graphs(b, nlgc ? 1 : 0, b->tuning.minb, b->tuning.grab);
        if (rc) return rc;
    }
    BCK(cudaEventRecord(b->ev0, b->stream));
    int parity = 0;
    int64_t launches = 0;
    rc = batch_run_chunks(b, 0, &parity, &launches);
    if (rc) return rc;
    BCK(cudaEventRecord(b->ev1, b->stream));
    BCK(cudaEventSynchronize(b->ev1));
    float ms = 0.0f;
    BCK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
    b->last_ms = ms;
    b->last_graph_launches = launches;
    return batch_finish(b, parity, &b->last_steps);
}

int gpat_batch_autotune(gpat_batch_t *b, const int *mhd_tframe, int nlgc, double kperp_kpara,
                        int nsteps_interval, int num_fine_steps, gpat_batch_tuning_t *best) {
    if (!b || !mhd_tframe) return GPAT_ERR_ARG;
    BCK(cudaSetDevice(b->device));
    int rc = batch_prepare(b, mhd_tframe, nlgc, kperp_kpara, nsteps_interval, num_fine_steps);
    if (rc) return rc;
    // Snapshot of every run's particles (buffer 0), counters and escaped
    // distribution: each trial moves one chunk from the same state.
    const size_t nr = b->runs.size();
    std::vector<void *> snap(nr, nullptr);
    std::vector<DevCounters> hc(nr);
    std::vector<int64_t> n0(nr);
    auto release = [&]() {
        for (void *p : snap)
            if (p) cudaFree(p);
    };
    for (size_t r = 0; r < nr; ++r) {
        gpat_handle_t *h = b->runs[r];
        const size_t bytes = particle_bytes(h->cap) + sizeof(DevCounters) +
                             sizeof(unsigned long long) * 3 * 6 * (size_t)h->prm.npp_global;
        if (cudaMalloc(&snap[r], bytes) != cudaSuccess) { release(); return bfail(b, GPAT_ERR_OOM, "autotune snapshot"); }
        char *q = static_cast<char *>(snap[r]);
        BCK(cudaMemcpyAsync(q, h->pmem[0], particle_bytes(h->cap), cudaMemcpyDeviceToDevice, b->stream));
        BCK(cudaMemcpyAsync(q + particle_bytes(h->cap), h->dcnt, sizeof(DevCounters),
                            cudaMemcpyDeviceToDevice, b->stream));
        BCK(cudaMemcpyAsync(q + particle_bytes(h->cap) + sizeof(DevCounters), h->desc,
                            sizeof(unsigned long long) * 3 * 6 * (size_t)h->prm.npp_global,
                            cudaMemcpyDeviceToDevice, b->stream));
        hc[r] = h->hcnt;
        n0[r] = h->n;
    }
    int variants[4];
    const int nv = batch_minb_variants(b->ndim, variants);
    const int grabs[2] = {1, 4};
    const int chunks[3] = {64, 128, 256};
    gpat_batch_tuning_t top{};
    top.pushes_per_s = -1.0;
    const int def_minb = b->ndim == 2 ? 6 : 5;
    const int bi0 = b->runs[0]->prm.bin_interval;
    const int def_chunk = bi0 == 0 ? 128 : (bi0 > 0 ? bi0 : 0);
    double def_rate = 0.0;
    for (int ci = 0; ci < 3; ++ci) {
        for (size_t r = 0; r < nr; ++r) b->desc[r].a.chunk_pushes = (uint32_t)chunks[ci];
        BCK(upload_batch_runs(b->desc.data(), (int)nr, b->stream));
    for (int v = 0; v < nv; ++v)
        for (int gi = 0; gi < 2; ++gi) {
            rc = capture_graphs(b, nlgc ? 1 : 0, variants[v], grabs[gi]);
            if (rc) { release(); return rc; }
            // counts back to the snapshot's
            for (size_t r = 0; r < nr; ++r) b->host_ull[r] = (unsigned long long)n0[r];
            BCK(cudaMemcpyAsync(run_n_dev(b), b->host_ull, sizeof(unsigned long long) * nr,
                                cudaMemcpyHostToDevice, b->stream));
            BCK(cudaMemsetAsync(b->dev + nr, 0, 2 * sizeof(unsigned long long), b->stream));
            std::vector<unsigned long long> before(nr);
            for (size_t r = 0; r < nr; ++r) before[r] = hc[r].steps;
            BCK(cudaEventRecord(b->ev0, b->stream));
            int parity = 0;
            int64_t launches = 0;
            rc = batch_run_chunks(b, 1, &parity, &launches);
            if (rc) { release(); return rc; }
            BCK(cudaEventRecord(b->ev1, b->stream));
            BCK(cudaEventSynchronize(b->ev1));
            float ms = 0.0f;
            BCK(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
            uint64_t pushes = 0;
            for (size_t r = 0; r < nr; ++r) {
                gpat_handle_t *h = b->runs[r];
                DevCounters c;
                BCK(cudaMemcpy(&c, h->dcnt, sizeof c, cudaMemcpyDeviceToHost));
                pushes += c.steps - before[r];
            }
            const double rate = ms > 0.0f ? (double)pushes / (ms * 1e-3) : 0.0;
            if (variants[v] == def_minb && grabs[gi] == 1 && chunks[ci] == def_chunk)
                def_rate = rate;
            if (rate > top.pushes_per_s) {
                top.minb = variants[v];
                top.grab = grabs[gi];
                top.pushes_per_s = rate;
                top.chunk_pushes = chunks[ci];
            }
            // restore the snapshot
            for (size_t r = 0; r < nr; ++r) {
                gpat_handle_t *h = b->runs[r];
                char *q = static_cast<char *>(snap[r]);
                BCK(cudaMemcpyAsync(h->pmem[0], q, particle_bytes(h->cap), cudaMemcpyDeviceToDevice,
                                    b->stream));
                BCK(cudaMemcpyAsync(h->dcnt, q + particle_bytes(h->cap), sizeof(DevCounters),
                                    cudaMemcpyDeviceToDevice, b->stream));
                BCK(cudaMemcpyAsync(h->desc, q + particle_bytes(h->cap) + sizeof(DevCounters),
                                    sizeof(unsigned long long) * 3 * 6 * (size_t)h->prm.npp_global,
                                    cudaMemcpyDeviceToDevice, b->stream));
            }
            BCK(cudaStreamSynchronize(b->stream));
        }
    }
    release();
    for (size_t r = 0; r < nr; ++r) {
        gpat_handle_t *h = b->runs[r];
        h->hcnt = hc[r];
        h->n = n0[r];
        h->cur = 0;
        h->unsorted = false;
    }
    top.default_pushes_per_s = def_rate;
    b->tuning = top;
    if (best) *best = top;
    return GPAT_OK;
}

int gpat_batch_get_tuning(const gpat_batch_t *b, gpat_batch_tuning_t *t) {
    if (!b || !t) return GPAT_ERR_ARG;
    *t = b->tuning;
    return GPAT_OK;
}

int gpat_batch_set_tuning(gpat_batch_t *b, const gpat_batch_tuning_t *t) {
    if (!b || !t) return GPAT_ERR_ARG;
    int variants[4];
    const int nv = batch_minb_variants(b->ndim, variants);
    bool ok = false;
    for (int v = 0; v < nv; ++v) ok = ok || variants[v] == t->minb;
    if (!ok || t->grab < 1 || t->grab > 64) return bfail(b, GPAT_ERR_ARG, "tuning outside the variants");
    if (t->chunk_pushes < 0 || (t->chunk_pushes > 0 && t->chunk_pushes < 8) ||
        t->chunk_pushes > 1 << 20)
        return bfail(b, GPAT_ERR_ARG, "chunk_pushes: 0 or 8 .. 2^20");
    b->tuning = *t;
    return GPAT_OK;
}

int gpat_batch_stats(const gpat_batch_t *b, double *ms, uint64_t *pushes, int64_t *graph_launches) {
    if (!b) return GPAT_ERR_ARG;
    if (ms) *ms = b->last_ms;
    if (pushes) *pushes = b->last_steps;
    if (graph_launches) *graph_launches = b->last_graph_launches;
    return GPAT_OK;
}

// ---------------------------------------------------------------------------
// Learned splitting: the importance network, its training records and the
// weighted split / roulette.
// ---------------------------------------------------------------------------
struct gpat_mlp {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    float *master = nullptr, *m1 = nullptr, *m2 = nullptr, *grad = nullptr;
    __nv_bfloat16 *w16 = nullptr;
    float *norm = nullptr;                 // mean[8], 1/std[8]
    float host_norm[2 * kMlpFeatures] = {};
    int adam_step = 0;
    // records: features [cap][8], injection tag, label
    int64_t rec_cap = 0;
    float *feat = nullptr, *labels = nullptr;
    int32_t *tags = nullptr;
    unsigned long long *dcount = nullptr;  // records written; positives; scratch
    float *p_by_tag = nullptr;
    int64_t p_by_tag_n = 0;
    // minibatch buffers
    int64_t tb = 0;
    MlpTrainBuffers t{};
    float *xbuf = nullptr, *ybuf = nullptr, *zbuf = nullptr, *dloss = nullptr;
    int64_t xcap = 0;
    int64_t *index = nullptr;
    int64_t index_cap = 0;
};

namespace {

int mfail(gpat_mlp_t *m, int code, const std::string &msg) {
    if (m) m->err = msg;
    return code;
}

#define MCK(call)                                                                     \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            return mfail(m, GPAT_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

int mlp_train_buffers(gpat_mlp_t *m, int64_t b) {
    if (b <= m->tb) return GPAT_OK;
    float *ptrs[8] = {m->t.h0, m->t.a1, m->t.a2, m->t.a3, m->t.h1, m->t.h2, m->t.h3, m->t.dz};
    for (float *p : ptrs)
        if (p) cudaFree(p);
    m->t = MlpTrainBuffers{};
    const size_t H = (size_t)kMlpHidden * (size_t)b;
    MCK(cudaMalloc(&m->t.h0, sizeof(float) * kMlpFeatures * (size_t)b));
    MCK(cudaMalloc(&m->t.a1, sizeof(float) * H));
    MCK(cudaMalloc(&m->t.a2, sizeof(float) * H));
    MCK(cudaMalloc(&m->t.a3, sizeof(float) * H));
    MCK(cudaMalloc(&m->t.h1, sizeof(float) * H));
    MCK(cudaMalloc(&m->t.h2, sizeof(float) * H));
    MCK(cudaMalloc(&m->t.h3, sizeof(float) * H));
    MCK(cudaMalloc(&m->t.dz, sizeof(float) * (size_t)b));
    m->tb = b;
    return GPAT_OK;
}

int mlp_xbuf(gpat_mlp_t *m, int64_t n) {
    if (n <= m->xcap) return GPAT_OK;
    if (m->xbuf) cudaFree(m->xbuf);
    if (m->ybuf) cudaFree(m->ybuf);
    if (m->zbuf) cudaFree(m->zbuf);
    MCK(cudaMalloc(&m->xbuf, sizeof(float) * kMlpFeatures * (size_t)n));
    MCK(cudaMalloc(&m->ybuf, sizeof(float) * (size_t)n));
    MCK(cudaMalloc(&m->zbuf, sizeof(float) * (size_t)n));
    m->xcap = n;
    return GPAT_OK;
}

FeatureArgs feature_args(const gpat_handle_t *h, double t_norm) {
    const gpat_mhd_config_t &c = h->cfg;
    FeatureArgs g{};
    g.rec = h->rec[0];
    g.xmin = c.xmin; g.ymin = c.ymin; g.zmin = c.zmin;
    g.idx = 1.0 / c.dx; g.idy = 1.0 / c.dy; g.idz = h->prm.ndim == 3 ? 1.0 / c.dz : 0.0;
    g.ilx = 1.0 / ((double)c.nx * c.dx); g.ily = 1.0 / ((double)c.ny * c.dy);
    g.ilz = h->prm.ndim == 3 ? 1.0 / ((double)c.nz * c.dz) : 0.0;
    g.ip0 = 1.0 / h->prm.p0;
    g.nxg = h->nxg; g.nyg = h->nyg; g.nzg = h->nzg;
    g.t_norm = (float)t_norm;
    return g;
}

}  // namespace

int gpat_mlp_create(int device, uint64_t seed, int64_t record_capacity, gpat_mlp_t **out) {
    if (!out || record_capacity < 0) return GPAT_ERR_ARG;
    *out = nullptr;
    gpat_mlp_t *m = new gpat_mlp_t;
    m->device = device;
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
        mlp_set_kernel_attributes() != cudaSuccess) {
        delete m;
        return GPAT_ERR_CUDA;
    }
    const size_t P = kMlpParams;
    bool ok = cudaMalloc(&m->master, 4 * P) == cudaSuccess && cudaMalloc(&m->m1, 4 * P) == cudaSuccess &&
              cudaMalloc(&m->m2, 4 * P) == cudaSuccess && cudaMalloc(&m->grad, 4 * P) == cudaSuccess &&
              cudaMalloc(&m->w16, 2 * P) == cudaSuccess &&
              cudaMalloc(&m->norm, sizeof(float) * 2 * kMlpFeatures) == cudaSuccess &&
              cudaMalloc(&m->dcount, sizeof(unsigned long long) * 4) == cudaSuccess &&
              cudaMalloc(&m->dloss, sizeof(float)) == cudaSuccess;
    m->rec_cap = record_capacity;
    if (ok && record_capacity > 0)
        ok = cudaMalloc(&m->feat, sizeof(float) * kMlpFeatures * (size_t)record_capacity) == cudaSuccess &&
             cudaMalloc(&m->labels, sizeof(float) * (size_t)record_capacity) == cudaSuccess &&
             cudaMalloc(&m->tags, sizeof(int32_t) * (size_t)record_capacity) == cudaSuccess;
    if (!ok) {
        gpat_mlp_destroy(m);
        return GPAT_ERR_OOM;
    }
    // He-style initialisation from a seeded host generator (uniform, var 2/fan_in)
    std::vector<float> w(P, 0.0f);
    uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
    auto uni = [&]() {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        return (double)(st >> 11) * (1.0 / 9007199254740992.0);
    };
    const int H = kMlpHidden, F = kMlpFeatures;
    auto fill = [&](size_t off, int rows, int cols) {
        const double a = std::sqrt(6.0 / cols);
        for (int k = 0; k < rows * cols; ++k) w[off + k] = (float)((2.0 * uni() - 1.0) * a);
    };
    fill(0, H, F);
    fill((size_t)H * F + H, H, H);
    fill((size_t)H * F + H + H * H + H, H, H);
    fill((size_t)H * F + 2 * (H + H * H) + H - H, 1, H);   // output row
    for (int k = 0; k < F; ++k) { m->host_norm[k] = 0.0f; m->host_norm[F + k] = 1.0f; }
    if (cudaMemcpy(m->master, w.data(), 4 * P, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(m->m1, 0, 4 * P) != cudaSuccess || cudaMemset(m->m2, 0, 4 * P) != cudaSuccess ||
        cudaMemset(m->grad, 0, 4 * P) != cudaSuccess ||
        cudaMemcpy(m->norm, m->host_norm, sizeof m->host_norm, cudaMemcpyHostToDevice) != cudaSuccess ||
        launch_to_bf16(m->master, m->w16, m->stream) != cudaSuccess ||
        cudaMemsetAsync(m->dcount, 0, sizeof(unsigned long long) * 4, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) {
        gpat_mlp_destroy(m);
        return GPAT_ERR_CUDA;
    }
    *out = m;
    return GPAT_OK;
}

int gpat_mlp_destroy(gpat_mlp_t *m) {
    if (!m) return GPAT_ERR_ARG;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    void *ptrs[] = {m->master, m->m1, m->m2, m->grad, m->w16, m->norm, m->feat, m->labels, m->tags,
                    m->dcount, m->p_by_tag, m->t.h0, m->t.a1, m->t.a2, m->t.a3, m->t.h1, m->t.h2,
                    m->t.h3, m->t.dz, m->xbuf, m->ybuf, m->zbuf, m->dloss, m->index};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return GPAT_OK;
}

const char *gpat_mlp_last_error(const gpat_mlp_t *m) { return m ? m->err.c_str() : "null network"; }

int gpat_mlp_set_params(gpat_mlp_t *m, const float *params, const float *norm) {
    if (!m) return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    if (params) {
        MCK(cudaMemcpy(m->master, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
        MCK(launch_to_bf16(m->master, m->w16, m->stream));
    }
    if (norm) {
        std::memcpy(m->host_norm, norm, sizeof m->host_norm);
        MCK(cudaMemcpyAsync(m->norm, m->host_norm, sizeof m->host_norm, cudaMemcpyHostToDevice,
                            m->stream));
    }
    MCK(cudaStreamSynchronize(m->stream));
    return GPAT_OK;
}

int gpat_mlp_get_params(gpat_mlp_t *m, float *params, float *norm) {
    if (!m) return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    if (params)
        MCK(cudaMemcpy(params, m->master, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    if (norm) std::memcpy(norm, m->host_norm, sizeof m->host_norm);
    return GPAT_OK;
}

int gpat_mlp_forward(gpat_mlp_t *m, const float *x, int64_t n, float *z) {
    if (!m || !x || !z || n < 0) return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    int rc = mlp_xbuf(m, n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(m->xbuf, x, sizeof(float) * kMlpFeatures * (size_t)n,
                        cudaMemcpyHostToDevice, m->stream));
    MCK(launch_mlp_infer(m->w16, m->norm, m->xbuf, n, m->zbuf, m->stream));
    MCK(cudaMemcpyAsync(z, m->zbuf, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return GPAT_OK;
}

int gpat_mlp_loss_grad(gpat_mlp_t *m, const float *x, const float *y, int64_t n, float *loss,
                       float *grad) {
    if (!m || !x || !y || n < 1) return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    int rc = mlp_xbuf(m, n);
    if (rc) return rc;
    rc = mlp_train_buffers(m, n);
    if (rc) return rc;
    MCK(cudaMemcpyAsync(m->xbuf, x, sizeof(float) * kMlpFeatures * (size_t)n,
                        cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemcpyAsync(m->ybuf, y, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemsetAsync(m->grad, 0, sizeof(float) * kMlpParams, m->stream));
    MCK(cudaMemsetAsync(m->dloss, 0, sizeof(float), m->stream));
    MCK(launch_mlp_train_step(m->t, m->w16, m->norm, m->xbuf, m->ybuf, nullptr, n, m->grad,
                              m->dloss, m->stream));
    if (grad)
        MCK(cudaMemcpyAsync(grad, m->grad, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost,
                            m->stream));
    if (loss) MCK(cudaMemcpyAsync(loss, m->dloss, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaMemsetAsync(m->grad, 0, sizeof(float) * kMlpParams, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return GPAT_OK;
}

int gpat_mlp_clear_records(gpat_mlp_t *m) {
    if (!m) return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    MCK(cudaMemsetAsync(m->dcount, 0, sizeof(unsigned long long) * 4, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return GPAT_OK;
}

int gpat_mlp_record(gpat_mlp_t *m, gpat_handle_t *h, double t_norm, int64_t *nrec) {
    if (!m || !h) return GPAT_ERR_ARG;
    if (m->rec_cap <= 0) return mfail(m, GPAT_ERR_STATE, "no record capacity");
    if (!h->rec_ready[0]) return mfail(m, GPAT_ERR_STATE, "run has no fields");
    MCK(cudaSetDevice(m->device));
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return mfail(m, GPAT_ERR_CUDA, "run stream");
    MCK(launch_record_features(feature_args(h, t_norm), h->prm.ndim, h->P[h->cur], h->n, m->feat,
                               m->tags, m->dcount, m->rec_cap, m->stream));
    unsigned long long c = 0;
    MCK(cudaMemcpyAsync(&c, m->dcount, sizeof c, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (nrec) *nrec = (int64_t)std::min<unsigned long long>(c, (unsigned long long)m->rec_cap);
    return GPAT_OK;
}

int gpat_mlp_label(gpat_mlp_t *m, gpat_handle_t *h, double p_threshold, int64_t *npos,
                   int64_t *nrec) {
    if (!m || !h) return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    unsigned long long c = 0;
    MCK(cudaMemcpy(&c, m->dcount, sizeof c, cudaMemcpyDeviceToHost));
    const int64_t n = (int64_t)std::min<unsigned long long>(c, (unsigned long long)m->rec_cap);
    const int64_t ntags = std::max<int64_t>(1, h->tag_max);
    if (ntags > m->p_by_tag_n) {
        if (m->p_by_tag) cudaFree(m->p_by_tag);
        m->p_by_tag = nullptr;
        MCK(cudaMalloc(&m->p_by_tag, sizeof(float) * (size_t)ntags));
        m->p_by_tag_n = ntags;
    }
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return mfail(m, GPAT_ERR_CUDA, "run stream");
    MCK(cudaMemsetAsync(m->dcount + 1, 0, sizeof(unsigned long long), m->stream));
    MCK(launch_label_records(h->P[h->cur], h->n, m->tags, n, m->p_by_tag, ntags,
                             (float)p_threshold, m->labels, m->dcount + 1, m->stream));
    unsigned long long pos = 0;
    MCK(cudaMemcpyAsync(&pos, m->dcount + 1, sizeof pos, cudaMemcpyDeviceToHost, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (npos) *npos = (int64_t)pos;
    if (nrec) *nrec = n;
    return GPAT_OK;
}

int gpat_mlp_train(gpat_mlp_t *m, int epochs, int64_t batch, double lr, double neg_keep,
                   uint64_t seed, double *final_loss) {
    if (!m || epochs < 1 || batch < 32 || !(lr > 0.0) || !(neg_keep > 0.0) || neg_keep > 1.0)
        return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    unsigned long long c = 0;
    MCK(cudaMemcpy(&c, m->dcount, sizeof c, cudaMemcpyDeviceToHost));
    const int64_t n = (int64_t)std::min<unsigned long long>(c, (unsigned long long)m->rec_cap);
    if (n < 1) return mfail(m, GPAT_ERR_STATE, "no labelled records");
    // Training set: every positive and a neg_keep fraction of negatives,
    // shuffled each epoch on the host (seeded).
    std::vector<float> lab((size_t)n);
    MCK(cudaMemcpy(lab.data(), m->labels, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost));
    uint64_t st = seed * 0xD1B54A32D192ED03ull + 7;
    auto next = [&]() {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        return st;
    };
    std::vector<int64_t> keep;
    keep.reserve((size_t)n);
    const uint64_t thr = (uint64_t)(neg_keep * 18446744073709551615.0);
    for (int64_t i = 0; i < n; ++i)
        if (lab[(size_t)i] > 0.5f || next() <= thr) keep.push_back(i);
    if (keep.empty()) return mfail(m, GPAT_ERR_STATE, "empty training set");
    // Feature standardisation from up to 4096 kept records spread evenly.
    {
        const size_t ns = std::min<size_t>(keep.size(), 4096);
        std::vector<float> row(kMlpFeatures);
        double sum[kMlpFeatures] = {}, sq[kMlpFeatures] = {};
        for (size_t k = 0; k < ns; ++k) {
            const size_t idx = (size_t)keep[(k * keep.size()) / ns];
            MCK(cudaMemcpy(row.data(), m->feat + idx * kMlpFeatures, sizeof(float) * kMlpFeatures,
                           cudaMemcpyDeviceToHost));
            for (int j = 0; j < kMlpFeatures; ++j) {
                sum[j] += row[j];
                sq[j] += (double)row[j] * row[j];
            }
        }
        for (int j = 0; j < kMlpFeatures; ++j) {
            const double mu = sum[j] / (double)ns;
            const double var = std::max(sq[j] / (double)ns - mu * mu, 1e-12);
            m->host_norm[j] = (float)mu;
            m->host_norm[kMlpFeatures + j] = (float)(1.0 / std::sqrt(var));
        }
        MCK(cudaMemcpy(m->norm, m->host_norm, sizeof m->host_norm, cudaMemcpyHostToDevice));
    }
    const int64_t b = std::min<int64_t>(batch, (int64_t)keep.size());
    int rc = mlp_train_buffers(m, b);
    if (rc) return rc;
    if ((int64_t)keep.size() > m->index_cap) {
        if (m->index) cudaFree(m->index);
        m->index = nullptr;
        MCK(cudaMalloc(&m->index, sizeof(int64_t) * keep.size()));
        m->index_cap = (int64_t)keep.size();
    }
    double last = 0.0;
    for (int e = 0; e < epochs; ++e) {
        for (size_t k = keep.size(); k > 1; --k) std::swap(keep[k - 1], keep[next() % k]);
        MCK(cudaMemcpyAsync(m->index, keep.data(), sizeof(int64_t) * keep.size(),
                            cudaMemcpyHostToDevice, m->stream));
        MCK(cudaMemsetAsync(m->dloss, 0, sizeof(float), m->stream));
        int64_t batches = 0;
        for (int64_t s0 = 0; s0 + b <= (int64_t)keep.size(); s0 += b, ++batches) {
            MCK(launch_mlp_train_step(m->t, m->w16, m->norm, m->feat, m->labels, m->index + s0, b,
                                      m->grad, m->dloss, m->stream));
            MCK(launch_adam(m->master, m->m1, m->m2, m->grad, m->w16, (float)lr, ++m->adam_step,
                            m->stream));
        }
        float l = 0.0f;
        MCK(cudaMemcpyAsync(&l, m->dloss, sizeof l, cudaMemcpyDeviceToHost, m->stream));
        MCK(cudaStreamSynchronize(m->stream));
        last = batches > 0 ? (double)l / (double)batches : 0.0;
    }
    // Negatives were kept with probability neg_keep: shift the output bias
    // by log(neg_keep) so that sigmoid(z) estimates the true probability.
    float b4 = 0.0f;
    MCK(cudaMemcpy(&b4, m->master + (kMlpParams - 1), sizeof b4, cudaMemcpyDeviceToHost));
    b4 += (float)std::log(neg_keep);
    MCK(cudaMemcpy(m->master + (kMlpParams - 1), &b4, sizeof b4, cudaMemcpyHostToDevice));
    MCK(launch_to_bf16(m->master, m->w16, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    if (final_loss) *final_loss = last;
    return GPAT_OK;
}

int gpat_mlp_score(gpat_mlp_t *m, gpat_handle_t *h, double t_norm, double *mean_z,
                   double *log_sum_wexpz, double *log_sum_w) {
    if (!m || !h) return GPAT_ERR_ARG;
    MCK(cudaSetDevice(m->device));
    const int64_t n = h->n;
    if (n < 1) return mfail(m, GPAT_ERR_STATE, "no particles");
    int rc = mlp_xbuf(m, n);
    if (rc) return rc;
    unsigned long long *out = nullptr;
    MCK(cudaMalloc(&out, 7 * sizeof(unsigned long long) + sizeof(int)));
    int *zmax_key = reinterpret_cast<int *>(out + 7);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
        cudaFree(out);
        return mfail(m, GPAT_ERR_CUDA, "run stream");
    }
    unsigned long long r[7] = {};
    int key = 0;
    cudaError_t e = launch_score(m->w16, m->norm, feature_args(h, t_norm), h->prm.ndim, h->P[h->cur],
                                 n, m->zbuf, zmax_key, out, m->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r, out, sizeof r, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&key, zmax_key, sizeof key, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    cudaFree(out);
    if (e != cudaSuccess) return mfail(m, GPAT_ERR_CUDA, cudaGetErrorString(e));
    if (r[0] == 0) return mfail(m, GPAT_ERR_STATE, "no live particles");
    const int kb = key >= 0 ? key : key ^ 0x7FFFFFFF;
    float zmax;
    std::memcpy(&zmax, &kb, sizeof zmax);
    if (mean_z) *mean_z = fixed_to_double(r[1], r[2]) / (double)r[0] - 64.0;
    if (log_sum_wexpz) *log_sum_wexpz = (double)zmax + std::log(fixed_to_double(r[3], r[4]));
    if (log_sum_w) *log_sum_w = std::log(fixed_to_double(r[5], r[6]));
    return GPAT_OK;
}

namespace {

// The device counter of weighted splitting's fresh lineage ids (copies split
// past the int32 tag's 30 binary levels get tag_splitted = -id), created at
// first use and raised past the ids of any particle set received since.
int ensure_fresh(gpat_handle_t *h) {
    if (!h->fresh_dev) {
        if (cudaMalloc(&h->fresh_dev, sizeof(unsigned long long)) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, GPAT_ERR_OOM, "lineage id counter");
        }
        CK(cudaMemsetAsync(h->fresh_dev, 0, sizeof(unsigned long long), h->stream));
    }
    if (h->fresh_floor > 0) {
        unsigned long long cur = 0;
        CK(cudaMemcpyAsync(&cur, h->fresh_dev, sizeof cur, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        if (cur < h->fresh_floor) {
            cur = h->fresh_floor;
            CK(cudaMemcpyAsync(h->fresh_dev, &cur, sizeof cur, cudaMemcpyHostToDevice, h->stream));
            CK(cudaStreamSynchronize(h->stream));
        }
        h->fresh_floor = 0;
    }
    return GPAT_OK;
}

}  // namespace

int gpat_weighted_split(gpat_handle_t *h, gpat_mlp_t *m, double t_norm, double w_ref, double z_ref,
                        double z_floor, double window_ratio, int max_level, int64_t *nsplit,
                        int64_t *nkilled) {
    if (!h || !m || !(w_ref > 0.0) || !(window_ratio > 1.0) || max_level < 1 || max_level > 8 ||
        std::isnan(z_ref) || std::isnan(z_floor) || z_floor == INFINITY)
        return GPAT_ERR_ARG;
    if (h->dtags)
        return fail(h, GPAT_ERR_UNSUPPORTED, "weighted splitting keeps no particle tracks");
    CK(cudaSetDevice(h->device));
    if (cudaStreamSynchronize(m->stream) != cudaSuccess)
        return fail(h, GPAT_ERR_CUDA, "network stream");
    int rc = ensure_fresh(h);
    if (rc) return rc;
    rc = pull_counters(h);
    if (rc) return rc;
    const unsigned long long split0 = h->hcnt.nsplit, kill0 = h->hcnt.nkilled;
    WSplitArgs a{};
    a.fresh = h->fresh_dev;
    a.w_ref = w_ref;
    a.z_ref = z_ref;
    a.z_floor = z_floor;
    a.sqrt_ratio = std::sqrt(window_ratio);
    a.max_level = max_level;
    a.key0 = (uint32_t)h->prm.seed;
    a.key1 = (uint32_t)(h->prm.seed >> 32) + 2u;
    // the child counter starts at n; children are appended up to nptl_max
    unsigned long long n0 = (unsigned long long)h->n;
    CK(cudaMemcpyAsync(&h->dcnt->ncells, &n0, sizeof n0, cudaMemcpyHostToDevice, h->stream));
    CK(launch_weighted_split(m->w16, m->norm, feature_args(h, t_norm), h->prm.ndim, h->P[h->cur],
                             h->n, h->cap, a, &h->dcnt->ncells, h->dcnt, h->stream));
    rc = pull_counters(h);
    if (rc) return rc;
    const int64_t created = (int64_t)h->hcnt.nsplit - (int64_t)split0;
    h->n = (int64_t)h->hcnt.ncells;
    h->nptl_split += created;
    if (created > 0 || h->hcnt.nkilled != kill0) h->unsorted = true;
    if (nsplit) *nsplit = created;
    if (nkilled) *nkilled = (int64_t)(h->hcnt.nkilled - kill0);
    return check_status(h);
}

int gpat_set_mover_learned(gpat_handle_t *h, gpat_mlp_t *m, double t_norm, double w_ref,
                           double z_ref, double z_floor, double window_ratio, int max_level) {
    if (!h) return GPAT_ERR_ARG;
    if (!m) {
        h->learn_on = false;
        return GPAT_OK;
    }
    if (!(w_ref > 0.0) || !(window_ratio > 1.0) || max_level < 1 || max_level > 8 ||
        !std::isfinite(z_ref) || std::isnan(z_floor) || z_floor == INFINITY)
        return fail(h, GPAT_ERR_ARG,
                    "w_ref > 0, window_ratio > 1, max_level in 1..8, z_ref finite, z_floor < inf");
    if (h->prm.precision != GPAT_PREC_MIXED || h->prm.ndim < 2)
        return fail(h, GPAT_ERR_UNSUPPORTED, "learned splitting runs in the split-precision mover");
    if (h->dtags)
        return fail(h, GPAT_ERR_UNSUPPORTED, "weighted splitting keeps no particle tracks");
    CK(cudaSetDevice(h->device));
    if (!h->learn_dev) {
        if (cudaMalloc(&h->learn_dev, 6 * sizeof(unsigned long long)) != cudaSuccess) {
            cudaGetLastError();
            return fail(h, GPAT_ERR_OOM, "learned splitting counters");
        }
    }
    if (cudaStreamSynchronize(m->stream) != cudaSuccess)
        return fail(h, GPAT_ERR_CUDA, "network stream");
    const int rcf = ensure_fresh(h);
    if (rcf) return rcf;
    FusedLearn L{};
    L.w16 = m->w16;
    L.norm = m->norm;
    L.f = feature_args(h, t_norm);
    L.s.w_ref = w_ref;
    L.s.z_ref = z_ref;
    L.s.z_floor = z_floor;
    L.s.sqrt_ratio = std::sqrt(window_ratio);
    L.s.max_level = max_level;
    L.s.key0 = (uint32_t)h->prm.seed;
    L.s.key1 = (uint32_t)(h->prm.seed >> 32) + 2u;
    L.s.fresh = h->fresh_dev;
    L.z_shift = z_ref;
    h->learn = L;
    h->learn_on = true;
    return GPAT_OK;
}

int gpat_get_mover_learned(const gpat_handle_t *h, double *log_sum_wexpz, double *log_sum_w,
                           int64_t *judged, int64_t *nsplit, int64_t *nkilled) {
    if (!h) return GPAT_ERR_ARG;
    const double s = fixed_to_double(h->learn_host[2], h->learn_host[3]);
    const double sw = fixed_to_double(h->learn_host[4], h->learn_host[5]);
    if (log_sum_wexpz) *log_sum_wexpz = s > 0.0 ? h->learn.z_shift + std::log(s) : -INFINITY;
    if (log_sum_w) *log_sum_w = sw > 0.0 ? std::log(sw) : -INFINITY;
    if (judged) *judged = (int64_t)h->learn_host[1];
    if (nsplit) *nsplit = h->learn_split;
    if (nkilled) *nkilled = h->learn_killed;
    return GPAT_OK;
}

int gpat_tail_weights(gpat_handle_t *h, double p_threshold, int64_t *count, double *wsum,
                      double *w2sum) {
    if (!h) return GPAT_ERR_ARG;
    CK(cudaSetDevice(h->device));
    unsigned long long *out = nullptr;
    CK(cudaMalloc(&out, 5 * sizeof(unsigned long long)));
    unsigned long long r[5] = {};
    cudaError_t e = launch_tail(h->P[h->cur], h->n, p_threshold, out, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(r, out, sizeof r, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(out);
    if (e != cudaSuccess) return fail(h, GPAT_ERR_CUDA, cudaGetErrorString(e));
    if (count) *count = (int64_t)r[0];
    if (wsum) *wsum = fixed_to_double(r[1], r[2]);
    if (w2sum) *w2sum = fixed_to_double(r[3], r[4]);
    return GPAT_OK;
}

int gpat_mlp_set_records(gpat_mlp_t *m, const float *x, const float *labels, int64_t n) {
    if (!m || !x || !labels || n < 0) return GPAT_ERR_ARG;
    if (n > m->rec_cap) return mfail(m, GPAT_ERR_CAPACITY, "more records than the capacity");
    MCK(cudaSetDevice(m->device));
    MCK(cudaMemcpyAsync(m->feat, x, sizeof(float) * kMlpFeatures * (size_t)n,
                        cudaMemcpyHostToDevice, m->stream));
    MCK(cudaMemcpyAsync(m->labels, labels, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice,
                        m->stream));
    unsigned long long c = (unsigned long long)n;
    MCK(cudaMemcpyAsync(m->dcount, &c, sizeof c, cudaMemcpyHostToDevice, m->stream));
    MCK(cudaStreamSynchronize(m->stream));
    return GPAT_OK;
}
