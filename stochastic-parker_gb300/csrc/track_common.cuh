// Particle tracking shared by the FP64 mover, injection and splitting:
// the search of tags_tracking and the writes into particles_tracked.
#pragma once

#include "gpat_internal.h"

namespace gpat {

// is_particle_selected (particle_module.f90:5923-5963): the first and last
// columns (0-based lo..hi) whose origin matches, then, between those, whose
// tag_injected matches |tag_inj|, then, after nsplit > 0 splits, whose row
// nsplit + 2 matches |tag_spl|.  A particle split more often than the table
// records is not selected.  locate_particle (:5971-5994) is the same search
// for a particle already tracked.
__device__ inline bool trk_select(const TrackArgs &t, int32_t origin, int32_t tag_inj, int nsplit,
                                  int32_t tag_spl, int &lo, int &hi) {
    if (nsplit < 0 || nsplit > t.nrows - 2) return false;
    const int32_t *T = t.tags;
    const size_t R = (size_t)t.nrows;
    int a = -1, b = -1;
    for (int j = 0; j < t.n; ++j)
        if (__ldg(T + R * j) == origin) { if (a < 0) a = j; b = j; }
    if (a < 0) return false;
    const int32_t ti = tag_inj < 0 ? -tag_inj : tag_inj;
    int c = -1, d = -1;
    for (int j = a; j <= b; ++j)
        if (__ldg(T + R * j + 1) == ti) { if (c < 0) c = j; d = j; }
    if (c < 0) return false;
    if (nsplit == 0) { lo = c; hi = d; return true; }
    const int32_t ts = tag_spl < 0 ? -tag_spl : tag_spl;
    int e = -1, f = -1;
    for (int j = c; j <= d; ++j)
        if (__ldg(T + R * j + nsplit + 1) == ts) { if (e < 0) e = j; f = j; }
    if (e < 0) return false;
    lo = e; hi = f;
    return true;
}

// One particle_type record.
struct TrkRecord {
    double x, y, z, p, v, mu, w, t, dt;
    int split_times, count_flag;
    int32_t origin, nsteps_tracked, nsteps_pushed, tag_inj, tag_spl;
    uint32_t ctr;
};

__device__ inline TrkRecord trk_from(const DevParticles &P, int64_t i) {
    TrkRecord r;
    r.x = P.x[i]; r.y = P.y[i]; r.z = P.z[i]; r.p = P.p[i]; r.v = P.v[i]; r.mu = P.mu[i];
    r.w = P.weight[i]; r.t = P.t[i]; r.dt = P.dt[i];
    r.split_times = P.split_times[i]; r.count_flag = P.count_flag[i];
    r.origin = P.origin[i]; r.nsteps_tracked = P.nsteps_tracked[i];
    r.nsteps_pushed = P.nsteps_pushed[i];
    r.tag_inj = P.tag_injected[i]; r.tag_spl = P.tag_splitted[i];
    r.ctr = P.rng_ctr[i];
    return r;
}

// particles_tracked(row, lo + 1 : hi + 1) = ptl, row 1-based.  A row past
// nsteps_tracking_max is counted in trk_dropped instead of written.
__device__ inline void trk_write(const TrackArgs &t, int64_t row, int lo, int hi,
                                 const TrkRecord &r, DevCounters *cnt) {
    if (row < 1 || row > t.nsteps_max) {
        atomicAdd(&cnt->trk_dropped, 1ull);
        return;
    }
    const DevParticles &D = t.rec;
    for (int j = lo; j <= hi; ++j) {
        const size_t e = (size_t)(row - 1) + (size_t)t.nsteps_max * (size_t)j;
        D.x[e] = r.x; D.y[e] = r.y; D.z[e] = r.z; D.p[e] = r.p; D.v[e] = r.v; D.mu[e] = r.mu;
        D.weight[e] = r.w; D.t[e] = r.t; D.dt[e] = r.dt;
        D.split_times[e] = (int8_t)r.split_times; D.count_flag[e] = (int8_t)r.count_flag;
        D.origin[e] = r.origin; D.nsteps_tracked[e] = r.nsteps_tracked;
        D.nsteps_pushed[e] = r.nsteps_pushed;
        D.tag_injected[e] = r.tag_inj; D.tag_splitted[e] = r.tag_spl;
        D.rng_ctr[e] = r.ctr;
    }
}

}  // namespace gpat
