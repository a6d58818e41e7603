// Device parts of learned splitting shared by its own kernels (learned.cu)
// and the split-precision mover that applies it as particles finish an
// interval (mover_mixed.cu): particle features from the packed field
// records, standardisation, and the weight-window split / Russian roulette.
#pragma once

#include "device_common.cuh"

namespace gpat {
namespace {

constexpr int kIn = kMlpFeatures, kH = kMlpHidden;
// Fresh lineage ids stop here: the concurrent additions that can pass the
// check (every resident thread x 255 copies) stay below 2^31.
constexpr unsigned long long kFreshIdLimit = 2000000000ull;

__device__ __forceinline__ void clone_particle(const DevParticles &P, int64_t i, int64_t j) {
    P.x[j] = P.x[i]; P.y[j] = P.y[i]; P.z[j] = P.z[i]; P.p[j] = P.p[i];
    P.v[j] = P.v[i]; P.mu[j] = P.mu[i]; P.weight[j] = P.weight[i];
    P.t[j] = P.t[i]; P.dt[j] = P.dt[i];
    P.split_times[j] = P.split_times[i]; P.count_flag[j] = P.count_flag[i];
    P.origin[j] = P.origin[i]; P.nsteps_tracked[j] = P.nsteps_tracked[i];
    P.nsteps_pushed[j] = P.nsteps_pushed[i]; P.tag_injected[j] = P.tag_injected[i];
    P.tag_splitted[j] = P.tag_splitted[i]; P.rng_ctr[j] = P.rng_ctr[i];
}

__device__ __forceinline__ void standardise(const float *x, const float *mean, const float *istd,
                                            float h0[kIn]) {
#pragma unroll
    for (int j = 0; j < kIn; ++j) h0[j] = (x[j] - mean[j]) * istd[j];
}

// ---------------------------------------------------------------------------
// Features of particles, from the packed field records (FP32, trilinear).
// ---------------------------------------------------------------------------
template <int NDIM>
__device__ void particle_features(const FeatureArgs &g, const DevParticles &P, int64_t i,
                                  float f[kIn]) {
    constexpr int R = (NDIM == 2) ? kRec2D : kRec3D;
    const double px = (P.x[i] - g.xmin) * g.idx, py = (P.y[i] - g.ymin) * g.idy;
    const double pz = (NDIM == 3) ? (P.z[i] - g.zmin) * g.idz : 0.0;
    int cx = (int)floor(px), cy = (int)floor(py), cz = (NDIM == 3) ? (int)floor(pz) : 0;
    float fx = (float)(px - cx), fy = (float)(py - cy), fz = (float)(pz - cz);
    // clamp into the ghost-padded grid (a particle about to leave keeps the
    // edge values)
    const int ix = min(max(cx + 2, 0), g.nxg - 2), iy = min(max(cy + 2, 0), g.nyg - 2);
    const int iz = (NDIM == 3) ? min(max(cz + 2, 0), g.nzg - 2) : 0;
    fx = fminf(fmaxf(fx, 0.0f), 1.0f); fy = fminf(fmaxf(fy, 0.0f), 1.0f);
    fz = fminf(fmaxf(fz, 0.0f), 1.0f);
    float v[R];
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = 0.0f;
    for (int kk = 0; kk < (NDIM == 3 ? 2 : 1); ++kk)
        for (int j = 0; j < 2; ++j)
            for (int ii = 0; ii < 2; ++ii) {
                float w = (ii ? fx : 1.0f - fx) * (j ? fy : 1.0f - fy);
                if (NDIM == 3) w *= (kk ? fz : 1.0f - fz);
                const size_t cell = (size_t)(ix + ii) +
                                    (size_t)g.nxg * ((size_t)(iy + j) + (size_t)g.nyg * (iz + kk));
                const float *r = g.rec + (size_t)R * cell;
#pragma unroll
                for (int k = 0; k < R; ++k) v[k] = fmaf(__ldg(r + k), w, v[k]);
            }
    f[0] = (float)((P.x[i] - g.xmin) * g.ilx);
    f[1] = (float)((P.y[i] - g.ymin) * g.ily);
    f[2] = (NDIM == 3) ? (float)((P.z[i] - g.zmin) * g.ilz) : 0.0f;
    f[3] = (float)log10(P.p[i] * g.ip0);
    if (NDIM == 2) {   // slots: vx vy bx by bz dvx/dx dvy/dy ... db/dx(13) db/dy(14)
        f[4] = v[5] + v[6];
        f[5] = sqrtf(v[2] * v[2] + v[3] * v[3] + v[4] * v[4]);
        f[6] = sqrtf(v[13] * v[13] + v[14] * v[14]);
    } else {           // slots: vx vy vz bx by bz dvx/dx dvy/dy dvz/dz ... db/dx(18..20)
        f[4] = v[6] + v[7] + v[8];
        f[5] = sqrtf(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
        f[6] = sqrtf(v[18] * v[18] + v[19] * v[19] + v[20] * v[20]);
    }
    f[7] = g.t_norm;
}


// Floored log-importance log(exp(z) + exp(z_floor)) of a network output.
__device__ __forceinline__ double floored_importance(double z, double z_floor) {
    z = fmin(fmax(z, -60.0), 60.0);
    if (!(z_floor > -1e300)) return z;
    const double hi = fmax(z, z_floor), lo = fmin(z, z_floor);
    return hi + log1p(exp(lo - hi));
}

// The weight window around w_t = w_ref exp(-(z' - z_ref)), z' the floored
// log-importance, for the particle of this lane (live: in the box and to be
// judged), then the warp-aggregated reservation of the children's slots.
// All 32 lanes of the warp must call.
__device__ __forceinline__ void window_split(const WSplitArgs &a, const DevParticles &P, int64_t i,
                                             bool live, float z, int64_t cap,
                                             unsigned long long *count, DevCounters *cnt) {
    int j = 0;
    bool fresh = false;
    double w = 0.0;
    if (live) {
        const double wt = a.w_ref * exp(-(floored_importance((double)z, a.z_floor) - a.z_ref));
        w = P.weight[i];
        if (w > wt * a.sqrt_ratio) {
            const int split_times = P.split_times[i];
            j = (int)ceil(log2(w / (wt * a.sqrt_ratio)));
            j = max(1, min(j, a.max_level));
            if (split_times + j > 30) {
                // past the int32 tag's 30 binary levels the copies take fresh
                // negative ids (every copy keeps a distinct Philox stream);
                // the ids stop short of the int32 range
                if (!a.fresh || *(volatile unsigned long long *)a.fresh > kFreshIdLimit) j = 0;
                else fresh = true;
            }
        } else if (w < wt / a.sqrt_ratio) {
            const uint4 r = philox4x32_10(
                make_uint4(P.rng_ctr[i], 0x524C5454u, (uint32_t)P.tag_injected[i],
                           (uint32_t)P.tag_splitted[i]),
                a.key0, a.key1);
            const double u = u01_53(r.x, r.y);
            if (u < w / wt) {
                P.weight[i] = wt;
            } else {
                P.count_flag[i] = 0;               // removed at the next removal
                atomicAdd(&cnt->nkilled, 1ull);
            }
        }
    }
    // Warp-aggregated reservation of the children slots.
    const int lane = threadIdx.x & 31;
    const unsigned m = (j > 0) ? ((1u << j) - 1u) : 0u;
    unsigned inc = m;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
    unsigned long long base = 0;
    int ok = 0;
    if (lane == 31 && total > 0) {
        unsigned long long old = *(volatile unsigned long long *)count;
        for (int t = 0; t < 1024; ++t) {       // bounded compare-and-swap
            if (old + total > (unsigned long long)cap) break;
            const unsigned long long prev = atomicCAS(count, old, old + total);
            if (prev == old) { ok = 1; base = old; break; }
            old = prev;
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 31);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (!ok || j == 0) return;
    const int64_t first = (int64_t)(base + inc - m);
    const int s = P.split_times[i];
    const double wc = w / (double)(1u << j);
    P.weight[i] = wc;
    P.split_times[i] = (int8_t)min(s + j, 120);
    const unsigned long long id0 = fresh ? atomicAdd(a.fresh, (unsigned long long)m) : 0ull;
    for (unsigned c = 1; c <= m; ++c) {
        const int64_t d = first + (int64_t)(c - 1);
        clone_particle(P, i, d);
        P.tag_splitted[d] = fresh ? -(int32_t)(id0 + c)
                                  : (int32_t)((uint32_t)P.tag_splitted[i] + (c << s));
    }
    atomicAdd(&cnt->nsplit, (unsigned long long)m);
}

}  // namespace
}  // namespace gpat
