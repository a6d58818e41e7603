// Particle-set kernels around the mover: injection, stable removal
// (remove_particles), splitting (split_particle), the global f(p) histogram
// (calc_particle_distributions) and the quick_check reductions.
#include <cfloat>

#include "cell_index.cuh"
#include "device_common.cuh"
#include "grid_common.cuh"
#include "track_common.cuh"

namespace gpat {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kTile = kScanThreads * kScanItems;   // particles per block

// ---------------------------------------------------------------------------
// Injection (inject_one_particle and the two injectors, particle_module.f90:
// 385-633).  One thread per new particle; its draws come from a Philox stream
// keyed (seed_lo, seed_hi + 1) with counter (tag, call, 'INJC', 0).
// ---------------------------------------------------------------------------
struct InjStream {
    uint32_t k0, k1, tag, call;
    double buf0, buf1;
    int avail;
    __device__ double next() {
        if (avail == 0) {
            const uint4 w = philox4x32_10(make_uint4(tag, call, 0x494E4A43u, 0u), k0, k1);
            call += 1u;
            buf0 = u01_53(w.x, w.y);
            buf1 = u01_53(w.z, w.w);
            avail = 2;
        }
        const double u = (avail == 2) ? buf0 : buf1;
        avail -= 1;
        return u;
    }
};

constexpr int kMaxRejections = 1 << 22;

__device__ double draw_p_power(const InjectArgs &a, InjStream &s) {
    const double r01 = s.next();
    if ((int)a.power_index == 1) return pow(a.pmax / a.p0, r01) * a.p0;
    const double norm = pow(a.pmax, -a.power_index + 1.0) - pow(a.p0, -a.power_index + 1.0);
    return pow(r01 * norm + pow(a.p0, -a.power_index + 1.0), 1.0 / (-a.power_index + 1.0));
}

// interp_fields of frame 1 at rt = 0 (mhd_data_parallel.f90:1751-1804) at a
// point inside the box, FP64 accumulation over the corners in the movers'
// order.
__device__ bool interp_frame1(const LargeArgs &g, int ndim, double x, double y, double z,
                              double f[32]) {
    if (g.spherical || g.nonuniform) {
        // spherical / non-uniform corner and weights (:866-880)
        GridCell c;
        if (!grid_cell(ndim, g.spherical, g.xpos, g.nxg, g.ypos, g.nyg, g.zpos, g.nzg, x, y, z, c))
            return false;
        for (int v = 0; v < 32; ++v) f[v] = 0.0;
        for (int k = 0; k < (ndim == 3 ? 2 : 1); ++k)
            for (int j = 0; j < 2; ++j)
                for (int i = 0; i < 2; ++i) {
                    const double wc = c.w[k * 4 + j * 2 + i];
                    const size_t cell = (size_t)(c.ix + i) +
                                        (size_t)g.nxg * ((size_t)(c.iy + j) +
                                                         (size_t)g.nyg * (size_t)(c.iz + k));
                    const float *r = g.full + 32 * cell;
                    for (int v = 0; v < 32; ++v) f[v] = f[v] + (double)__ldg(r + v) * wc;
                }
        return true;
    }
    const double px = (x - g.gxmin) / g.dx, py = (y - g.gymin) / g.dy, pz = (z - g.gzmin) / g.dz;
    const int fx = (int)floor(px), fy = (int)floor(py), fz = (ndim == 3) ? (int)floor(pz) : 0;
    const double rx = (px - (double)(fx + 1)) + 1.0;
    const double ry = (py - (double)(fy + 1)) + 1.0;
    const double rz = (ndim == 3) ? (pz - (double)(fz + 1)) + 1.0 : 0.0;
    const double rx1 = 1.0 - rx, ry1 = 1.0 - ry, rz1 = 1.0 - rz;
    const double w[8] = {rx1 * ry1 * rz1, rx * ry1 * rz1, rx1 * ry * rz1, rx * ry * rz1,
                         rx1 * ry1 * rz,  rx * ry1 * rz,  rx1 * ry * rz,  rx * ry * rz};
    const int ix = fx + 2, iy = fy + 2, iz = (ndim == 3) ? fz + 2 : 0;
    for (int v = 0; v < 32; ++v) f[v] = 0.0;
    for (int k = 0; k < (ndim == 3 ? 2 : 1); ++k)
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i) {
                const double wc = w[k * 4 + j * 2 + i];
                const size_t cell = (size_t)(ix + i) +
                                    (size_t)g.nxg * ((size_t)(iy + j) + (size_t)g.nyg * (size_t)(iz + k));
                const float *r = g.full + 32 * cell;
                for (int v = 0; v < 32; ++v) f[v] = f[v] + (double)__ldg(r + v) * wc;
            }
    return true;
}

// db2_slab(1) interpolated at a point (interp_magnetic_fluctuation,
// mhd_data_parallel.f90:1806-1854, rt = 0), same weights as the fields.
__device__ bool interp_db2(const LargeArgs &g, int ndim, double x, double y, double z,
                           double &out) {
    if (g.spherical || g.nonuniform) {
        GridCell c;
        if (!grid_cell(ndim, g.spherical, g.xpos, g.nxg, g.ypos, g.nyg, g.zpos, g.nzg, x, y, z, c))
            return false;
        double v = 0.0;
        for (int k = 0; k < (ndim == 3 ? 2 : 1); ++k)
            for (int j = 0; j < 2; ++j)
                for (int i = 0; i < 2; ++i) {
                    const size_t cell = (size_t)(c.ix + i) +
                                        (size_t)g.nxg * ((size_t)(c.iy + j) +
                                                         (size_t)g.nyg * (size_t)(c.iz + k));
                    v = v + (double)__ldg(g.aux + 16 * cell) * c.w[k * 4 + j * 2 + i];
                }
        out = v;
        return true;
    }
    const double px = (x - g.gxmin) / g.dx, py = (y - g.gymin) / g.dy, pz = (z - g.gzmin) / g.dz;
    const int fx = (int)floor(px), fy = (int)floor(py), fz = (ndim == 3) ? (int)floor(pz) : 0;
    const double rx = (px - (double)(fx + 1)) + 1.0;
    const double ry = (py - (double)(fy + 1)) + 1.0;
    const double rz = (ndim == 3) ? (pz - (double)(fz + 1)) + 1.0 : 0.0;
    const double rx1 = 1.0 - rx, ry1 = 1.0 - ry, rz1 = 1.0 - rz;
    const double w[8] = {rx1 * ry1 * rz1, rx * ry1 * rz1, rx1 * ry * rz1, rx * ry * rz1,
                         rx1 * ry1 * rz,  rx * ry1 * rz,  rx1 * ry * rz,  rx * ry * rz};
    const int ix = fx + 2, iy = fy + 2, iz = (ndim == 3) ? fz + 2 : 0;
    double v = 0.0;
    for (int k = 0; k < (ndim == 3 ? 2 : 1); ++k)
        for (int j = 0; j < 2; ++j)
            for (int i = 0; i < 2; ++i) {
                const size_t cell = (size_t)(ix + i) +
                                    (size_t)g.nxg * ((size_t)(iy + j) + (size_t)g.nyg * (size_t)(iz + k));
                v = v + (double)__ldg(g.aux + 16 * cell) * w[k * 4 + j * 2 + i];
            }
    out = v;
    return true;
}

// The quantity each inject_particles_at_large_* tests, from interpolated
// fields (:874-890, :1027-1044, :1305-1320, :1437); the divv test is on
// -div v.  Spherical coordinates use the reference's spherical forms with
// r = x, theta = y (its divv adds vz / (r sin theta), not dvz/dz / ...).
__device__ double large_quantity(int quantity, int ndim, bool sph, double x, double y,
                                 const double f[32]) {
    if (sph) {
        if (quantity == GPAT_LARGE_JZ) return fabs(f[23] + (f[5] - f[21]) / x);
        if (quantity == GPAT_LARGE_ABSJ) {
            const double ctheta = cos(y), stheta = sin(y), r = x;
            const double t1 = (ctheta * f[6] + stheta * f[27] - f[25]) / (r * stheta);
            const double t2 = (f[22] / stheta - f[6] - r * f[26]) / r;
            const double t3 = (f[5] + r * f[23] - f[21]) / r;
            return sqrt(t1 * t1 + t2 * t2 + t3 * t3);
        }
        if (quantity == GPAT_LARGE_DIVV) {
            double d = f[8] + 2.0 * f[0] / x;
            if (ndim > 1) {
                const double ctheta = cos(y), istheta = 1.0 / sin(y);
                d = d + (f[12] + f[1] * ctheta * istheta) / x;
                if (ndim > 2) d = d + f[2] * istheta / x;
            }
            return -d;
        }
        return f[3];
    }
    if (quantity == GPAT_LARGE_JZ) return fabs(f[23] - f[21]);
    if (quantity == GPAT_LARGE_ABSJ) {
        const double a = f[25] - f[27], b = f[26] - f[22], c = f[21] - f[23];
        return sqrt(a * a + b * b + c * c);
    }
    if (quantity == GPAT_LARGE_DIVV) {
        double d = f[8];
        d = d + f[12];
        if (ndim > 2) d = d + f[16];
        return -d;
    }
    return f[3];
}

// inject_particles_at_shock's position (particle_module.f90:568-588) with
// interp_shock_location (mhd_data_parallel.f90:2017-2046) as intended: the
// shock index of the rows either side of y (and z), linear in (y - ymin) / dy,
// mapped to x = xmin + (index - 3) dx (index 3 is the first physical node).
__device__ double shock_x(const InjectArgs &a, double y, double z) {
    const int32_t *S = a.shock_ix;
    double sx;
    if (a.ndim == 1) {
        sx = (double)S[0];
    } else {
        const double dpy = (y - a.gymin) / a.dy;
        const int jy = (int)floor(dpy);
        const double ry = dpy - (double)jy;
        const int r0 = min(max(jy + 2, 0), a.nyg - 1), r1 = min(max(jy + 3, 0), a.nyg - 1);
        if (a.ndim == 2) {
            sx = (1.0 - ry) * (double)S[r0] + ry * (double)S[r1];
        } else {
            const double dpz = (z - a.gzmin) / a.dz;
            const int jz = (int)floor(dpz);
            const double rz = dpz - (double)jz;
            const int k0 = min(max(jz + 2, 0), a.nzg - 1), k1 = min(max(jz + 3, 0), a.nzg - 1);
            sx = (1.0 - ry) * (1.0 - rz) * (double)S[r0 + a.nyg * k0] +
                 ry * (1.0 - rz) * (double)S[r1 + a.nyg * k0] +
                 (1.0 - ry) * rz * (double)S[r0 + a.nyg * k1] + ry * rz * (double)S[r1 + a.nyg * k1];
        }
    }
    return a.gxmin + (sx - 3.0) * a.dx;
}

// One warp per row: the first x index of the largest |dvx/dx| (slot 8 of the
// 32-variable records), NaN never wins; written 1-based like maxloc.
__global__ void __launch_bounds__(256) locate_shock_kernel(const float *full, int nxg, int nrows,
                                                           int32_t *shock_ix) {
    const int row = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
    if (row >= nrows) return;
    const int lane = threadIdx.x & 31;
    float best = -1.0f;
    int at = nxg;
    for (int ix = lane; ix < nxg; ix += 32) {
        const float v = fabsf(full[8 + 32 * ((size_t)ix + (size_t)nxg * (size_t)row)]);
        if (v > best) { best = v; at = ix; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oa = __shfl_xor_sync(0xffffffffu, at, o);
        if (ob > best || (ob == best && oa < at)) { best = ob; at = oa; }
    }
    if (lane == 0) shock_ix[row] = (at < nxg ? at : 0) + 1;
}

__global__ void inject_kernel(const InjectArgs a, unsigned int *status) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.count) return;
    const int32_t tag = a.tag0 + (int32_t)i;
    InjStream s{a.key0, a.key1 + 1u, (uint32_t)tag, 0u, 0.0, 0.0, 0};
    double x, y, z, p = a.p0, mu, t;
    const double mu_max = (double)0.99f;
    if (a.mode == 0) {
        x = s.next() * (a.box[3] - a.box[0]) + a.box[0];
        y = s.next() * (a.box[4] - a.box[1]) + a.box[1];
        z = s.next() * (a.box[5] - a.box[2]) + a.box[2];
        mu = mu_max * (2.0 * s.next() - 1.0);
        if (a.dist_flag == 0) {
            double ftest = 1.0, fxp = 0.5, ptmp = 0.0;
            int it = 0;
            while (ftest > fxp) {
                if (++it > kMaxRejections) { atomicOr(status, kStatusStepLimit); break; }
                ptmp = (s.next() * (a.pmax - a.pmin) + a.pmin) / a.p0;
                fxp = ptmp * ptmp * exp(-(ptmp * ptmp));
                ftest = s.next() * (double)0.37f;
            }
            p = ptmp * a.p0;
        } else if (a.dist_flag == 2) {
            p = draw_p_power(a, s);
        }
        t = a.t_frame + s.next() * a.dt_mhd;
    } else if (a.mode == 2) {
        // Rejection over the whole box until the point is in part_box with
        // the quantity >= qmin.  The loop runs only when the quantity's
        // starting value (-2; -divv = -2; rho = 0) is below qmin; otherwise
        // the particle stays at the part_box corner, as in the reference.
        const LargeArgs &g = a.lg;
        const bool rho = g.quantity == GPAT_LARGE_RHO;
        double q = rho ? 0.0 : -2.0;
        x = a.box[0]; y = a.box[1]; z = a.box[2];
        int it = 0;
        while (q < g.qmin) {
            if (++it > kMaxRejections) { atomicOr(status, kStatusStepLimit); break; }
            x = s.next() * (g.dom[3] - g.dom[0]) + g.dom[0];
            y = s.next() * (g.dom[4] - g.dom[1]) + g.dom[1];
            z = s.next() * (g.dom[5] - g.dom[2]) + g.dom[2];
            if (x >= a.box[0] && x <= a.box[3] && y >= a.box[1] && y <= a.box[4] &&
                z >= a.box[2] && z <= a.box[5]) {
                if (g.quantity == GPAT_LARGE_DB2) {
                    if (!interp_db2(g, a.ndim, x, y, z, q)) q = rho ? 0.0 : -3.0;
                } else {
                    double f[32];
                    if (interp_frame1(g, a.ndim, x, y, z, f))
                        q = large_quantity(g.quantity, a.ndim, g.spherical != 0, x, y, f);
                    else
                        q = rho ? 0.0 : -3.0;
                }
            } else {
                q = rho ? 0.0 : -3.0;
            }
        }
        mu = mu_max * (2.0 * s.next() - 1.0);
        if (a.dist_flag == 0) {
            double ftest = 1.0, fxp = 0.5, ptmp = 0.0;
            int jt = 0;
            while (ftest > fxp) {
                if (++jt > kMaxRejections) { atomicOr(status, kStatusStepLimit); break; }
                ptmp = (s.next() * (a.pmax - a.pmin) + a.pmin) / a.p0;
                fxp = ptmp * ptmp * exp(-(ptmp * ptmp));
                ftest = s.next() * (double)0.37f;
            }
            p = ptmp * a.p0;
        } else if (a.dist_flag == 2) {
            p = draw_p_power(a, s);
        }
        t = a.t_frame + s.next() * a.dt_mhd;
    } else {
        x = a.xpos;
        y = s.next() * (a.box[4] - a.box[1]) + a.box[1];
        z = s.next() * (a.box[5] - a.box[2]) + a.box[2];
        if (a.mode == 3) x = shock_x(a, y, z);
        if (a.dist_flag == 0) {
            double ftest = 1.0, fxp = 0.5, ptmp = 0.0;
            int it = 0;
            while (ftest > fxp) {
                if (++it > kMaxRejections) { atomicOr(status, kStatusStepLimit); break; }
                ptmp = (s.next() * (a.pmax - a.pmin) + a.pmin) / a.p0;
                fxp = ptmp * ptmp * exp((double)(-0.5f) * (ptmp * ptmp));
                ftest = s.next() * (double)0.75f;
            }
            p = ptmp * a.p0;
        } else if (a.dist_flag == 2) {
            p = draw_p_power(a, s);
        }
        mu = mu_max * (2.0 * s.next() - 1.0);
        t = a.t_frame;
    }
    const int64_t c = a.base + i;
    a.P.x[c] = x; a.P.y[c] = y; a.P.z[c] = z; a.P.p[c] = p;
    a.P.v[c] = a.particle_v0 * p / a.p0;
    a.P.mu[c] = mu; a.P.weight[c] = 1.0; a.P.t[c] = t; a.P.dt[c] = a.dt;
    a.P.split_times[c] = 0; a.P.count_flag[c] = 1; a.P.origin[c] = 0;
    a.P.nsteps_tracked[c] = 0; a.P.nsteps_pushed[c] = 0;
    a.P.tag_injected[c] = tag; a.P.tag_splitted[c] = 1; a.P.rng_ctr[c] = 0u;
}

// ---------------------------------------------------------------------------
// Block-tiled stable stream compaction: count per tile, scan the tile
// counts, scatter with warp-ballot prefixes.  The tile counts and offsets
// are the scratch buffer (2 * nblocks int64).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double split_threshold(double pmin_split, double p0, double ratio,
                                                  int k) {
    double rk = 1.0;
    for (int j = 0; j < k; ++j) rk = rk * ratio;
    return pmin_split * p0 * rk;
}

struct SplitRule {
    double ratio, pmin_split, p0, pmax;
};

// Adds a removed escaped particle to the escaped distribution
// (calc_escaped_distributions, diagnostics.f90:950-957): global p binning,
// column |count_flag|.
__device__ __forceinline__ void escaped_add(const EscHist &e, const DevParticles &P, int64_t i,
                                            int flag) {
    if (e.bins == nullptr || flag >= 0 || flag < -6) return;
    const double p = P.p[i], mu = P.mu[i];
    if (!(p > e.pmin && p <= e.pmax && mu >= -1.0 && mu <= 1.0)) return;
    const int ip = (int)floor((log10(p) - e.pmin_log) / e.dp_log);
    if (ip < 0 || ip >= e.npp) return;
    unsigned long long *b = e.bins + 3 * ((size_t)(-flag - 1) * e.npp + ip);
    atomicAdd(b, 1ull);
    atomic_add_fixed(b + 1, b + 2, P.weight[i]);
}

// mode 0: keep count_flag == INBOX; mode 1: split candidates; mode 2:
// escaped particles (count_flag < 0).
template <int MODE>
__device__ __forceinline__ bool select(const DevParticles &P, int64_t i, const SplitRule &r) {
    if (MODE == 0) return P.count_flag[i] == 1;
    if (MODE == 2) return P.count_flag[i] < 0;
    const double p = P.p[i];
    return p > split_threshold(r.pmin_split, r.p0, r.ratio, P.split_times[i]) && p <= r.pmax;
}

template <int MODE>
__global__ void __launch_bounds__(kScanThreads) tile_count_kernel(const DevParticles P, int64_t n,
                                                                  SplitRule r, long long *tile_counts,
                                                                  DevCounters *cnt, const EscHist esc_hist) {
    __shared__ int warp_tot[kScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kTile;
    int mine = 0, esc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k * kScanThreads + threadIdx.x;
        if (i < n) {
            mine += select<MODE>(P, i, r) ? 1 : 0;
            if (MODE == 0) {
                const int f = P.count_flag[i];
                if (f < 0) {
                    esc += 1;
                    escaped_add(esc_hist, P, i, f);
                }
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mine += __shfl_xor_sync(0xffffffffu, mine, o);
        esc += __shfl_xor_sync(0xffffffffu, esc, o);
    }
    if ((threadIdx.x & 31) == 0) {
        warp_tot[threadIdx.x >> 5] = mine;
        if (MODE == 0 && esc) atomicAdd(&cnt->nescaped, (unsigned long long)esc);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += warp_tot[w];
        tile_counts[blockIdx.x] = t;
    }
}

// Exclusive scan of the tile counts by one block; writes offsets and the total.
__global__ void __launch_bounds__(1024) tile_scan_kernel(const long long *tile_counts,
                                                         long long *tile_offsets, int64_t ntiles,
                                                         unsigned long long *total) {
    __shared__ long long warp_sums[32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < ntiles; base += 1024) {
        const int64_t i = base + threadIdx.x;
        const long long v = (i < ntiles) ? tile_counts[i] : 0;
        long long x = v;
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sums[wid] = x;
        __syncthreads();
        if (wid == 0) {
            long long ws = warp_sums[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long y = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += y;
            }
            warp_sums[lane] = ws;
        }
        __syncthreads();
        const long long excl = x - v + (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
        if (i < ntiles) tile_offsets[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = (unsigned long long)carry;
}

__device__ __forceinline__ void copy_particle(const DevParticles &S, int64_t i,
                                              const DevParticles &D, int64_t j) {
    D.x[j] = S.x[i]; D.y[j] = S.y[i]; D.z[j] = S.z[i]; D.p[j] = S.p[i];
    D.v[j] = S.v[i]; D.mu[j] = S.mu[i]; D.weight[j] = S.weight[i];
    D.t[j] = S.t[i]; D.dt[j] = S.dt[i];
    D.split_times[j] = S.split_times[i]; D.count_flag[j] = S.count_flag[i];
    D.origin[j] = S.origin[i]; D.nsteps_tracked[j] = S.nsteps_tracked[i];
    D.nsteps_pushed[j] = S.nsteps_pushed[i]; D.tag_injected[j] = S.tag_injected[i];
    D.tag_splitted[j] = S.tag_splitted[i]; D.rng_ctr[j] = S.rng_ctr[i];
}

// split_particle's branch for a tracked parent (particle_module.f90:5452-5474)
// once child c is a copy of parent i with split_times = kk + 1: the child's
// tag_splitted counts down, and child and parent each stay tracked (and
// record their state when the push count is 0) only if the table lists
// them at the new split level.
__device__ void split_tracked(const TrackArgs &t, const DevParticles &S, int64_t i, int64_t c,
                              int kk, DevCounters *cnt) {
    const int32_t tg = S.tag_splitted[i];
    const int32_t tc = (int32_t)((uint32_t)tg - (1u << kk));
    S.tag_splitted[c] = tc;
    const bool rec = S.nsteps_pushed[i] == 0;
    int lo, hi;
    if (trk_select(t, S.origin[c], S.tag_injected[c], kk + 1, tc, lo, hi)) {
        if (rec) {
            S.nsteps_tracked[c] += 1;
            trk_write(t, S.nsteps_tracked[c], lo, hi, trk_from(S, c), cnt);
        }
    } else {
        S.tag_splitted[c] = -tc;
    }
    if (trk_select(t, S.origin[i], S.tag_injected[i], kk + 1, tg, lo, hi)) {
        if (rec) {
            S.nsteps_tracked[i] += 1;
            trk_write(t, S.nsteps_tracked[i], lo, hi, trk_from(S, i), cnt);
        }
    } else {
        S.tag_splitted[i] = -tg;   // stop tracking
    }
}

// MODE 0: kept particles of S go to D in order.  MODE 1: S == D; each split
// candidate gets a child at n + rank (if < cap) and is updated in place.
// MODE 2: escaped particles go to D at cap + rank (cap is the base there).
template <int MODE>
__global__ void __launch_bounds__(kScanThreads) tile_scatter_kernel(
    const DevParticles S, const DevParticles D, int64_t n, int64_t cap, SplitRule r,
    const long long *tile_offsets, DevCounters *cnt, const TrackArgs trk) {
    __shared__ int warp_pre[kScanThreads / 32];
    __shared__ int sub_total;
    const int64_t base = (int64_t)blockIdx.x * kTile;
    long long running = tile_offsets[blockIdx.x];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int created = 0;
    for (int k = 0; k < kScanItems; ++k) {
        const int64_t i = base + k * kScanThreads + threadIdx.x;
        const bool sel = (i < n) && select<MODE>(S, i, r);
        const unsigned bal = __ballot_sync(0xffffffffu, sel);
        const int wpre = __popc(bal & ((1u << lane) - 1u));
        if (lane == 0) warp_pre[wid] = __popc(bal);
        __syncthreads();
        if (threadIdx.x == 0) {
            int acc = 0;
            for (int w = 0; w < kScanThreads / 32; ++w) {
                const int c = warp_pre[w];
                warp_pre[w] = acc;
                acc += c;
            }
            sub_total = acc;
        }
        __syncthreads();
        if (sel) {
            const long long rank = running + warp_pre[wid] + wpre;
            if (MODE == 0) {
                copy_particle(S, i, D, rank);
            } else if (MODE == 2) {
                copy_particle(S, i, D, cap + rank);
            } else {
                const int64_t c = n + rank;
                if (c < cap) {
                    const int kk = S.split_times[i];
                    S.weight[i] = ldexp(1.0, -(kk + 1));
                    S.split_times[i] = (int8_t)(kk + 1);
                    copy_particle(S, i, S, c);
                    if (trk.tags && S.tag_splitted[i] < 0)
                        split_tracked(trk, S, i, c, kk, cnt);
                    else
                        S.tag_splitted[c] = (int32_t)((uint32_t)S.tag_splitted[i] + (1u << kk));
                    created += 1;
                }
            }
        }
        running += sub_total;
        __syncthreads();
    }
    if (MODE == 1) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) created += __shfl_xor_sync(0xffffffffu, created, o);
        if (lane == 0 && created) atomicAdd(&cnt->nsplit, (unsigned long long)created);
    }
}

// ---------------------------------------------------------------------------
// Global f(p) histogram: block-private shared bins (count, weight hi, lo),
// warp-aggregated by bin with __match_any_sync, exact 128-bit weights.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) histogram_kernel(const DevParticles P, int64_t n, int npp,
                                                        double pmin, double pmax, double pmin_log,
                                                        double dp_log, unsigned long long *bins) {
    extern __shared__ unsigned long long sh[];  // 3 * npp
    for (int b = threadIdx.x; b < 3 * npp; b += blockDim.x) sh[b] = 0ull;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t iters = (n + stride - 1) / stride;
    for (int64_t it = 0; it < iters; ++it) {
        const int64_t i = start + it * stride;
        int bin = -1;
        unsigned long long wh = 0, wl = 0;
        if (i < n) {
            const double p = P.p[i], mu = P.mu[i];
            if (p > pmin && p <= pmax && mu >= -1.0 && mu <= 1.0) {
                const int ip = (int)floor((log10(p) - pmin_log) / dp_log);
                if (ip >= 0 && ip < npp) {
                    bin = ip;
                    fixed_split(P.weight[i], wh, wl);
                }
            }
        }
        const unsigned grp = __match_any_sync(0xffffffffu, bin);
        const int leader = __ffs(grp) - 1;
        unsigned long long sh_h = 0, sh_l = 0;
        unsigned m = grp;
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const unsigned long long oh = __shfl_sync(grp, wh, src);
            const unsigned long long ol = __shfl_sync(grp, wl, src);
            add_u128(sh_h, sh_l, oh, ol);
        }
        if (bin >= 0 && (int)(threadIdx.x & 31) == leader) {
            atomicAdd(&sh[3 * bin], (unsigned long long)__popc(grp));
            atomic_add_u128(&sh[3 * bin + 1], &sh[3 * bin + 2], sh_h, sh_l);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < npp; b += blockDim.x) {
        if (sh[3 * b]) atomicAdd(&bins[3 * b], sh[3 * b]);
        atomic_add_u128(&bins[3 * b + 1], &bins[3 * b + 2], sh[3 * b + 1], sh[3 * b + 2]);
    }
}

// ---------------------------------------------------------------------------
// quick_check: exact sums of weight and dt, min/max dt (positive doubles
// order like their bit patterns).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) quick_check_kernel(const DevParticles P, int64_t n,
                                                          DevCounters *cnt) {
    unsigned long long wh = 0, wl = 0, th = 0, tl = 0;
    double mn = 1.0, mx = 0.0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        unsigned long long h, l;
        fixed_split(P.weight[i], h, l);
        add_u128(wh, wl, h, l);
        const double dt = P.dt[i];
        fixed_split(dt, h, l);
        add_u128(th, tl, h, l);
        if (dt < mn) mn = dt;
        if (dt > mx) mx = dt;
    }
    warp_sum_u128(wh, wl);
    warp_sum_u128(th, tl);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_add_u128(&cnt->wsum_hi, &cnt->wsum_lo, wh, wl);
        atomic_add_u128(&cnt->dtsum_hi, &cnt->dtsum_lo, th, tl);
        if (mn >= 0.0)
            atomicMin(reinterpret_cast<unsigned long long *>(&cnt->dt_min),
                      (unsigned long long)__double_as_longlong(mn));
        if (mx >= 0.0)
            atomicMax(reinterpret_cast<unsigned long long *>(&cnt->dt_max),
                      (unsigned long long)__double_as_longlong(mx));
    }
}

// ---------------------------------------------------------------------------
// Spatial binning: counting sort of the in-box particles by grid cell, which
// also removes everything else (remove_particles).  Lanes of a warp then
// gather neighbouring field records.  Cells are the interpolation base cell
// (Fortran floor(px) + 1, i.e. C index floor(px) + 2); order inside a cell
// follows atomic arrival and is not reproducible, the particle set is.
// ---------------------------------------------------------------------------
constexpr int kBinScanThreads = 256;
constexpr int kBinScanItems = 8;
constexpr int kBinTile = kBinScanThreads * kBinScanItems;

// n_dev, when given, holds the particle count on the device (graph replays).
__global__ void __launch_bounds__(256) cell_key_kernel(const DevParticles P, int64_t n,
                                                       const unsigned long long *n_dev,
                                                       const CellGrid g, int32_t *keys,
                                                       unsigned int *counts, DevCounters *cnt,
                                                       const EscHist esc_hist) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n = (int64_t)*n_dev;
    int esc = 0;
    bool done = false;
    if (i < n) {
        const int flag = P.count_flag[i];
        int32_t key = -1;
        const bool spatial = !g.done_bin || g.all_active || *g.nactive == 0ull ||
                             (i < g.n_moved && g.pause[i] != 0);
        if (flag == 1 && !spatial) {
            // finished the interval: the trailing done bin (counted per warp
            // below: most particles of a late chunk land in this one bin)
            key = (int32_t)(cell_grid_bins(g) - 1);
            done = true;
        } else if (flag == 1 && g.tile) {
            // the mover's own cell (cell_of), so the particle lands in the
            // brick whose records are staged for it; clamped into the grid
            int cx, cy, cz = 0;
            float f;
            cell_of(P.x[i], g.xmin, g.dx, cx, f);
            cell_of(P.y[i], g.ymin, g.dy, cy, f);
            cx = min(max(cx + 2, 0), g.nxg - 1);
            cy = min(max(cy + 2, 0), g.nyg - 1);
            if (g.nzg > 1) {
                cell_of(P.z[i], g.zmin, g.dz, cz, f);
                cz = min(max(cz + 2, 0), g.nzg - 1);
            }
            const int bxi = cx / g.bx, byi = cy / g.by, bzi = cz / g.bz;
            const int lx = cx - bxi * g.bx, ly = cy - byi * g.by, lz = cz - bzi * g.bz;
            const int64_t brick = ((int64_t)bzi * g.nby + byi) * g.nbx + bxi;
            key = (int32_t)(brick * ((int64_t)g.bx * g.by * g.bz) + (lz * g.by + ly) * g.bx + lx);
            atomicAdd(&counts[key], 1u);
        } else if (flag == 1) {
            const double px = (P.x[i] - g.xmin) * g.idx;
            const double py = (P.y[i] - g.ymin) * g.idy;
            int cx = (int)floor(fmin(fmax(px, -2.0), (double)g.nxg)) + 2;
            int cy = (int)floor(fmin(fmax(py, -2.0), (double)g.nyg)) + 2;
            cx = min(max(cx, 0), g.nxg - 1);
            cy = min(max(cy, 0), g.nyg - 1);
            int cz = 0;
            if (g.nzg > 1) {
                const double pz = (P.z[i] - g.zmin) * g.idz;
                cz = (int)floor(fmin(fmax(pz, -2.0), (double)g.nzg)) + 2;
                cz = min(max(cz, 0), g.nzg - 1);
            }
            key = cx + g.nxg * (cy + g.nyg * cz);
            atomicAdd(&counts[key], 1u);
        } else if (flag < 0) {
            esc = 1;
            escaped_add(esc_hist, P, i, flag);
        }
        keys[i] = key;
    }
    const unsigned dm = __ballot_sync(0xffffffffu, done);
    if ((threadIdx.x & 31) == 0 && dm)
        atomicAdd(&counts[cell_grid_bins(g) - 1], (unsigned)__popc(dm));
    const unsigned e = __ballot_sync(0xffffffffu, esc);
    if ((threadIdx.x & 31) == 0 && e) atomicAdd(&cnt->nescaped, (unsigned long long)__popc(e));
}

__global__ void __launch_bounds__(kBinScanThreads) bin_tile_sum_kernel(const unsigned int *counts,
                                                                       int64_t nbins,
                                                                       long long *tile_sums) {
    __shared__ unsigned int warp_tot[kBinScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kBinTile;
    unsigned int s = 0;
#pragma unroll
    for (int k = 0; k < kBinScanItems; ++k) {
        const int64_t b = base + k * kBinScanThreads + threadIdx.x;
        if (b < nbins) s += counts[b];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) warp_tot[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long t = 0;
        for (int w = 0; w < kBinScanThreads / 32; ++w) t += warp_tot[w];
        tile_sums[blockIdx.x] = t;
    }
}

// In-place exclusive scan of the bin counts, one tile of kBinTile bins per
// block, offset by the scanned tile sums.  Each thread owns kBinScanItems
// consecutive bins.
__global__ void __launch_bounds__(kBinScanThreads) bin_tile_scan_kernel(unsigned int *counts,
                                                                        int64_t nbins,
                                                                        const long long *tile_offsets) {
    __shared__ unsigned int warp_pre[kBinScanThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kBinTile + (int64_t)threadIdx.x * kBinScanItems;
    unsigned int v[kBinScanItems];
    unsigned int mine = 0;
#pragma unroll
    for (int k = 0; k < kBinScanItems; ++k) {
        v[k] = (base + k < nbins) ? counts[base + k] : 0u;
        mine += v[k];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned int x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_pre[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned int acc = 0;
        for (int w = 0; w < kBinScanThreads / 32; ++w) {
            const unsigned int c = warp_pre[w];
            warp_pre[w] = acc;
            acc += c;
        }
    }
    __syncthreads();
    unsigned int run = (unsigned int)tile_offsets[blockIdx.x] + warp_pre[wid] + (x - mine);
#pragma unroll
    for (int k = 0; k < kBinScanItems; ++k) {
        if (base + k < nbins) counts[base + k] = run;
        run += v[k];
    }
}

// done_key: the trailing done bin (-1: none), whose slots are reserved per
// warp, one atomic for all its lanes that go there.
__global__ void __launch_bounds__(256) cell_scatter_kernel(const DevParticles S, const DevParticles D,
                                                           int64_t n,
                                                           const unsigned long long *n_dev,
                                                           const int32_t *keys,
                                                           unsigned int *cursor, int32_t done_key) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n_dev) n = (int64_t)*n_dev;
    const int32_t key = i < n ? keys[i] : -1;
    const unsigned dm = __ballot_sync(0xffffffffu, key >= 0 && key == done_key);
    unsigned int pos = 0;
    if (dm) {
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(dm) - 1;
        unsigned int base = 0;
        if (lane == leader) base = atomicAdd(&cursor[done_key], (unsigned)__popc(dm));
        base = __shfl_sync(0xffffffffu, base, leader);
        pos = base + (unsigned)__popc(dm & ((1u << lane) - 1u));
    }
    if (key < 0) return;
    if (key != done_key) pos = atomicAdd(&cursor[key], 1u);
    copy_particle(S, i, D, (int64_t)pos);
}

}  // namespace

__host__ __device__ int64_t cell_grid_bins(const CellGrid &g) {
    const int64_t spatial = g.tile ? (int64_t)g.nbx * g.nby * g.nbz * ((int64_t)g.bx * g.by * g.bz)
                                   : (int64_t)g.nxg * g.nyg * g.nzg;
    return spatial + (g.done_bin ? 1 : 0);
}

const unsigned int *cell_sort_counts(const void *scratch, int64_t nbins) {
    const int64_t ntiles = (nbins + kBinTile - 1) / kBinTile;
    const long long *tile_sums = static_cast<const long long *>(scratch);
    return reinterpret_cast<const unsigned int *>(tile_sums + 2 * (ntiles + 1));
}

size_t cell_sort_scratch_bytes(int64_t cap, int64_t nbins) {
    const int64_t ntiles = (nbins + kBinTile - 1) / kBinTile;
    return (size_t)cap * 4 + (size_t)nbins * 4 + (size_t)(2 * ntiles + 2) * 8 + 256;
}

cudaError_t launch_cell_sort(const DevParticles &src, const DevParticles &dst, int64_t n,
                             const CellGrid &g, void *scratch, DevCounters *cnt,
                             const EscHist &esc, cudaStream_t s) {
    const int64_t nbins = cell_grid_bins(g);
    const int64_t ntiles = (nbins + kBinTile - 1) / kBinTile;
    char *q = static_cast<char *>(scratch);
    long long *tile_sums = reinterpret_cast<long long *>(q);
    long long *tile_offsets = tile_sums + ntiles + 1;
    unsigned int *counts = reinterpret_cast<unsigned int *>(tile_offsets + ntiles + 1);
    int32_t *keys = reinterpret_cast<int32_t *>(counts + nbins);
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(unsigned int) * (size_t)nbins, s);
    if (e != cudaSuccess) return e;
    if (n <= 0) return cudaMemsetAsync(&cnt->nkept, 0, sizeof(unsigned long long), s);
    const unsigned blocks = (unsigned)((n + 255) / 256);
    cell_key_kernel<<<blocks, 256, 0, s>>>(src, n, nullptr, g, keys, counts, cnt, esc);
    bin_tile_sum_kernel<<<(unsigned)ntiles, kBinScanThreads, 0, s>>>(counts, nbins, tile_sums);
    tile_scan_kernel<<<1, 1024, 0, s>>>(tile_sums, tile_offsets, ntiles, &cnt->nkept);
    bin_tile_scan_kernel<<<(unsigned)ntiles, kBinScanThreads, 0, s>>>(counts, nbins, tile_offsets);
    cell_scatter_kernel<<<blocks, 256, 0, s>>>(src, dst, n, nullptr, keys, counts,
                                               g.done_bin ? (int32_t)(nbins - 1) : -1);
    return cudaGetLastError();
}

cudaError_t launch_cell_sort_dev(const DevParticles &src, const DevParticles &dst,
                                 unsigned long long *n_dev, int64_t cap, const CellGrid &g,
                                 void *scratch, DevCounters *cnt, const EscHist &esc,
                                 cudaStream_t s) {
    const int64_t nbins = cell_grid_bins(g);
    const int64_t ntiles = (nbins + kBinTile - 1) / kBinTile;
    char *q = static_cast<char *>(scratch);
    long long *tile_sums = reinterpret_cast<long long *>(q);
    long long *tile_offsets = tile_sums + ntiles + 1;
    unsigned int *counts = reinterpret_cast<unsigned int *>(tile_offsets + ntiles + 1);
    int32_t *keys = reinterpret_cast<int32_t *>(counts + nbins);
    cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(unsigned int) * (size_t)nbins, s);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)((cap + 255) / 256);
    if (blocks == 0) return cudaSuccess;
    cell_key_kernel<<<blocks, 256, 0, s>>>(src, 0, n_dev, g, keys, counts, cnt, esc);
    bin_tile_sum_kernel<<<(unsigned)ntiles, kBinScanThreads, 0, s>>>(counts, nbins, tile_sums);
    tile_scan_kernel<<<1, 1024, 0, s>>>(tile_sums, tile_offsets, ntiles, &cnt->nkept);
    bin_tile_scan_kernel<<<(unsigned)ntiles, kBinScanThreads, 0, s>>>(counts, nbins, tile_offsets);
    cell_scatter_kernel<<<blocks, 256, 0, s>>>(src, dst, 0, n_dev, keys, counts,
                                               g.done_bin ? (int32_t)(nbins - 1) : -1);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(n_dev, &cnt->nkept, sizeof(unsigned long long),
                           cudaMemcpyDeviceToDevice, s);
}

size_t compaction_scratch_bytes(int64_t n) {
    const int64_t ntiles = (n + kTile - 1) / kTile;
    return (size_t)(2 * (ntiles > 0 ? ntiles : 1)) * sizeof(long long);
}

cudaError_t launch_remove_particles(const DevParticles &src, const DevParticles &dst, int64_t n,
                                    void *scratch, DevCounters *cnt, const EscHist &esc,
                                    cudaStream_t s) {
    if (n <= 0) return cudaMemsetAsync(&cnt->nkept, 0, sizeof(unsigned long long), s);
    const int64_t ntiles = (n + kTile - 1) / kTile;
    long long *counts = static_cast<long long *>(scratch);
    long long *offsets = counts + ntiles;
    const SplitRule r{0, 0, 0, 0};
    tile_count_kernel<0><<<(unsigned)ntiles, kScanThreads, 0, s>>>(src, n, r, counts, cnt, esc);
    tile_scan_kernel<<<1, 1024, 0, s>>>(counts, offsets, ntiles, &cnt->nkept);
    tile_scatter_kernel<0><<<(unsigned)ntiles, kScanThreads, 0, s>>>(src, dst, n, n, r, offsets, cnt,
                                                                     TrackArgs{});
    return cudaGetLastError();
}

cudaError_t launch_select_escaped(const DevParticles &src, int64_t n, const DevParticles &dst,
                                  int64_t base, void *scratch, DevCounters *cnt, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(&cnt->nselected, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess || n <= 0) return e;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    long long *counts = static_cast<long long *>(scratch);
    long long *offsets = counts + ntiles;
    const SplitRule r{0, 0, 0, 0};
    const EscHist none{nullptr, 0, 0.0, 0.0, 0.0, 0.0};
    tile_count_kernel<2><<<(unsigned)ntiles, kScanThreads, 0, s>>>(src, n, r, counts, cnt, none);
    tile_scan_kernel<<<1, 1024, 0, s>>>(counts, offsets, ntiles, &cnt->nselected);
    tile_scatter_kernel<2><<<(unsigned)ntiles, kScanThreads, 0, s>>>(src, dst, n, base, r,
                                                                     offsets, cnt, TrackArgs{});
    return cudaGetLastError();
}

cudaError_t launch_split_particles(const DevParticles &P, int64_t n, int64_t cap,
                                   double split_ratio, double pmin_split, double p0, double pmax,
                                   void *scratch, DevCounters *cnt, cudaStream_t s,
                                   const TrackArgs *trk) {
    // nkept is read back as the number of split candidates
    if (n <= 0) return cudaMemsetAsync(&cnt->nkept, 0, sizeof(unsigned long long), s);
    const int64_t ntiles = (n + kTile - 1) / kTile;
    long long *counts = static_cast<long long *>(scratch);
    long long *offsets = counts + ntiles;
    const SplitRule r{split_ratio, pmin_split, p0, pmax};
    const EscHist none{nullptr, 0, 0.0, 0.0, 0.0, 0.0};
    tile_count_kernel<1><<<(unsigned)ntiles, kScanThreads, 0, s>>>(P, n, r, counts, cnt, none);
    tile_scan_kernel<<<1, 1024, 0, s>>>(counts, offsets, ntiles, &cnt->nkept);
    tile_scatter_kernel<1><<<(unsigned)ntiles, kScanThreads, 0, s>>>(P, P, n, cap, r, offsets, cnt,
                                                                     trk ? *trk : TrackArgs{});
    return cudaGetLastError();
}

namespace {

// inject_one_particle's tracking block (particle_module.f90:434-440; the
// same at :622-628): a new particle the table lists is tracked from its
// first record.
__global__ void __launch_bounds__(256) track_injected_kernel(const DevParticles P, int64_t first,
                                                             int64_t n, const TrackArgs t,
                                                             DevCounters *cnt) {
    const int64_t i = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo, hi;
    if (!trk_select(t, P.origin[i], P.tag_injected[i], P.split_times[i], P.tag_splitted[i], lo,
                    hi))
        return;
    P.nsteps_tracked[i] = 1;
    P.tag_injected[i] = -P.tag_injected[i];
    P.tag_splitted[i] = -1;
    trk_write(t, 1, lo, hi, trk_from(P, i), cnt);
}

__device__ __forceinline__ void trk_store(const DevParticles &D, size_t e, const TrkRecord &r) {
    D.x[e] = r.x; D.y[e] = r.y; D.z[e] = r.z; D.p[e] = r.p; D.v[e] = r.v; D.mu[e] = r.mu;
    D.weight[e] = r.w; D.t[e] = r.t; D.dt[e] = r.dt;
    D.split_times[e] = (int8_t)r.split_times; D.count_flag[e] = (int8_t)r.count_flag;
    D.origin[e] = r.origin; D.nsteps_tracked[e] = r.nsteps_tracked;
    D.nsteps_pushed[e] = r.nsteps_pushed;
    D.tag_injected[e] = r.tag_inj; D.tag_splitted[e] = r.tag_spl;
    D.rng_ctr[e] = r.ctr;
}

// sync_tracked_particles on one rank: one warp per column compacts the rows
// with tag_splitted < 0 to the front in order (32 rows at a time, every
// lane reading before any lane writes; a kept row only moves up) and zeroes
// the rest.
__global__ void __launch_bounds__(256) sync_tracked_kernel(const TrackArgs t) {
    const int col = (int)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5));
    if (col >= t.n) return;
    const int lane = threadIdx.x & 31;
    const DevParticles &D = t.rec;
    const size_t base = (size_t)t.nsteps_max * (size_t)col;
    int64_t kept = 0;
    for (int64_t r0 = 0; r0 < t.nsteps_max; r0 += 32) {
        const int64_t r = r0 + lane;
        bool keep = false;
        TrkRecord rec{};
        if (r < t.nsteps_max && D.tag_splitted[base + r] < 0) {
            keep = true;
            rec = trk_from(D, (int64_t)(base + r));
        }
        __syncwarp();   // every read of this block of rows before any write
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (keep) trk_store(D, base + kept + __popc(bal & ((1u << lane) - 1u)), rec);
        kept += __popc(bal);
        __syncwarp();
    }
    const TrkRecord zero{};
    for (int64_t r = kept + lane; r < t.nsteps_max; r += 32) trk_store(D, base + r, zero);
}

}  // namespace

cudaError_t launch_track_injected(const DevParticles &P, int64_t first, int64_t n,
                                  const TrackArgs &trk, DevCounters *cnt, cudaStream_t s) {
    if (!trk.tags || n <= first) return cudaSuccess;
    const int64_t m = n - first;
    track_injected_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(P, first, n, trk, cnt);
    return cudaGetLastError();
}

namespace {

// Non-negative doubles order like their bit patterns, so the maximum is an
// integer atomicMax of the bits (p <= 0 and NaN are left out; the start is
// +0.0).
__global__ void __launch_bounds__(256) pmax_kernel(const DevParticles P, int64_t n,
                                                   unsigned long long *bits) {
    unsigned long long m = 0ull;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double p = P.p[i];
        if (p > 0.0) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(p);
            if (b > m) m = b;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xffffffffu, m, o);
        if (v > m) m = v;
    }
    if ((threadIdx.x & 31) == 0 && m) atomicMax(bits, m);
}

}  // namespace

cudaError_t launch_pmax(const DevParticles &P, int64_t n, unsigned long long *bits,
                        cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    pmax_kernel<<<(unsigned)blocks, 256, 0, s>>>(P, n, bits);
    return cudaGetLastError();
}

cudaError_t launch_sync_tracked(const TrackArgs &trk, cudaStream_t s) {
    if (!trk.tags || trk.n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((trk.n + 7) / 8);
    sync_tracked_kernel<<<blocks, 256, 0, s>>>(trk);
    return cudaGetLastError();
}

cudaError_t launch_histogram(const DevParticles &P, int64_t n, int npp, double pmin, double pmax,
                             unsigned long long *bins, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bins, 0, sizeof(unsigned long long) * 3 * (size_t)npp, s);
    if (e != cudaSuccess || n <= 0) return e;
    const double pmin_log = log10(pmin), pmax_log = log10(pmax);
    const double dp_log = (pmax_log - pmin_log) / npp;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    const size_t shmem = sizeof(unsigned long long) * 3 * (size_t)npp;
    histogram_kernel<<<(unsigned)blocks, 256, shmem, s>>>(P, n, npp, pmin, pmax, pmin_log, dp_log,
                                                          bins);
    return cudaGetLastError();
}

// The bins of particle i for one local-distribution parameter set
// (diagnostics.f90:785-800): spatial ix, iy, iz, momentum ip, pitch imu and
// the weight (over r^2 sin(theta) in spherical coordinates, :765-772).
struct LocalBin {
    int ix, iy, iz, ip, imu;
    double w;
};

__device__ __forceinline__ LocalBin local_bin(const DevParticles &P, int64_t i,
                                              const LocalDistArgs &a) {
    LocalBin b;
    const double p = P.p[i], mu = P.mu[i];
    int ix, iy, iz;
    if (a.nonuniform) {
        // (binarySearch_R(xpos_local, x) - 1) / rx + 1 (diagnostics.f90:790-792)
        ix = (grid_count(a.xpos, a.nxg, P.x[i]) - 1) / a.rx + 1;
        // 1D runs keep no y positions (ypos_global is never set there)
        iy = (a.ndim > 1) ? (grid_count(a.ypos, a.nyg, P.y[i]) - 1) / a.ry + 1
                          : (int)floor((P.y[i] - a.ymin) / a.dyd) + 1;
        iz = (a.ndim == 3) ? (grid_count(a.zpos, a.nzg, P.z[i]) - 1) / a.rz + 1
                           : (int)floor((P.z[i] - a.zmin) / a.dzd) + 1;
    } else {
        ix = (int)floor((P.x[i] - a.xmin) / a.dxd) + 1;
        iy = (int)floor((P.y[i] - a.ymin) / a.dyd) + 1;
        iz = (int)floor((P.z[i] - a.zmin) / a.dzd) + 1;
    }
    b.ix = ix; b.iy = iy; b.iz = iz;
    b.ip = (int)floor((log10(p) - a.pmin_log) / a.dp_log) + 1;
    b.imu = (int)floor((mu + 1.0) / a.dmu) + 1;
    double w = P.weight[i];
    if (a.spherical) {
        // F = f p^2 r^2 (sin theta from 2D on), diagnostics.f90:765-772
        w = w / (P.x[i] * P.x[i]);
        if (a.ndim >= 2) w = w / sin(P.y[i]);
    }
    b.w = w;
    return b;
}

__device__ __forceinline__ void bin_add(unsigned long long *bins, size_t e, double w) {
    unsigned long long *b = bins + 3 * e;
    atomicAdd(b, 1ull);
    atomic_add_fixed(b + 1, b + 2, w);
}

// Local distributions (calc_particle_distributions, diagnostics.f90:782-878):
// one (count, weight hi, lo) triple per flocal element.
__global__ void __launch_bounds__(256) local_dist_kernel(const DevParticles P, int64_t n,
                                                         const LocalDistArgs a,
                                                         unsigned long long *bins) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const LocalBin b = local_bin(P, i, a);
    if (b.ix < 1 || b.ix > a.nrx || b.iy < 1 || b.iy > a.nry || b.iz < 1 || b.iz > a.nrz) return;
    if (!(b.ip > 0 && b.ip < a.npb) || b.imu < 1 || b.imu > a.nmu) return;
    const size_t e = (size_t)(b.imu - 1) +
                     (size_t)a.nmu * ((size_t)(b.ip - 1) +
                                      (size_t)a.npb * ((size_t)(b.ix - 1) +
                                                       (size_t)a.nrx * ((size_t)(b.iy - 1) +
                                                                        (size_t)a.nry * (b.iz - 1))));
    bin_add(bins, e, b.w);
}

// Local escaped distributions (calc_escaped_distributions, diagnostics.f90:
// 958-1230) over escaped particles: the x faces into fx(nmu, npb, nry, nrz,
// 2), the y faces into fy(nmu, npb, nrx, nrz, 2) and the z faces into
// fz(nmu, npb, nrx, nry, 2), low face first; a face whose array the
// reference does not allocate (y below 2D, z below 3D) is skipped.
__global__ void __launch_bounds__(256) local_escaped_kernel(const DevParticles P, int64_t n,
                                                            const LocalDistArgs a,
                                                            unsigned long long *fx,
                                                            unsigned long long *fy,
                                                            unsigned long long *fz) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const LocalBin b = local_bin(P, i, a);
    if (!(b.ip > 0 && b.ip < a.npb) || b.imu < 1 || b.imu > a.nmu) return;
    const bool cx = b.ix >= 1 && b.ix <= a.nrx, cy = b.iy >= 1 && b.iy <= a.nry;
    const bool cz = b.iz >= 1 && b.iz <= a.nrz;
    const int flag = P.count_flag[i];
    const size_t mp = (size_t)(b.imu - 1) + (size_t)a.nmu * (size_t)(b.ip - 1);
    const size_t nmp = (size_t)a.nmu * (size_t)a.npb;
    if ((flag == -1 || flag == -2) && cy && cz && fx) {
        const size_t side = (size_t)(-flag - 1);
        bin_add(fx, mp + nmp * ((size_t)(b.iy - 1) + (size_t)a.nry * ((size_t)(b.iz - 1) +
                                                                       (size_t)a.nrz * side)),
                b.w);
    } else if ((flag == -3 || flag == -4) && a.ndim > 1 && cx && cz && fy) {
        const size_t side = (size_t)(-flag - 3);
        bin_add(fy, mp + nmp * ((size_t)(b.ix - 1) + (size_t)a.nrx * ((size_t)(b.iz - 1) +
                                                                       (size_t)a.nrz * side)),
                b.w);
    } else if ((flag == -5 || flag == -6) && a.ndim > 2 && cx && cy && fz) {
        const size_t side = (size_t)(-flag - 5);
        bin_add(fz, mp + nmp * ((size_t)(b.ix - 1) + (size_t)a.nrx * ((size_t)(b.iy - 1) +
                                                                       (size_t)a.nry * side)),
                b.w);
    }
}

// Global distribution with pitch-angle bins (calc_particle_distributions
// :773-779, calc_escaped_distributions :949-957): fglobal(nmu, npp) or, with
// by_face, fescaped(nmu, npp, |count_flag|); the particle's own weight.
// p == pmax and mu == 1 index past the last bin in the reference and are
// dropped.
__device__ __forceinline__ int64_t mu_bin(const DevParticles &P, int64_t i, const MuDistArgs &a) {
    const double p = P.p[i], mu = P.mu[i];
    if (!(p > a.pmin && p <= a.pmax && mu >= -1.0 && mu <= 1.0)) return -1;
    const int ip = (int)floor((log10(p) - a.pmin_log) / a.dp_log) + 1;
    const int imu = (int)floor((mu + 1.0) / a.dmu) + 1;
    if (ip < 1 || ip > a.npp || imu < 1 || imu > a.nmu) return -1;
    int64_t face = 0;
    if (a.by_face) {
        const int flag = P.count_flag[i];
        if (flag >= 0 || flag < -6) return -1;
        face = -flag - 1;
    }
    return (int64_t)(imu - 1) + (int64_t)a.nmu * ((int64_t)(ip - 1) + (int64_t)a.npp * face);
}

__global__ void __launch_bounds__(256) mu_dist_kernel(const DevParticles P, int64_t n,
                                                      const MuDistArgs a,
                                                      unsigned long long *bins) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t b = mu_bin(P, i, a);
    if (b >= 0) bin_add(bins, (size_t)b, P.weight[i]);
}

// The same with block-private bins in shared memory (nbins triples) and
// lanes of a warp that share a bin merged first, as histogram_kernel does.
__global__ void __launch_bounds__(256) mu_dist_shared_kernel(const DevParticles P, int64_t n,
                                                             const MuDistArgs a, int nbins,
                                                             unsigned long long *bins) {
    extern __shared__ unsigned long long sh[];
    for (int b = threadIdx.x; b < 3 * nbins; b += blockDim.x) sh[b] = 0ull;
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t start = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t iters = (n + stride - 1) / stride;
    for (int64_t it = 0; it < iters; ++it) {
        const int64_t i = start + it * stride;
        int bin = -1;
        unsigned long long wh = 0, wl = 0;
        if (i < n) {
            bin = (int)mu_bin(P, i, a);
            if (bin >= 0) fixed_split(P.weight[i], wh, wl);
        }
        const unsigned grp = __match_any_sync(0xffffffffu, bin);
        const int leader = __ffs(grp) - 1;
        unsigned long long sh_h = 0, sh_l = 0;
        unsigned m = grp;
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const unsigned long long oh = __shfl_sync(grp, wh, src);
            const unsigned long long ol = __shfl_sync(grp, wl, src);
            add_u128(sh_h, sh_l, oh, ol);
        }
        if (bin >= 0 && (int)(threadIdx.x & 31) == leader) {
            atomicAdd(&sh[3 * bin], (unsigned long long)__popc(grp));
            atomic_add_u128(&sh[3 * bin + 1], &sh[3 * bin + 2], sh_h, sh_l);
        }
    }
    __syncthreads();
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) {
        if (sh[3 * b]) atomicAdd(&bins[3 * b], sh[3 * b]);
        atomic_add_u128(&bins[3 * b + 1], &bins[3 * b + 2], sh[3 * b + 1], sh[3 * b + 2]);
    }
}

// Largest table the shared-memory path holds: 8192 triples, 192 KiB.
constexpr int kMuSharedBins = 8192;

cudaError_t launch_local_dist(const DevParticles &P, int64_t n, const LocalDistArgs &a,
                              unsigned long long *bins, size_t nbins, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bins, 0, sizeof(unsigned long long) * 3 * nbins, s);
    if (e != cudaSuccess || n <= 0) return e;
    local_dist_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, n, a, bins);
    return cudaGetLastError();
}

cudaError_t launch_local_escaped(const DevParticles &P, int64_t n, const LocalDistArgs &a,
                                 unsigned long long *fx, unsigned long long *fy,
                                 unsigned long long *fz, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    local_escaped_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, n, a, fx, fy, fz);
    return cudaGetLastError();
}

cudaError_t launch_mu_dist(const DevParticles &P, int64_t n, const MuDistArgs &a,
                           unsigned long long *bins, size_t nbins, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(bins, 0, sizeof(unsigned long long) * 3 * nbins, s);
    if (e != cudaSuccess || n <= 0) return e;
    if (nbins <= (size_t)kMuSharedBins) {
        const size_t shmem = sizeof(unsigned long long) * 3 * nbins;
        // per device, so set on every call (it is cheap)
        e = cudaFuncSetAttribute(mu_dist_shared_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(unsigned long long) * 3 * kMuSharedBins));
        if (e != cudaSuccess) return e;
        int64_t blocks = (n + 255) / 256;
        if (blocks > 1024) blocks = 1024;
        mu_dist_shared_kernel<<<(unsigned)blocks, 256, shmem, s>>>(P, n, a, (int)nbins, bins);
    } else {
        mu_dist_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, n, a, bins);
    }
    return cudaGetLastError();
}

cudaError_t launch_quick_check(const DevParticles &P, int64_t n, DevCounters *cnt, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 2048) blocks = 2048;
    quick_check_kernel<<<(unsigned)blocks, 256, 0, s>>>(P, n, cnt);
    return cudaGetLastError();
}

namespace {

// get_ncells_large_* (mhd_data_parallel.f90:2211-2498) over the nodes
// ix = 1..nx (position xmin + (ix - 1) dx), single-precision quantities as
// the reference's real(sp) arrays give them.
__global__ void count_large_kernel(const LargeArgs g, int ndim, double b0, double b1, double b2,
                                   double b3, double b4, double b5,
                                   unsigned long long *ncells) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = (int64_t)g.nx * g.ny * g.nz;
    bool hit = false;
    if (i < n) {
        const int ix = (int)(i % g.nx) + 1;
        const int iy = (int)((i / g.nx) % g.ny) + 1;
        const int iz = (int)(i / ((int64_t)g.nx * g.ny)) + 1;
        const bool grid = g.spherical || g.nonuniform;
        // xpos_local(ix) is node ix + 1 of the ghost-padded positions
        const double xp = grid ? g.xpos[ix + 1] : g.dx * (double)(ix - 1) + g.gxmin;
        const double yp = grid ? g.ypos[iy + 1] : g.dy * (double)(iy - 1) + g.gymin;
        const double zp = (grid && ndim == 3) ? g.zpos[iz + 1] : g.dz * (double)(iz - 1) + g.gzmin;
        bool in = xp > b0 && xp < b3;
        if (ndim > 1) in = in && yp > b1 && yp < b4;
        if (ndim > 2) in = in && zp > b2 && zp < b5;
        if (in) {
            const int cz = (ndim == 3) ? iz + 1 : 0;
            const float *r = g.full + 32 * ((size_t)(ix + 1) + (size_t)g.nxg *
                                            ((size_t)(iy + 1) + (size_t)g.nyg * (size_t)cz));
            double q;
            if (g.spherical && g.quantity == GPAT_LARGE_JZ) {
                // :2226-2234, (by - dbx_dy) in single precision
                const float t = r[5] - r[21];
                q = fabs((double)r[23] + (double)t / xp);
            } else if (g.spherical && g.quantity == GPAT_LARGE_ABSJ) {
                // :2285-2303
                const double stheta = sin(yp), ctheta = cos(yp);
                const double t1 = (ctheta * (double)r[6] + stheta * (double)r[27] - (double)r[25]) /
                                  (xp * stheta);
                const double t2 = ((double)r[22] / stheta - (double)r[6] - xp * (double)r[26]) / xp;
                const double t3 = ((double)r[5] - xp * (double)r[23] - (double)r[21]) / xp;
                q = sqrt(t1 * t1 + t2 * t2 + t3 * t3);
            } else if (g.spherical && g.quantity == GPAT_LARGE_DIVV) {
                // :2404-2420: ctheta and istheta are re-allocated over all
                // ny + 4 nodes, so row iy reads node iy - 2 (memory iy - 1);
                // the dvz/dz term is added from ndim > 1; 2.0 * vx is single.
                const double yq = g.ypos[iy - 1];
                const double ctheta = cos(yq), istheta = 1.0 / sin(yq);
                const float vx2 = 2.0f * r[0];
                double d = (double)r[8] + (double)vx2 / xp;
                if (ndim > 1) {
                    d = d + ((double)r[12] + (double)r[1] * ctheta * istheta) / xp;
                    d = d + (double)r[16] * istheta / xp;
                }
                q = -d;
            } else if (g.quantity == GPAT_LARGE_JZ) {
                q = (double)fabsf(r[23] - r[21]);
            } else if (g.quantity == GPAT_LARGE_ABSJ) {
                const float t1 = r[25] - r[27], t2 = r[26] - r[22], t3 = r[21] - r[23];
                q = (double)sqrtf(t1 * t1 + t2 * t2 + t3 * t3);
            } else if (g.quantity == GPAT_LARGE_DIVV) {
                // divv = farray1(nfields+1, :, :, :) re-allocates divv over
                // the ghost-padded extent with lower bound 1, so node (ix, iy,
                // iz) reads the value two nodes lower along each axis.
                const int sz = (ndim == 3) ? iz - 1 : 0;
                const float *u = g.full + 32 * ((size_t)(ix - 1) + (size_t)g.nxg *
                                                ((size_t)(iy - 1) + (size_t)g.nyg * (size_t)sz));
                double d = (double)u[8];
                d = d + (double)u[12];
                if (ndim > 2) d = d + (double)u[16];
                q = -d;
            } else if (g.quantity == GPAT_LARGE_DB2) {
                q = (double)g.aux[16 * ((size_t)(ix + 1) + (size_t)g.nxg *
                                        ((size_t)(iy + 1) + (size_t)g.nyg * (size_t)cz))];
            } else {
                q = (double)r[3];
            }
            hit = q > g.qmin;
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(ncells, (unsigned long long)__popc(m));
}

}  // namespace

cudaError_t launch_count_large(const LargeArgs &lg, int ndim, const double box[6],
                               unsigned long long *ncells, cudaStream_t s) {
    const int64_t n = (int64_t)lg.nx * lg.ny * lg.nz;
    if (n <= 0) return cudaSuccess;
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    count_large_kernel<<<(unsigned)blocks, threads, 0, s>>>(lg, ndim, box[0], box[1], box[2],
                                                             box[3], box[4], box[5], ncells);
    return cudaGetLastError();
}

cudaError_t launch_locate_shock(const float *full, int nxg, int nrows, int32_t *shock_ix,
                                cudaStream_t s) {
    if (nrows <= 0) return cudaSuccess;
    locate_shock_kernel<<<(unsigned)((nrows + 7) / 8), 256, 0, s>>>(full, nxg, nrows, shock_ix);
    return cudaGetLastError();
}

cudaError_t launch_inject(const InjectArgs &a, unsigned int *status, cudaStream_t s) {
    if (a.count <= 0) return cudaSuccess;
    const int threads = 128;
    const int64_t blocks = (a.count + threads - 1) / threads;
    inject_kernel<<<(unsigned)blocks, threads, 0, s>>>(a, status);
    return cudaGetLastError();
}

}  // namespace gpat
