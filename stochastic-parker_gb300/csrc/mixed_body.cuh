// Per-particle body of the split-precision mover, shared by the kernel that
// gathers field records from global memory (mover_mixed.cu) and the kernel
// that stages bricks of records in shared memory (mover_tile.cu).  The gather
// is a policy: GlobalGather reads the packed records in HBM through L1/L2,
// TileGather reads a brick staged in shared memory and makes a particle that
// leaves the brick pause between pushes, as at the end of a chunk.
#pragma once

#include <cfloat>
#include <cmath>

#include "cell_index.cuh"
#include "device_common.cuh"

namespace gpat {

namespace {

// Kahan-compensated running sum: the value is s - c.
__device__ __forceinline__ void kadd(float &s, float &c, float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ __forceinline__ float fsqrt(float x) { return x > 0.0f ? x * rsqrtf(x) : 0.0f; }

// Adds d cells to (c, f), keeping f in [0, 1).
__device__ __forceinline__ void advance(int &c, float &f, float d) {
    f += d;
    const float fl = floorf(f);
    f -= fl;
    c += (int)fl;
    if (f >= 1.0f) { f -= 1.0f; c += 1; }
}

// Boundary test along one axis in cell units.  ext: the half-cell-extended
// box (period n + 1 cells); otherwise the exact box (period n).
__device__ __forceinline__ void bc_axis(int &c, float f, int n, bool ext, int open, int flo,
                                        int fhi, int &flag, const MixedRunArgs &a,
                                        const double *w) {
    if (flag != 1) return;
    const bool lo = ext ? (c < -1 || (c == -1 && f < 0.5f)) : (c < 0);
    const bool hi = ext ? (c > n || (c == n && f > 0.5f)) : (c > n || (c == n && f > 0.0f));
    if (!lo && !hi) return;
    if (open) {
        atomic_add_fixed(&a.cnt->leak_hi, &a.cnt->leak_lo, *w);
        flag = lo ? flo : fhi;
    } else {
        const int per = ext ? n + 1 : n;
        c += lo ? per : -per;   // the reference's wrap by one period
        // A push longer than a period (a drift near a magnetic null at dt_min)
        // leaves the particle outside even so; the reference would then index
        // outside its arrays.  Whole periods more bring it back into the box.
        if (c < -1) c += per * ((-1 - c + per - 1) / per);
        else if (c > n) c -= per * ((c - n + per - 1) / per);
    }
}

struct Pos {
    int cx, cy, cz;
    float fx, fy, fz;
};

template <int NDIM>
__device__ __forceinline__ void boundary(const MixedRunArgs &a, const MixedConsts &k, Pos &q,
                                         bool ext, int &flag, const double *w) {
    bc_axis(q.cx, q.fx, k.nx, ext, a.pbcx, -1, -2, flag, a, w);
    bc_axis(q.cy, q.fy, k.ny, ext, a.pbcy, -3, -4, flag, a, w);
    if (NDIM == 3) bc_axis(q.cz, q.fz, k.nz, ext, a.pbcz, -5, -6, flag, a, w);
}

template <int NDIM>
__device__ __forceinline__ void negp_or_boundary(const MixedRunArgs &a, const MixedConsts &k, Pos &q,
                                                 float p, int &flag, const double *w) {
    if (p < 0.0f) {
        flag = 0;
        atomic_add_fixed(&a.cnt->negp_hi, &a.cnt->negp_lo, *w);
    } else {
        boundary<NDIM>(a, k, q, true, flag, w);
    }
}

// 256-bit read-only global load (8 floats, 32-byte aligned address).  Records
// are 64 B (2D) or 96 B (3D) at 32-byte aligned offsets, so one corner costs 2
// or 3 of these instead of 4 or 6 128-bit loads.
__device__ __forceinline__ void ld8(const float *p, float (&v)[8]) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]),
          "=f"(v[7])
        : "l"(p));
}

// Index guard: the first offending node index (16 bits per axis) and the
// gather that met it (1 global, 2 shared-memory brick) go to bad_value.
__device__ __forceinline__ void record_guard(DevCounters *cnt, int ix, int iy, int iz, int kind) {
    const unsigned long long v = (unsigned long long)(ix & 0xffff) |
                                 ((unsigned long long)(iy & 0xffff) << 16) |
                                 ((unsigned long long)(iz & 0xffff) << 32) |
                                 ((unsigned long long)kind << 48);
    atomicCAS(&cnt->bad_value, 0ull, v);
    set_status(cnt, kStatusIndexGuard);
}

// FP32 bilinear / trilinear interpolation of the packed record.
template <int NDIM, int NV>
__device__ __forceinline__ bool interp_global(const MixedRunArgs &a, const Pos &q, float rt,
                                              float f[NV]) {
    constexpr int R = (NDIM == 2) ? kRec2D : kRec3D;
    const int ix = q.cx + 2, iy = q.cy + 2, iz = (NDIM == 3) ? q.cz + 2 : 0;
    if ((unsigned)ix > (unsigned)(a.nxg - 2) || (unsigned)iy > (unsigned)(a.nyg - 2) ||
        (NDIM == 3 && (unsigned)iz > (unsigned)(a.nzg - 2))) {
        record_guard(a.cnt, ix, iy, iz, 1);
        return false;
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = 0.0f;
    const size_t row = (size_t)a.nxg;
    const size_t plane = (size_t)a.nxg * a.nyg;
    const size_t base = (size_t)ix + row * iy + plane * iz;
#pragma unroll
    for (int kk = 0; kk < (NDIM == 3 ? 2 : 1); ++kk)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int ii = 0; ii < 2; ++ii) {
                float wc = (ii ? q.fx : 1.0f - q.fx) * (j ? q.fy : 1.0f - q.fy);
                if (NDIM == 3) wc *= (kk ? q.fz : 1.0f - q.fz);
                const size_t cell = base + ii + row * j + plane * kk;
                float w1 = wc;
                if (a.time_interp) w1 = wc * (1.0f - rt);
                const float *r1 = a.rec1 + (size_t)R * cell;
#pragma unroll
                for (int v8 = 0; v8 < (NV + 7) / 8; ++v8) {
                    float g[8];
                    ld8(r1 + 8 * v8, g);
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (8 * v8 + e < NV) f[8 * v8 + e] = fmaf(g[e], w1, f[8 * v8 + e]);
                }
                if (a.time_interp) {
                    const float w2 = wc * rt;
                    const float *r2 = a.rec2 + (size_t)R * cell;
#pragma unroll
                    for (int v8 = 0; v8 < (NV + 7) / 8; ++v8) {
                        float g[8];
                        ld8(r2 + 8 * v8, g);
#pragma unroll
                        for (int e = 0; e < 8; ++e)
                            if (8 * v8 + e < NV) f[8 * v8 + e] = fmaf(g[e], w2, f[8 * v8 + e]);
                    }
                }
            }
    return true;
}

// Gathers from the packed records in global memory; every position is
// reachable, so a particle never pauses for its position.
struct GlobalGather {
    template <int NDIM>
    __device__ __forceinline__ bool inside(const Pos &) const { return true; }
    __device__ __forceinline__ void record_miss(DevCounters *, const Pos &) const {}
    template <int NDIM, int NV>
    __device__ __forceinline__ bool interp(const MixedRunArgs &a, const Pos &q, float rt,
                                           float f[NV]) const {
        return interp_global<NDIM, NV>(a, q, rt, f);
    }
};

// Gathers from node records staged in shared memory: cells [o, o + b) per
// axis (ghost-padded indices), nodes [o, o + b] in chunk planes: float4
// chunk j of node n at tile[j * cst + n], nodes x fastest (the TMA box of
// the chunk-planar records).  Lanes reading one chunk of neighbouring nodes
// hit neighbouring bank groups; lanes reading the same node broadcast.
// tile2 is frame 2's copy when the run interpolates in time.
struct TileGather {
    const float4 *tile1, *tile2;
    int ox, oy, oz;       // staged origin, ghost-padded node index
    int bx, by, bz;       // staged cells per axis
    int sy, sz;           // node strides: bx + 1, (bx + 1)(by + 1)
    int cst;              // chunk plane stride: staged nodes

    template <int NDIM>
    __device__ __forceinline__ bool inside(const Pos &q) const {
        bool in = (unsigned)(q.cx + 2 - ox) < (unsigned)bx && (unsigned)(q.cy + 2 - oy) < (unsigned)by;
        if (NDIM == 3) in = in && (unsigned)(q.cz + 2 - oz) < (unsigned)bz;
        return in;
    }

    // The first particle found outside the region it was binned for: its
    // node index and the region's origin, 16 bits each (x, y, origin x,
    // origin y), for the host's message.
    __device__ __forceinline__ void record_miss(DevCounters *cnt, const Pos &q) const {
        const unsigned long long v =
            (unsigned long long)((q.cx + 2) & 0xffff) | ((unsigned long long)((q.cy + 2) & 0xffff) << 16) |
            ((unsigned long long)(ox & 0xffff) << 32) | ((unsigned long long)(oy & 0xffff) << 48);
        atomicCAS(&cnt->bad_value, 0ull, v);
        set_status(cnt, kStatusTileMiss);
    }

    // NV values of one node record (chunk j at r[j * cst]), scaled by w and
    // added to f.
    template <int R4, int NV>
    __device__ __forceinline__ void accumulate(const float4 *r, float w, float f[NV]) const {
#pragma unroll
        for (int v4 = 0; v4 < (NV + 3) / 4; ++v4) {
            if (NV - 4 * v4 == 1) {
                // last value alone: a 4-byte read instead of 16
                f[4 * v4] = fmaf(reinterpret_cast<const float *>(r + v4 * cst)[0], w, f[4 * v4]);
            } else {
                const float4 g = r[v4 * cst];
                f[4 * v4] = fmaf(g.x, w, f[4 * v4]);
                if (4 * v4 + 1 < NV) f[4 * v4 + 1] = fmaf(g.y, w, f[4 * v4 + 1]);
                if (4 * v4 + 2 < NV) f[4 * v4 + 2] = fmaf(g.z, w, f[4 * v4 + 2]);
                if (4 * v4 + 3 < NV) f[4 * v4 + 3] = fmaf(g.w, w, f[4 * v4 + 3]);
            }
        }
    }

    // Same weights and summation order as interp_global; only the source of
    // the records differs.  The caller has checked inside() (the base cell is
    // in the brick, so all corners are staged); the ghost-range guard of the
    // global path is kept for positions the brick origin does not cover.
    template <int NDIM, int NV>
    __device__ __forceinline__ bool interp(const MixedRunArgs &a, const Pos &q, float rt,
                                           float f[NV]) const {
        constexpr int R4 = ((NDIM == 2) ? kRec2D : kRec3D) / 4;
        const int ix = q.cx + 2, iy = q.cy + 2, iz = (NDIM == 3) ? q.cz + 2 : 0;
        if ((unsigned)ix > (unsigned)(a.nxg - 2) || (unsigned)iy > (unsigned)(a.nyg - 2) ||
            (NDIM == 3 && (unsigned)iz > (unsigned)(a.nzg - 2))) {
            record_guard(a.cnt, ix, iy, iz, 2);
            return false;
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) f[v] = 0.0f;
        const int base = (ix - ox) + sy * (iy - oy) + (NDIM == 3 ? sz * (iz - oz) : 0);
#pragma unroll
        for (int kk = 0; kk < (NDIM == 3 ? 2 : 1); ++kk)
#pragma unroll
            for (int j = 0; j < 2; ++j)
#pragma unroll
                for (int ii = 0; ii < 2; ++ii) {
                    float wc = (ii ? q.fx : 1.0f - q.fx) * (j ? q.fy : 1.0f - q.fy);
                    if (NDIM == 3) wc *= (kk ? q.fz : 1.0f - q.fz);
                    const int node = base + ii + sy * j + sz * kk;
                    float w1 = wc;
                    if (a.time_interp) w1 = wc * (1.0f - rt);
                    accumulate<R4, NV>(tile1 + node, w1, f);
                    if (a.time_interp) accumulate<R4, NV>(tile2 + node, wc * rt, f);
                }
        return true;
    }
};

__device__ __forceinline__ void noise4(const MixedRunArgs &a, uint32_t ctr, uint32_t ti, uint32_t ts,
                                       float r[4]) {
    const uint4 w = philox4x32_10(make_uint4(ctr, 2u, ti, ts), a.key0, a.key1);
    if (a.noise == GPAT_NOISE_UNIFORM) {
        // (2u - 1) sqrt(3) with u at the centre of one of 2^24 cells.
        const float sc = 1.7320508f / 8388608.0f;
        const float off = 1.7320508f * (1.0f / 16777216.0f - 1.0f);
        r[0] = fmaf((float)(w.x >> 8), sc, off);
        r[1] = fmaf((float)(w.y >> 8), sc, off);
        r[2] = fmaf((float)(w.z >> 8), sc, off);
        r[3] = fmaf((float)(w.w >> 8), sc, off);
    } else {
        const float u0 = ((float)(w.x >> 8) + 0.5f) * (1.0f / 16777216.0f);
        const float u2 = ((float)(w.z >> 8) + 0.5f) * (1.0f / 16777216.0f);
        const float ra = fsqrt(-2.0f * __logf(u0)), rb = fsqrt(-2.0f * __logf(u2));
        float sa, ca, sb, cb;
        __sincosf(6.2831853f * (float)(w.y >> 8) * (1.0f / 16777216.0f), &sa, &ca);
        __sincosf(6.2831853f * (float)(w.w >> 8) * (1.0f / 16777216.0f), &sb, &cb);
        r[0] = ra * ca; r[1] = ra * sa; r[2] = rb * cb; r[3] = rb * sb;
    }
}

template <int NDIM>
__device__ __forceinline__ bool in_acc_region(const MixedConsts &k, const Pos &q) {
    const float xn = ((float)q.cx + q.fx + k.acc_off[0]) * k.acc_scale[0];
    const float yn = ((float)q.cy + q.fy + k.acc_off[1]) * k.acc_scale[1];
    bool in = xn >= k.acc[0] && xn <= k.acc[1] && yn >= k.acc[2] && yn <= k.acc[3];
    if (NDIM == 3) {
        const float zn = ((float)q.cz + q.fz + k.acc_off[2]) * k.acc_scale[2];
        in = in && zn >= k.acc[4] && zn <= k.acc[5];
    }
    return in;
}

// One push: interpolation, kappa, drift, dt, noise.  Outputs increments in
// cell units (dX, dY, dZ), the momentum increment dp (before the floor) and,
// unless fixed, the adaptive dt.  NLGC: kperp from
// calc_spatial_diffusion_coefficients_nlgc (particle_module.f90:2464-2771),
// kpara0 kperp_kpara |B|^((gamma-2)/3) (p/p0)^((5-gamma)/3) mu^2, with the
// gradient terms T_i = kperp dkperp_i, A_i = kpara dkpara_i - kperp dkperp_i
// in place of kperp dk_i and kpp dk_i.
template <int NDIM, bool NLGC, class G>
__device__ __forceinline__ bool push(const MixedRunArgs &a, const MixedConsts &k, const G &g,
                                     const Pos &q, float p, float mu, float rt, bool fixed,
                                     float &dt, uint32_t ctr, uint32_t ti, uint32_t ts, float &dX,
                                     float &dY, float &dZ, float &dp) {
    constexpr int NV = (NDIM == 2) ? 15 : 21;
    float f[NV];
    if (!g.template interp<NDIM, NV>(a, q, rt, f)) return false;
    // slots: 2D vx vy bx by bz dvx/dx dvy/dy dbx/dx dbx/dy dby/dx dby/dy dbz/dx dbz/dy db/dx db/dy
    //        3D vx vy vz bx by bz dvx/dx dvy/dy dvz/dz dbi/dj (9) db/dx db/dy db/dz
    constexpr int OB = (NDIM == 2) ? 2 : 3;
    const float bx = f[OB], by = f[OB + 1], bz = f[OB + 2];
    const float b2 = fmaf(bx, bx, fmaf(by, by, bz * bz));
    const bool bzero = b2 < FLT_EPSILON * FLT_EPSILON;
    const float ib = bzero ? 0.0f : rsqrtf(b2);   // 1/B, or 0 for B = 0 (push)
    const float b = b2 * ib;
    const float ib1 = bzero ? 1.0f : ib;           // kappa's guard uses 1
    const float ib2 = ib1 * ib1, ib3 = ib1 * ib2;
    float knorm = 1.0f, knorm_perp = 1.0f;
    const float lb = (a.mag_dependency == 1) ? __log2f(b) : 0.0f;
    const float lp = (a.momentum_dependency == 1) ? __log2f(p * k.ip0) : 0.0f;
    if (a.mag_dependency == 1) knorm = exp2f(k.gm2 * lb);
    if (a.momentum_dependency == 1) knorm *= exp2f(k.pindex * lp);
    if (NLGC) {
        if (a.mag_dependency == 1) knorm_perp = exp2f(k.gm2_3 * lb);
        if (a.momentum_dependency == 1) knorm_perp *= exp2f(k.pindex_perp * lp);
    }
    const float kpara = k.kpara0 * knorm;
    const float kperp = NLGC ? k.kperp0 * knorm_perp * (mu * mu) : kpara * k.kret;
    const float kpp = kpara - kperp;
    const float skpara = fsqrt(2.0f * kpara), skperp = fsqrt(2.0f * kperp), skpp = fsqrt(2.0f * kpp);
    const float ip = __fdividef(1.0f, p);
    const float t1 = k.d1p0 * ip, t2 = k.d2p0sq * ip * ip;
    const float vdp = k.vdq * rsqrtf(fmaf(t1, t1, t2 * t2));
    const float jb2 = ib * ib, jb3 = ib * jb2;
    float dx_dt, dy_dt, dz_dt = 0.0f, divv;
    if (NDIM == 2) {
        const float dbx_dx = f[7], dbx_dy = f[8], dby_dx = f[9], dby_dy = f[10];
        const float dbz_dx = f[11], dbz_dy = f[12], db_dx = f[13], db_dy = f[14];
        float dkdx = 0.0f, dkdy = 0.0f;
        if (a.mag_dependency == 1) { dkdx = db_dx * ib1 * k.gm2; dkdy = db_dy * ib1 * k.gm2; }
        // T_i and A_i / B^2 of the gradient terms (T_i = kperp dk_i, A_i = kpp dk_i
        // without NLGC; dkperp_i = dk_i / 3 with it)
        float tx = kperp * dkdx, ty = kperp * dkdy;
        if (NLGC) { tx *= (1.0f / 3.0f); ty *= (1.0f / 3.0f); }
        const float gx = (NLGC ? kpara * dkdx - tx : kpp * dkdx) * ib2;
        const float gy = (NLGC ? kpara * dkdy - ty : kpp * dkdy) * ib2;
        const float ax = kpp * ib2, a3 = 2.0f * kpp * ib3;
        const float dkxx_dx = tx + gx * bx * bx + a3 * bx * (dbx_dx * b - bx * db_dx);
        const float dkyy_dy = ty + gy * by * by + a3 * by * (dby_dy * b - by * db_dy);
        const float dkxy_dx = gx * bx * by + ax * (dbx_dx * by + bx * dby_dx) - a3 * bx * by * db_dx;
        const float dkxy_dy = gy * bx * by + ax * (dbx_dy * by + bx * dby_dy) - a3 * bx * by * db_dy;
        const float vdx = vdp * (dbz_dy * jb2 - 2.0f * bz * db_dy * jb3);
        const float vdy = vdp * (2.0f * bz * db_dx * jb3 - dbz_dx * jb2);
        if (a.check_drift_2d)
            dz_dt = vdp * ((dby_dx - dbx_dy) * jb2 - 2.0f * (by * db_dx - bx * db_dy) * jb3);
        dx_dt = f[0] + vdx + dkxx_dx + dkxy_dy;
        dy_dt = f[1] + vdy + dkxy_dx + dkyy_dy;
        divv = f[5] + f[6];
    } else {
        const float dbx_dx = f[9], dbx_dy = f[10], dbx_dz = f[11];
        const float dby_dx = f[12], dby_dy = f[13], dby_dz = f[14];
        const float dbz_dx = f[15], dbz_dy = f[16], dbz_dz = f[17];
        const float db_dx = f[18], db_dy = f[19], db_dz = f[20];
        float dkdx = 0.0f, dkdy = 0.0f, dkdz = 0.0f;
        // the fixed-ratio 3D branch has no 1/B factor (:2406-2408); NLGC has
        if (a.mag_dependency == 1) {
            const float s = NLGC ? ib1 * k.gm2 : k.gm2;
            dkdx = db_dx * s; dkdy = db_dy * s; dkdz = db_dz * s;
        }
        float tx = kperp * dkdx, ty = kperp * dkdy, tz = kperp * dkdz;
        if (NLGC) { tx *= (1.0f / 3.0f); ty *= (1.0f / 3.0f); tz *= (1.0f / 3.0f); }
        const float gx = (NLGC ? kpara * dkdx - tx : kpp * dkdx) * ib2;
        const float gy = (NLGC ? kpara * dkdy - ty : kpp * dkdy) * ib2;
        const float gz = (NLGC ? kpara * dkdz - tz : kpp * dkdz) * ib2;
        const float ax = kpp * ib2, a3 = 2.0f * kpp * ib3;
        const float dkxx_dx = tx + gx * bx * bx + a3 * bx * (dbx_dx * b - bx * db_dx);
        const float dkyy_dy = ty + gy * by * by + a3 * by * (dby_dy * b - by * db_dy);
        const float dkzz_dz = tz + gz * bz * bz + a3 * bz * (dbz_dz * b - bz * db_dz);
        const float dkxy_dx = gx * bx * by + ax * (dbx_dx * by + bx * dby_dx) - a3 * bx * by * db_dx;
        const float dkxy_dy = gy * bx * by + ax * (dbx_dy * by + bx * dby_dy) - a3 * bx * by * db_dy;
        const float dkxz_dx = gx * bx * bz + ax * (dbx_dx * bz + bx * dbz_dx) - a3 * bx * bz * db_dx;
        const float dkxz_dz = gz * bx * bz + ax * (dbx_dz * bz + bx * dbz_dz) - a3 * bx * bz * db_dz;
        const float dkyz_dy = gy * by * bz + ax * (dby_dy * bz + by * dbz_dy) - a3 * by * bz * db_dy;
        const float dkyz_dz = gz * by * bz + ax * (dby_dz * bz + by * dbz_dz) - a3 * by * bz * db_dz;
        const float vdx = vdp * ((dbz_dy - dby_dz) * jb2 - 2.0f * (bz * db_dy - by * db_dz) * jb3);
        const float vdy = vdp * ((dbx_dz - dbz_dx) * jb2 - 2.0f * (bx * db_dz - bz * db_dx) * jb3);
        const float vdz = vdp * ((dby_dx - dbx_dy) * jb2 - 2.0f * (by * db_dx - bx * db_dy) * jb3);
        dx_dt = f[0] + vdx + dkxx_dx + dkxy_dy + dkxz_dz;
        dy_dt = f[1] + vdy + dkxy_dx + dkyy_dy + dkyz_dz;
        dz_dt = f[2] + vdz + dkxz_dx + dkyz_dy + dkzz_dz;
        divv = f[6] + f[7] + f[8];
    }
    const float dp_dt = -p * divv * (1.0f / 3.0f);
    if (!fixed) {
        // The reference's min() of diffusion / drift / momentum limits; dt_min
        // when a rate (dx, dy, dp) is exactly zero; clamp to [dt_min, dt_max].
        if (dx_dt != 0.0f && dy_dt != 0.0f && dp_dt != 0.0f) {
            const float sk = (skperp > 0.0f) ? skperp : skpara;
            const float isk = __fdividef(1.0f, skpara);
            float m = 0.5f * k.dxf * isk;
            m = fminf(m, 0.5f * k.dyf * isk);
            if (NDIM == 3) m = fminf(m, 0.5f * k.dzf * isk);
            m = fminf(m, fabsf(__fdividef(sk, dx_dt)));
            m = fminf(m, fabsf(__fdividef(sk, dy_dt)));
            if (NDIM == 3) m = fminf(m, fabsf(__fdividef(sk, dz_dt)));
            dt = fminf(m * m, __fdividef(0.1f * p, fabsf(dp_dt)));
        } else {
            dt = k.dt_min;
        }
        dt = fminf(fmaxf(dt, k.dt_min), k.dt_max);
    }
    const float sdt = fsqrt(dt);
    float r[4];
    noise4(a, ctr, ti, ts, r);
    if (NDIM == 2) {
        const float a3n = r[2] * skpp * sdt * ib;
        dX = fmaf(dx_dt, dt, fmaf(r[0] * skperp, sdt, a3n * bx)) * k.idx;
        dY = fmaf(dy_dt, dt, fmaf(r[1] * skperp, sdt, a3n * by)) * k.idy;
        dZ = dz_dt * dt;   // physical units; only non-zero with check_drift_2d
    } else {
        const float bxn = bx * ib, byn = by * ib, bzn = bz * ib;
        const float bxy2 = fmaf(bxn, bxn, byn * byn);
        const bool bxy0 = bxy2 < FLT_EPSILON * FLT_EPSILON;
        const float ibxyn = bxy0 ? 0.0f : rsqrtf(bxy2);
        const float bxyn = bxy2 * ibxyn;
        const float sp1 = skpara * r[0] * sdt;
        const float sq = skperp * ibxyn * sdt;
        dX = fmaf(dx_dt, dt, bxn * sp1 - bxn * bzn * sq * r[1] - byn * sq * r[2]) * k.idx;
        dY = fmaf(dy_dt, dt, byn * sp1 - byn * bzn * sq * r[1] + bxn * sq * r[2]) * k.idy;
        dZ = fmaf(dz_dt, dt, bzn * sp1 + bxyn * skperp * r[1] * sdt) * k.idz;
    }
    dp = dp_dt * dt;
    return true;
}

// Resident 128-thread blocks per SM the register allocation targets (2D: 6
// blocks = 80 registers, 3D: 5 blocks = 96 registers, measured best on GB300).
#ifndef GPAT_MIXED_MINB_2D
#define GPAT_MIXED_MINB_2D 6
#endif
#ifndef GPAT_MIXED_MINB_3D
#define GPAT_MIXED_MINB_3D 5
#endif

// One particle's interval (or chunk of it): particle_mover_one_cycle's body
// for particle i of P.  Returns the pushes made; active is set when the
// particle paused at chunk_pushes and must be resumed by the next launch.
//
// limit: pushes after which the particle pauses (0: none; a.chunk_pushes for
// a chunk launch).  exited is set when the particle paused because it left
// the gather's staged region (TileGather); it is then not counted active.
template <int NDIM, bool NLGC, class G>
__device__ __forceinline__ uint32_t move_particle(const MixedRunArgs &a, const MixedConsts &k,
                                                  const DevParticles &P, int64_t i,
                                                  bool &active, const G &g, uint32_t limit,
                                                  bool &exited) {
    uint32_t pushes = 0;
    active = false;
    exited = false;
    {
        const double *wp = P.weight + i;
        const double x_in = P.x[i], y_in = P.y[i], z_in = P.z[i];
        const double p_in = P.p[i], t_in = P.t[i];
        Pos q;
        cell_of(x_in, a.xmin, a.dx, q.cx, q.fx);
        cell_of(y_in, a.ymin, a.dy, q.cy, q.fy);
        if (NDIM == 3) {
            cell_of(z_in, a.zmin, a.dz, q.cz, q.fz);
        } else {
            q.cz = 0; q.fz = 0.0f;
        }
        const Pos q_in = q;
        float z2 = 0.0f;                       // 2D out-of-plane drift, physical units
        const float p_f0 = (float)p_in;
        float p = p_f0, pc = 0.0f;
        const double tau_in = t_in - a.t0;
        const float tau_f0 = (float)tau_in;
        float tau = tau_f0, tc = 0.0f;
        float dt = (float)P.dt[i];
        int flag = P.count_flag[i];
        int nsp = P.nsteps_pushed[i];
        uint32_t ctr = P.rng_ctr[i];
        const uint32_t ti = (uint32_t)P.tag_injected[i], ts = (uint32_t)P.tag_splitted[i];
        const float mu = NLGC ? (float)P.mu[i] : 0.0f;

        const double stepd = ceil(tau_in / a.dt_fine);
        double target_d = (stepd <= 0.0) ? a.dt_fine : stepd * a.dt_fine;
        if (target_d > a.dtf) target_d = a.dtf;
        double landed_at = -1.0;
        float uX = 0.0f, uY = 0.0f, uZ = 0.0f, uP = 0.0f;

        if (p < 0.0f && flag == 1) {
            flag = 0;
            atomic_add_fixed(&a.cnt->negp_hi, &a.cnt->negp_lo, *wp);
        } else {
            boundary<NDIM>(a, k, q, true, flag, wp);
        }
        bool alive = (flag == 1);
        bool paused = false;
        while (alive && target_d < a.limit) {
            const float target = (float)target_d;
            while (tau - tc < target && flag == 1) {
                negp_or_boundary<NDIM>(a, k, q, p - pc, flag, wp);
                if (flag != 1) break;
                if (limit != 0 && pushes >= limit) {
                    paused = true;   // between pushes: the next launch resumes from t
                    break;
                }
                if (!g.template inside<NDIM>(q)) {
                    // Left the staged region: pause between pushes; the caller
                    // finishes the chunk with global gathers.  A particle that
                    // has neither pushed nor moved since entry is outside the
                    // staged range altogether (not in the brick it is binned in).
                    if (pushes == 0 && q.cx == q_in.cx && q.cy == q_in.cy && q.cz == q_in.cz) {
                        g.record_miss(a.cnt, q);
                        flag = 0; alive = false; break;
                    }
                    paused = true;
                    exited = true;
                    break;
                }
                if (pushes >= a.max_pushes) { set_status(a.cnt, kStatusStepLimit); alive = false; break; }
                const float pe = p - pc;
                float dp;
                if (!push<NDIM, NLGC>(a, k, g, q, pe, mu, tau * k.inv_dtf, false, dt, ctr, ti, ts, uX,
                                      uY, uZ, dp)) {
                    flag = 0; alive = false; break;
                }
                ++ctr;
                ++pushes;
                advance(q.cx, q.fx, uX);
                advance(q.cy, q.fy, uY);
                if (NDIM == 3) advance(q.cz, q.fz, uZ); else z2 += uZ;
                kadd(tau, tc, dt);
                if (a.acc_region_flag == 1 && !in_acc_region<NDIM>(k, q)) dp = 0.0f;
                if (pe + dp < k.pfloor) { dp = k.pfloor - pe; p = k.pfloor; pc = 0.0f; }
                else kadd(p, pc, dp);
                uP = dp;
                landed_at = -1.0;
                nsp = (nsp + 1) % a.nsteps_interval;
                if (!(fabsf(tau) < 1e30f) || !(fabsf(p) < 1e30f) || !(q.fx <= 1.0f) ||
                    !(q.fy <= 1.0f) || !(q.fz <= 1.0f)) {
                    set_status(a.cnt, kStatusNonFinite);
                    flag = 0; alive = false; break;
                }
            }
            if (!alive || paused) break;
            if (tau - tc > target && flag == 1) {
                // Undo the overshooting push, redo it with dt = target - t.
                advance(q.cx, q.fx, -uX);
                advance(q.cy, q.fy, -uY);
                // push_particle_2d's deltaz is local to it: the undo keeps the
                // out-of-plane drift of the overshooting push.
                if (NDIM == 3) advance(q.cz, q.fz, -uZ);
                kadd(p, pc, -uP);
                kadd(tau, tc, -dt);
                const float dt_old = dt;
                float dtr = target - (tau - tc);
                if (dtr > 0.0f) {
                    nsp = nsp - 1;
                    const float pe = p - pc;
                    float dp;
                    if (!push<NDIM, NLGC>(a, k, g, q, pe, mu, tau * k.inv_dtf, true, dtr, ctr, ti,
                                          ts, uX, uY, uZ, dp)) {
                        flag = 0; alive = false; break;
                    }
                    ++ctr;
                    ++pushes;
                    advance(q.cx, q.fx, uX);
                    advance(q.cy, q.fy, uY);
                    if (NDIM == 3) advance(q.cz, q.fz, uZ); else z2 += uZ;
                    if (a.acc_region_flag == 1 && !in_acc_region<NDIM>(k, q)) dp = 0.0f;
                    if (pe + dp < k.pfloor) { dp = k.pfloor - pe; p = k.pfloor; pc = 0.0f; }
                    else kadd(p, pc, dp);
                    uP = dp;
                    tau = target; tc = 0.0f;
                    landed_at = target_d;
                    nsp = (nsp + 1) % a.nsteps_interval;
                }
                dt = dt_old;
                negp_or_boundary<NDIM>(a, k, q, p - pc, flag, wp);
            } else if (flag == 1 && tau - tc == target) {
                landed_at = target_d;   // reached the target without overshoot
            }
            target_d = target_d + a.dt_fine;
        }
        if (flag == 1 && !paused) boundary<NDIM>(a, k, q, false, flag, wp);
        active = paused && !exited;
        // Write back input + change, computed in FP64.
        const double dcx = (double)(q.cx - q_in.cx) + ((double)q.fx - (double)q_in.fx);
        const double dcy = (double)(q.cy - q_in.cy) + ((double)q.fy - (double)q_in.fy);
        P.x[i] = x_in + dcx * a.dx;
        P.y[i] = y_in + dcy * a.dy;
        if (NDIM == 3) {
            const double dcz = (double)(q.cz - q_in.cz) + ((double)q.fz - (double)q_in.fz);
            P.z[i] = z_in + dcz * a.dz;
        } else if (z2 != 0.0f) {
            P.z[i] = z_in + (double)z2;
        }
        P.p[i] = p_in + (((double)p - (double)pc) - (double)p_f0);
        P.t[i] = landed_at >= 0.0 ? a.t0 + landed_at
                                    : t_in + (((double)tau - (double)tc) - (double)tau_f0);
        P.dt[i] = (double)dt;
        P.count_flag[i] = (int8_t)flag;
        P.nsteps_pushed[i] = nsp;
        P.nsteps_tracked[i] = 1;
        P.rng_ctr[i] = ctr;
    }
    return pushes;
}

// Per-warp sums of pushes and paused particles into a run's counters.
__device__ __forceinline__ void add_warp_counters(DevCounters *cnt, uint32_t pushes, bool active,
                                                  unsigned long long *nactive_total) {
    const unsigned long long steps = warp_sum_u64(pushes);
    const unsigned act = __ballot_sync(0xffffffffu, active);
    if ((threadIdx.x & 31) == 0) {
        if (steps) atomicAdd(&cnt->steps, steps);
        if (act) {
            atomicAdd(&cnt->nactive, (unsigned long long)__popc(act));
            if (nactive_total) atomicAdd(nactive_total, (unsigned long long)__popc(act));
        }
    }
}

}  // namespace
}  // namespace gpat
