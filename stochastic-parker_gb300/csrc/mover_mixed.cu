// Split-precision particle mover.
//
// Field records, interpolation, the kappa tensor, drift and the adaptive-dt
// candidates run in FP32.  The quantities that accumulate over thousands of
// steps -- position, momentum and the particle clock -- are carried as
// compensated float-float pairs (hi + lo, error-free TwoSum / TwoProduct,
// about 48 significant bits), so no per-step work lands on the FP64 pipe;
// the FP64 particle record is read once at entry and written once at exit.
//
// Control flow is the reference's particle_mover_one_cycle
// (particle_module.f90:1481-1833): fine-step targets, adaptive pushes, the
// undo-and-redo landing on each target, boundary handling with the
// half-cell-extended box, and the exact-box pass at the end of the interval.
// Increments are the reference's (2u-1)*sqrt(3) (or Gaussian) variates from
// one Philox-4x32-10 call per push.
#include <cfloat>

#include "device_common.cuh"

namespace gpat {
namespace {

// ---- float-float arithmetic (Dekker / Knuth error-free transformations) --
struct ff {
    float h, l;
};

__device__ __forceinline__ ff two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return {s, e};
}
__device__ __forceinline__ ff fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ ff ff_add_f(ff a, float b) {
    ff s = two_sum(a.h, b);
    return fast_two_sum(s.h, s.l + a.l);
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
    ff s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, s.l + (a.l + b.l));
}
__device__ __forceinline__ ff ff_from_d(double d) {
    const float h = (float)d;
    return {h, (float)(d - (double)h)};
}
__device__ __forceinline__ double ff_to_d(ff a) { return (double)a.h + (double)a.l; }
__device__ __forceinline__ bool ff_lt(ff a, ff b) { return a.h < b.h || (a.h == b.h && a.l < b.l); }
__device__ __forceinline__ bool ff_gt(ff a, ff b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.h, -a.l}; }

// Grid coordinate of a position relative to the box minimum: integer cell
// and the in-cell fraction in full float precision.
__device__ __forceinline__ float grid_coord(ff xr, ff id, int &cell) {
    const float p = xr.h * id.h;
    const float e = fmaf(xr.h, id.h, -p);               // exact product error
    const float tail = e + fmaf(xr.h, id.l, xr.l * id.h);
    const float fl = floorf(p);
    float r = (p - fl) + tail;                          // p - fl is exact
    cell = (int)fl;
    if (r < 0.0f) { r += 1.0f; cell -= 1; }
    else if (r >= 1.0f) { r -= 1.0f; cell += 1; }
    return r;
}

struct Consts {
    ff idx, idy, idz;               // 1/dx, ...
    ff lo1x, hi1x, lo1y, hi1y, lo1z, hi1z;   // extended box relative to min
    ff lox, hix, loy, hiy, loz, hiz;         // exact box relative to min
    ff perx1, pery1, perz1, perx, pery, perz;  // periods of the two boxes
    float dxf, dyf, dzf;
    float dt_min, dt_max;
    float p0, ip0, pindex, gm2, kpara0, kret;
    float vdq;                      // single-precision 1/(3 charge)
    float d1p0, d2p0sq;             // drift1 * p0, drift2 * p0^2
    float pfloor;
    float accx0, accx1, accy0, accy1, accz0, accz1, ilx, ily, ilz, offx, offy, offz;
};

__device__ __forceinline__ Consts make_consts(const MoverArgs &a) {
    Consts c;
    c.idx = ff_from_d(a.idx); c.idy = ff_from_d(a.idy); c.idz = ff_from_d(a.idz);
    c.lo1x = ff_from_d(a.xmin1 - a.xmin); c.hi1x = ff_from_d(a.xmax1 - a.xmin);
    c.lo1y = ff_from_d(a.ymin1 - a.ymin); c.hi1y = ff_from_d(a.ymax1 - a.ymin);
    c.lo1z = ff_from_d(a.zmin1 - a.zmin); c.hi1z = ff_from_d(a.zmax1 - a.zmin);
    c.lox = ff_from_d(0.0); c.hix = ff_from_d(a.xmax - a.xmin);
    c.loy = ff_from_d(0.0); c.hiy = ff_from_d(a.ymax - a.ymin);
    c.loz = ff_from_d(0.0); c.hiz = ff_from_d(a.zmax - a.zmin);
    c.perx1 = ff_from_d(a.xmax1 - a.xmin1); c.pery1 = ff_from_d(a.ymax1 - a.ymin1);
    c.perz1 = ff_from_d(a.zmax1 - a.zmin1);
    c.perx = ff_from_d(a.xmax - a.xmin); c.pery = ff_from_d(a.ymax - a.ymin);
    c.perz = ff_from_d(a.zmax - a.zmin);
    c.dxf = (float)a.dx; c.dyf = (float)a.dy; c.dzf = (float)a.dz;
    c.dt_min = (float)a.dt_min; c.dt_max = (float)a.dt_max;
    c.p0 = (float)a.p0; c.ip0 = (float)(1.0 / a.p0); c.pindex = (float)a.pindex;
    c.gm2 = (float)(a.gamma_turb - 2.0);
    c.kpara0 = (float)a.kpara0; c.kret = (float)a.kret;
    c.vdq = 1.0f / (float)(3 * a.charge);
    c.d1p0 = (float)(a.drift1 * a.p0);
    c.d2p0sq = (float)(a.drift2 * (a.p0 * a.p0));
    c.pfloor = (float)(0.25 * a.p0);
    c.accx0 = (float)a.acc_region[0]; c.accx1 = (float)a.acc_region[1];
    c.accy0 = (float)a.acc_region[2]; c.accy1 = (float)a.acc_region[3];
    c.accz0 = (float)a.acc_region[4]; c.accz1 = (float)a.acc_region[5];
    c.ilx = (float)(1.0 / a.cfg_lx); c.ily = (float)(1.0 / a.cfg_ly); c.ilz = (float)(1.0 / a.cfg_lz);
    c.offx = (float)(a.xmin - a.cfg_xmin); c.offy = (float)(a.ymin - a.cfg_ymin);
    c.offz = (float)(a.zmin - a.cfg_zmin);
    return c;
}

struct S {
    ff x, y, z, p, tau;   // position relative to the box minimum, momentum, t - t0
    float dt;
    double w;
    int flag;
    int32_t nsp, tag_inj, tag_spl;
    uint32_t ctr;
};

struct Acc {
    unsigned long long leak_h, leak_l, negp_h, negp_l, steps;
};

__device__ __forceinline__ void acc_add(unsigned long long &h, unsigned long long &l, double w) {
    unsigned long long bh, bl;
    fixed_split(w, bh, bl);
    add_u128(h, l, bh, bl);
}

// One open/periodic boundary test along one axis.
__device__ __forceinline__ void bc_axis(ff &x, ff lo, ff hi, ff per, int open, int flo, int fhi,
                                        S &s, Acc &acc) {
    if (s.flag != 1) return;
    if (ff_lt(x, lo)) {
        if (open) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = flo; }
        else x = ff_add(x, per);
    } else if (ff_gt(x, hi)) {
        if (open) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = fhi; }
        else x = ff_add(x, ff_neg(per));
    }
}

template <int NDIM>
__device__ __forceinline__ void boundary_ext(const MoverArgs &a, const Consts &c, S &s, Acc &acc) {
    bc_axis(s.x, c.lo1x, c.hi1x, c.perx1, a.pbcx, -1, -2, s, acc);
    bc_axis(s.y, c.lo1y, c.hi1y, c.pery1, a.pbcy, -3, -4, s, acc);
    if (NDIM == 3) bc_axis(s.z, c.lo1z, c.hi1z, c.perz1, a.pbcz, -5, -6, s, acc);
}

template <int NDIM>
__device__ __forceinline__ void negp_or_boundary(const MoverArgs &a, const Consts &c, S &s, Acc &acc) {
    if (s.p.h < 0.0f) {
        s.flag = 0;
        acc_add(acc.negp_h, acc.negp_l, s.w);
    } else {
        boundary_ext<NDIM>(a, c, s, acc);
    }
}

// FP32 interpolation of the packed record at the particle.
template <int NDIM, int NV>
__device__ __forceinline__ bool interp(const MoverArgs &a, const Consts &c, const S &s, float f[NV]) {
    constexpr int R = (NDIM == 2) ? kRec2D : kRec3D;
    int cx, cy, cz = 0;
    const float rx = grid_coord(s.x, c.idx, cx);
    const float ry = grid_coord(s.y, c.idy, cy);
    const float rz = (NDIM == 3) ? grid_coord(s.z, c.idz, cz) : 0.0f;
    const int ix = cx + 2, iy = cy + 2, iz = (NDIM == 3) ? cz + 2 : 0;
    if (ix < 0 || ix + 1 >= a.nxg || iy < 0 || iy + 1 >= a.nyg ||
        (NDIM == 3 && (iz < 0 || iz + 1 >= a.nzg))) {
        set_status(a.cnt, kStatusIndexGuard);
        return false;
    }
    const float rx1 = 1.0f - rx, ry1 = 1.0f - ry, rz1 = 1.0f - rz;
#pragma unroll
    for (int v = 0; v < NV; ++v) f[v] = 0.0f;
    const float rt = a.time_interp ? (float)((double)s.tau.h / a.dtf) : 0.0f;
#pragma unroll
    for (int k = 0; k < (NDIM == 3 ? 2 : 1); ++k)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                float wc = (i ? rx : rx1) * (j ? ry : ry1);
                if (NDIM == 3) wc *= (k ? rz : rz1);
                const size_t cell = (size_t)(ix + i) +
                                    (size_t)a.nxg * ((size_t)(iy + j) + (size_t)a.nyg * (size_t)(iz + k));
                const float4 *r4 = reinterpret_cast<const float4 *>(a.rec1 + (size_t)R * cell);
                float w1 = wc, w2 = 0.0f;
                if (a.time_interp) { w1 = wc * (1.0f - rt); w2 = wc * rt; }
#pragma unroll
                for (int q = 0; q < (NV + 3) / 4; ++q) {
                    const float4 v4 = __ldg(r4 + q);
                    const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (4 * q + e < NV) f[4 * q + e] = fmaf(vv[e], w1, f[4 * q + e]);
                }
                if (a.time_interp) {
                    const float4 *s4 = reinterpret_cast<const float4 *>(a.rec2 + (size_t)R * cell);
#pragma unroll
                    for (int q = 0; q < (NV + 3) / 4; ++q) {
                        const float4 v4 = __ldg(s4 + q);
                        const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (4 * q + e < NV) f[4 * q + e] = fmaf(vv[e], w2, f[4 * q + e]);
                    }
                }
            }
    return true;
}

__device__ __forceinline__ void noise4(const MoverArgs &a, S &s, float r[4]) {
    const uint4 w = philox4x32_10(make_uint4(s.ctr, 2u, (uint32_t)s.tag_inj, (uint32_t)s.tag_spl),
                                  a.key0, a.key1);
    s.ctr += 1u;
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
        const float ra = sqrtf(-2.0f * __logf(u0)), rb = sqrtf(-2.0f * __logf(u2));
        float sa, ca, sb, cb;
        __sincosf(6.2831853f * (float)(w.y >> 8) * (1.0f / 16777216.0f), &sa, &ca);
        __sincosf(6.2831853f * (float)(w.w >> 8) * (1.0f / 16777216.0f), &sb, &cb);
        r[0] = ra * ca; r[1] = ra * sa; r[2] = rb * cb; r[3] = rb * sb;
    }
}

__device__ __forceinline__ bool in_acc_region(const Consts &c, const S &s, int ndim) {
    const float xn = (s.x.h + c.offx) * c.ilx;
    bool in = (xn >= c.accx0) && (xn <= c.accx1);
    if (ndim > 1) {
        const float yn = (s.y.h + c.offy) * c.ily;
        in = in && (yn >= c.accy0) && (yn <= c.accy1);
    }
    if (ndim == 3) {
        const float zn = (s.z.h + c.offz) * c.ilz;
        in = in && (zn >= c.accz0) && (zn <= c.accz1);
    }
    return in;
}

struct KF {
    float kperp, skpara, skperp, skpp, kpp, b, ib1, ib2, ib3;
};

__device__ __forceinline__ KF kappa_f(const MoverArgs &a, const Consts &c, float p, float bx,
                                      float by, float bz) {
    KF k;
    const float b2 = fmaf(bx, bx, fmaf(by, by, bz * bz));
    k.b = sqrtf(b2);
    k.ib1 = (k.b < FLT_EPSILON) ? 1.0f : __frcp_rn(k.b);
    k.ib2 = k.ib1 * k.ib1;
    k.ib3 = k.ib1 * k.ib2;
    float knorm = 1.0f;
    if (a.mag_dependency == 1) knorm = exp2f(c.gm2 * __log2f(k.b));
    if (a.momentum_dependency == 1) knorm *= exp2f(c.pindex * __log2f(p * c.ip0));
    const float kpara = c.kpara0 * knorm;
    k.kperp = kpara * c.kret;
    k.skpara = sqrtf(2.0f * kpara);
    k.skperp = sqrtf(2.0f * k.kperp);
    k.kpp = kpara - k.kperp;
    k.skpp = sqrtf(2.0f * k.kpp);
    return k;
}

__device__ __forceinline__ float vdrift_prefactor(const Consts &c, float p) {
    const float ip = __frcp_rn(p);
    const float t1 = c.d1p0 * ip;
    const float t2 = c.d2p0sq * ip * ip;
    return c.vdq * rsqrtf(fmaf(t1, t1, t2 * t2));
}

// Adaptive step: the reference's min() of diffusion / drift / momentum
// limits, dt_min when any rate is exactly zero, clamped to [dt_min, dt_max].
__device__ __forceinline__ float pick_dt(const Consts &c, float skpara, float skperp, float dx_dt,
                                         float dy_dt, float dz_dt, float dp_dt, float p, int ndim) {
    if (!(dx_dt != 0.0f && dy_dt != 0.0f && dp_dt != 0.0f)) return c.dt_min;
    const float sk = (skperp > 0.0f) ? skperp : skpara;
    const float isk = __frcp_rn(skpara);
    float q = 0.5f * c.dxf * isk, m = q * q;
    q = 0.5f * c.dyf * isk; m = fminf(m, q * q);
    if (ndim == 3) { q = 0.5f * c.dzf * isk; m = fminf(m, q * q); }
    q = __fdividef(sk, dx_dt); m = fminf(m, q * q);
    q = __fdividef(sk, dy_dt); m = fminf(m, q * q);
    if (ndim == 3) { q = __fdividef(sk, dz_dt); m = fminf(m, q * q); }
    m = fminf(m, __fdividef(0.1f * p, fabsf(dp_dt)));
    return fminf(fmaxf(m, c.dt_min), c.dt_max);
}

__device__ __forceinline__ void update_p(const MoverArgs &a, const Consts &c, S &s, float dp,
                                         int ndim, float &dP_o) {
    if (a.acc_region_flag == 1 && !in_acc_region(c, s, ndim)) dp = 0.0f;
    ff np = ff_add_f(s.p, dp);
    if (np.h < c.pfloor) {
        dp = c.pfloor - s.p.h - s.p.l;
        np = ff{c.pfloor, 0.0f};
    }
    s.p = np;
    dP_o = dp;
}

template <int NDIM>
__device__ __forceinline__ void push(const MoverArgs &a, const Consts &c, S &s, const float *f,
                                     bool fixed_dt, float &dX, float &dY, float &dZ, float &dP) {
    const float p = s.p.h;
    if (NDIM == 2) {
        const float bx = f[2], by = f[3], bz = f[4];
        const KF k = kappa_f(a, c, p, bx, by, bz);
        const float dbx_dx = f[7], dbx_dy = f[8], dby_dx = f[9], dby_dy = f[10];
        const float dbz_dx = f[11], dbz_dy = f[12], db_dx = f[13], db_dy = f[14];
        float dkdx = 0.0f, dkdy = 0.0f;
        if (a.mag_dependency == 1) { dkdx = db_dx * k.ib1 * c.gm2; dkdy = db_dy * k.ib1 * c.gm2; }
        const float b = k.b, kpp = k.kpp, ib2 = k.ib2, ib3 = k.ib3;
        const float dkxx_dx = k.kperp * dkdx + kpp * dkdx * bx * bx * ib2 +
                              2.0f * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3;
        const float dkyy_dy = k.kperp * dkdy + kpp * dkdy * by * by * ib2 +
                              2.0f * kpp * by * (dby_dy * b - by * db_dy) * ib3;
        const float dkxy_dx = kpp * dkdx * bx * by * ib2 +
                              kpp * ((dbx_dx * by + bx * dby_dx) * ib2 - 2.0f * bx * by * db_dx * ib3);
        const float dkxy_dy = kpp * dkdy * bx * by * ib2 +
                              kpp * ((dbx_dy * by + bx * dby_dy) * ib2 - 2.0f * bx * by * db_dy * ib3);
        const float ib = (b < FLT_EPSILON) ? 0.0f : k.ib1;
        const float jb2 = ib * ib, jb3 = ib * jb2;
        const float vdp = vdrift_prefactor(c, p);
        const float vdx = vdp * (dbz_dy * jb2 - 2.0f * bz * db_dy * jb3);
        const float vdy = vdp * (2.0f * bz * db_dx * jb3 - dbz_dx * jb2);
        float vdz = 0.0f;
        if (a.check_drift_2d)
            vdz = vdp * ((dby_dx - dbx_dy) * jb2 - 2.0f * (by * db_dx - bx * db_dy) * jb3);
        const float dx_dt = f[0] + vdx + dkxx_dx + dkxy_dy;
        const float dy_dt = f[1] + vdy + dkxy_dx + dkyy_dy;
        const float divv = f[5] + f[6];
        const float dp_dt = -p * divv * (1.0f / 3.0f);
        if (!fixed_dt) s.dt = pick_dt(c, k.skpara, k.skperp, dx_dt, dy_dt, 0.0f, dp_dt, p, 2);
        const float dt = s.dt, sdt = sqrtf(dt);
        float r[4];
        noise4(a, s, r);
        const float a3 = r[2] * k.skpp * sdt * ib;
        dX = fmaf(dx_dt, dt, fmaf(r[0] * k.skperp, sdt, a3 * bx));
        dY = fmaf(dy_dt, dt, fmaf(r[1] * k.skperp, sdt, a3 * by));
        dZ = vdz * dt;
        s.x = ff_add_f(s.x, dX);
        s.y = ff_add_f(s.y, dY);
        s.z = ff_add_f(s.z, dZ);
        s.tau = ff_add_f(s.tau, dt);
        update_p(a, c, s, dp_dt * dt, 2, dP);
    } else {
        const float bx = f[3], by = f[4], bz = f[5];
        const KF k = kappa_f(a, c, p, bx, by, bz);
        const float dbx_dx = f[9], dbx_dy = f[10], dbx_dz = f[11];
        const float dby_dx = f[12], dby_dy = f[13], dby_dz = f[14];
        const float dbz_dx = f[15], dbz_dy = f[16], dbz_dz = f[17];
        const float db_dx = f[18], db_dy = f[19], db_dz = f[20];
        float dkdx = 0.0f, dkdy = 0.0f, dkdz = 0.0f;
        if (a.mag_dependency == 1) { dkdx = db_dx * c.gm2; dkdy = db_dy * c.gm2; dkdz = db_dz * c.gm2; }
        const float b = k.b, kpp = k.kpp, kperp = k.kperp, ib2 = k.ib2, ib3 = k.ib3;
        const float dkxx_dx = kperp * dkdx + kpp * dkdx * bx * bx * ib2 +
                              2.0f * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3;
        const float dkyy_dy = kperp * dkdy + kpp * dkdy * by * by * ib2 +
                              2.0f * kpp * by * (dby_dy * b - by * db_dy) * ib3;
        const float dkzz_dz = kperp * dkdz + kpp * dkdz * bz * bz * ib2 +
                              2.0f * kpp * bz * (dbz_dz * b - bz * db_dz) * ib3;
        const float dkxy_dx = kpp * dkdx * bx * by * ib2 +
                              kpp * ((dbx_dx * by + bx * dby_dx) * ib2 - 2.0f * bx * by * db_dx * ib3);
        const float dkxy_dy = kpp * dkdy * bx * by * ib2 +
                              kpp * ((dbx_dy * by + bx * dby_dy) * ib2 - 2.0f * bx * by * db_dy * ib3);
        const float dkxz_dx = kpp * dkdx * bx * bz * ib2 +
                              kpp * ((dbx_dx * bz + bx * dbz_dx) * ib2 - 2.0f * bx * bz * db_dx * ib3);
        const float dkxz_dz = kpp * dkdz * bx * bz * ib2 +
                              kpp * ((dbx_dz * bz + bx * dbz_dz) * ib2 - 2.0f * bx * bz * db_dz * ib3);
        const float dkyz_dy = kpp * dkdy * by * bz * ib2 +
                              kpp * ((dby_dy * bz + by * dbz_dy) * ib2 - 2.0f * by * bz * db_dy * ib3);
        const float dkyz_dz = kpp * dkdz * by * bz * ib2 +
                              kpp * ((dby_dz * bz + by * dbz_dz) * ib2 - 2.0f * by * bz * db_dz * ib3);
        const float ib = (b < FLT_EPSILON) ? 0.0f : k.ib1;
        const float bxn = bx * ib, byn = by * ib, bzn = bz * ib;
        const float bxyn = sqrtf(fmaf(bxn, bxn, byn * byn));
        const float ibxyn = (bxyn < FLT_EPSILON) ? 0.0f : __frcp_rn(bxyn);
        const float jb2 = ib * ib, jb3 = ib * jb2;
        const float vdp = vdrift_prefactor(c, p);
        const float vdx = vdp * ((dbz_dy - dby_dz) * jb2 - 2.0f * (bz * db_dy - by * db_dz) * jb3);
        const float vdy = vdp * ((dbx_dz - dbz_dx) * jb2 - 2.0f * (bx * db_dz - bz * db_dx) * jb3);
        const float vdz = vdp * ((dby_dx - dbx_dy) * jb2 - 2.0f * (by * db_dx - bx * db_dy) * jb3);
        const float dx_dt = f[0] + vdx + dkxx_dx + dkxy_dy + dkxz_dz;
        const float dy_dt = f[1] + vdy + dkxy_dx + dkyy_dy + dkyz_dz;
        const float dz_dt = f[2] + vdz + dkxz_dx + dkyz_dy + dkzz_dz;
        const float divv = f[6] + f[7] + f[8];
        const float dp_dt = -p * divv * (1.0f / 3.0f);
        if (!fixed_dt) s.dt = pick_dt(c, k.skpara, k.skperp, dx_dt, dy_dt, dz_dt, dp_dt, p, 3);
        const float dt = s.dt, sdt = sqrtf(dt);
        float r[4];
        noise4(a, s, r);
        const float sp1 = k.skpara * r[0];
        const float sq = k.skperp * ibxyn;
        dX = fmaf(dx_dt, dt, (bxn * sp1 - bxn * bzn * sq * r[1] - byn * sq * r[2]) * sdt);
        dY = fmaf(dy_dt, dt, (byn * sp1 - byn * bzn * sq * r[1] + bxn * sq * r[2]) * sdt);
        dZ = fmaf(dz_dt, dt, (bzn * sp1 + bxyn * k.skperp * r[1]) * sdt);
        s.x = ff_add_f(s.x, dX);
        s.y = ff_add_f(s.y, dY);
        s.z = ff_add_f(s.z, dZ);
        s.tau = ff_add_f(s.tau, dt);
        update_p(a, c, s, dp_dt * dt, 3, dP);
    }
}

template <int NDIM>
__device__ __forceinline__ bool do_push(const MoverArgs &a, const Consts &c, S &s, bool fixed_dt,
                                        float &dX, float &dY, float &dZ, float &dP) {
    constexpr int NV = (NDIM == 2) ? 15 : 21;
    float f[NV];
    if (!interp<NDIM, NV>(a, c, s, f)) return false;
    push<NDIM>(a, c, s, f, fixed_dt, dX, dY, dZ, dP);
    if (!isfinite(s.x.h) || !isfinite(s.y.h) || !isfinite(s.z.h) || !isfinite(s.p.h) ||
        !isfinite(s.tau.h)) {
        set_status(a.cnt, kStatusNonFinite);
        return false;
    }
    return true;
}

template <int NDIM>
__global__ void __launch_bounds__(128) mover_mixed_kernel(const MoverArgs a) {
    Acc acc = {0, 0, 0, 0, 0};
    const Consts c = make_consts(a);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n) {
        S s;
        s.x = ff_from_d(a.P.x[i] - a.xmin);
        s.y = ff_from_d(a.P.y[i] - a.ymin);
        s.z = ff_from_d(a.P.z[i] - a.zmin);
        s.p = ff_from_d(a.P.p[i]);
        s.tau = ff_from_d(a.P.t[i] - a.t0);
        s.dt = (float)a.P.dt[i];
        s.w = a.P.weight[i];
        s.flag = a.P.count_flag[i];
        s.nsp = a.P.nsteps_pushed[i];
        s.tag_inj = a.P.tag_injected[i];
        s.tag_spl = a.P.tag_splitted[i];
        s.ctr = a.P.rng_ctr[i];
        const double tau0 = a.P.t[i] - a.t0;
        const double stepd = ceil(tau0 / a.dt_fine);
        double target_d = (stepd <= 0.0) ? a.dt_fine : stepd * a.dt_fine;
        if (target_d > a.dtf) target_d = a.dtf;
        float dX = 0.0f, dY = 0.0f, dZ = 0.0f, dP = 0.0f;
        if (s.p.h < 0.0f && s.flag == 1) {
            s.flag = 0;
            acc_add(acc.negp_h, acc.negp_l, s.w);
        } else {
            boundary_ext<NDIM>(a, c, s, acc);
        }
        uint32_t pushes = 0;
        bool alive = (s.flag == 1);
        while (alive && target_d < a.limit) {
            if (s.flag != 1) break;
            const ff target = ff_from_d(target_d);
            while (ff_lt(s.tau, target) && s.flag == 1) {
                negp_or_boundary<NDIM>(a, c, s, acc);
                if (s.flag != 1) break;
                if (pushes >= a.max_pushes) { set_status(a.cnt, kStatusStepLimit); alive = false; break; }
                if (!do_push<NDIM>(a, c, s, false, dX, dY, dZ, dP)) { s.flag = 0; alive = false; break; }
                ++pushes;
                s.nsp = (s.nsp + 1) % a.nsteps_interval;
            }
            if (!alive) break;
            if (ff_gt(s.tau, target) && s.flag == 1) {
                // Undo the overshooting push and redo it with dt = target - t.
                s.x = ff_add_f(s.x, -dX);
                s.y = ff_add_f(s.y, -dY);
                s.z = ff_add_f(s.z, -dZ);
                s.p = ff_add_f(s.p, -dP);
                s.tau = ff_add_f(s.tau, -s.dt);
                const float dt_old = s.dt;
                const ff rem = ff_add(target, ff_neg(s.tau));
                s.dt = rem.h + rem.l;
                if (s.dt > 0.0f) {
                    s.nsp = s.nsp - 1;
                    if (!do_push<NDIM>(a, c, s, true, dX, dY, dZ, dP)) { s.flag = 0; alive = false; break; }
                    ++pushes;
                    s.nsp = (s.nsp + 1) % a.nsteps_interval;
                    s.tau = target;   // the redo lands on the target by construction
                }
                s.dt = dt_old;
                negp_or_boundary<NDIM>(a, c, s, acc);
            }
            target_d = target_d + a.dt_fine;
        }
        if (s.flag == 1) {
            bc_axis(s.x, c.lox, c.hix, c.perx, a.pbcx, -1, -2, s, acc);
            bc_axis(s.y, c.loy, c.hiy, c.pery, a.pbcy, -3, -4, s, acc);
            if (NDIM == 3) bc_axis(s.z, c.loz, c.hiz, c.perz, a.pbcz, -5, -6, s, acc);
        }
        acc.steps = pushes;
        // Write back input + accumulated change, so untouched coordinates
        // keep every bit of their FP64 value (a float pair holds 48 bits).
        const double x0 = a.P.x[i], y0 = a.P.y[i], z0 = a.P.z[i], p0 = a.P.p[i], t0 = a.P.t[i];
        a.P.x[i] = x0 + ff_to_d(ff_add(s.x, ff_neg(ff_from_d(x0 - a.xmin))));
        a.P.y[i] = y0 + ff_to_d(ff_add(s.y, ff_neg(ff_from_d(y0 - a.ymin))));
        a.P.z[i] = z0 + ff_to_d(ff_add(s.z, ff_neg(ff_from_d(z0 - a.zmin))));
        a.P.p[i] = p0 + ff_to_d(ff_add(s.p, ff_neg(ff_from_d(p0))));
        a.P.t[i] = t0 + ff_to_d(ff_add(s.tau, ff_neg(ff_from_d(t0 - a.t0))));
        a.P.dt[i] = (double)s.dt;
        a.P.count_flag[i] = (int8_t)s.flag;
        a.P.nsteps_pushed[i] = s.nsp;
        a.P.nsteps_tracked[i] = 1;
        a.P.rng_ctr[i] = s.ctr;
    }
    const unsigned long long steps = warp_sum_u64(acc.steps);
    unsigned long long lh = acc.leak_h, ll = acc.leak_l, nh = acc.negp_h, nl = acc.negp_l;
    warp_sum_u128(lh, ll);
    warp_sum_u128(nh, nl);
    if ((threadIdx.x & 31) == 0) {
        if (steps) atomicAdd(&a.cnt->steps, steps);
        if (lh | ll) atomic_add_u128(&a.cnt->leak_hi, &a.cnt->leak_lo, lh, ll);
        if (nh | nl) atomic_add_u128(&a.cnt->negp_hi, &a.cnt->negp_lo, nh, nl);
    }
}

}  // namespace

cudaError_t launch_mover_mixed(const MoverArgs &a, int sm_count, cudaStream_t s) {
    (void)sm_count;
    if (a.n <= 0) return cudaSuccess;
    const int threads = 128;
    const int64_t blocks = (a.n + threads - 1) / threads;
    if (a.ndim == 2) mover_mixed_kernel<2><<<(unsigned)blocks, threads, 0, s>>>(a);
    else mover_mixed_kernel<3><<<(unsigned)blocks, threads, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace gpat
