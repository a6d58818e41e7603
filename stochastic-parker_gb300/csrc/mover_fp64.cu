// FP64 particle mover: the reference's Parker path with its exact operation
// order.  This translation unit is compiled with -fmad=false so every
// +, -, *, / and sqrt is a single IEEE-rounded operation, which makes the
// trajectories bit-identical to a CPU FP64 evaluation of the same formulas
// (only pow() in momentum/|B|-dependent kappa is library-dependent).
//
// Follows particle_mover_one_cycle (particle_module.f90:1481-1833),
// get_interp_paramters (:642-674), interp_fields (mhd_data_parallel.f90:
// 1751-1804), calc_spatial_diffusion_coefficients (:2208-2450),
// push_particle_2d (:3358-3606), push_particle_3d (:4625-4907) and
// particle_boundary_condition (:1984-2129) on a single rank.
#include <cfloat>

#include "device_common.cuh"

namespace gpat {
namespace {

// Packed record slots (fields.cu).
enum R2 { A_VX, A_VY, A_BX, A_BY, A_BZ, A_DVXDX, A_DVYDY, A_DBXDX, A_DBXDY, A_DBYDX, A_DBYDY,
          A_DBZDX, A_DBZDY, A_DBDX, A_DBDY };
enum R3 { B_VX, B_VY, B_VZ, B_BX, B_BY, B_BZ, B_DVXDX, B_DVYDY, B_DVZDZ, B_DBXDX, B_DBXDY,
          B_DBXDZ, B_DBYDX, B_DBYDY, B_DBYDZ, B_DBZDX, B_DBZDY, B_DBZDZ, B_DBDX, B_DBDY, B_DBDZ };

struct State {
    double x, y, z, p, t, dt, w;
    int flag;
    int32_t nsteps_pushed, tag_inj, tag_spl;
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

// Interpolated fields at the particle, in the packed-record slot order.
template <int NDIM, int NV>
__device__ __forceinline__ bool interp(const MoverArgs &a, const State &s, double f[NV]) {
    constexpr int R = (NDIM == 2) ? kRec2D : kRec3D;
    const double px = (s.x - a.xmin) / a.dx;
    const double py = (s.y - a.ymin) / a.dy;
    const double pz = (s.z - a.zmin) / a.dz;
    const int nx = a.nxg - 4, ny = a.nyg - 4, nz = a.nzg - 4;
    if (!(px >= -1.0 && px < nx + 1.0) || !(py >= -1.0 && py < ny + 1.0) ||
        (NDIM == 3 && !(pz >= -1.0 && pz < nz + 1.0))) {
        set_status(a.cnt, kStatusIndexGuard);
        return false;
    }
    // get_interp_paramters: pos = floor(p) + 1 (Fortran), r = p - pos + 1.
    const int fx = (int)floor(px), fy = (int)floor(py);
    const int fz = (NDIM == 3) ? (int)floor(pz) : 0;
    const double rx = (px - (double)(fx + 1)) + 1.0;
    const double ry = (py - (double)(fy + 1)) + 1.0;
    const double rz = (NDIM == 3) ? (pz - (double)(fz + 1)) + 1.0 : 0.0;
    const double rx1 = 1.0 - rx, ry1 = 1.0 - ry, rz1 = 1.0 - rz;
    double w[8];
    w[0] = rx1 * ry1 * rz1;
    w[1] = rx * ry1 * rz1;
    w[2] = rx1 * ry * rz1;
    w[3] = rx * ry * rz1;
    w[4] = rx1 * ry1 * rz;
    w[5] = rx * ry1 * rz;
    w[6] = rx1 * ry * rz;
    w[7] = rx * ry * rz;
    const int ix = fx + 2, iy = fy + 2, iz = (NDIM == 3) ? fz + 2 : 0;
    double f2[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) { f[v] = 0.0; f2[v] = 0.0; }
    const double rt = (s.t - a.t0) / a.dtf;
#pragma unroll
    for (int k = 0; k < (NDIM == 3 ? 2 : 1); ++k)
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const double wc = w[k * 4 + j * 2 + i];
                const size_t cell = (size_t)(ix + i) +
                                    (size_t)a.nxg * ((size_t)(iy + j) + (size_t)a.nyg * (size_t)(iz + k));
                const float4 *r4 = reinterpret_cast<const float4 *>(a.rec1 + (size_t)R * cell);
#pragma unroll
                for (int q = 0; q < (NV + 3) / 4; ++q) {
                    const float4 v4 = __ldg(r4 + q);
                    const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (4 * q + e < NV) f[4 * q + e] = f[4 * q + e] + (double)vv[e] * wc;
                }
                if (a.time_interp) {
                    const float4 *s4 = reinterpret_cast<const float4 *>(a.rec2 + (size_t)R * cell);
#pragma unroll
                    for (int q = 0; q < (NV + 3) / 4; ++q) {
                        const float4 v4 = __ldg(s4 + q);
                        const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            if (4 * q + e < NV) f2[4 * q + e] = f2[4 * q + e] + (double)vv[e] * wc;
                    }
                }
            }
    if (a.time_interp) {
#pragma unroll
        for (int v = 0; v < NV; ++v) f[v] = f[v] * (1.0 - rt) + f2[v] * rt;
    }
    return true;
}

__device__ __forceinline__ void noise4(const MoverArgs &a, State &s, double r[4]) {
    const uint4 w0 = philox4x32_10(make_uint4(s.ctr, 0u, (uint32_t)s.tag_inj, (uint32_t)s.tag_spl),
                                   a.key0, a.key1);
    const uint4 w1 = philox4x32_10(make_uint4(s.ctr, 1u, (uint32_t)s.tag_inj, (uint32_t)s.tag_spl),
                                   a.key0, a.key1);
    s.ctr += 1u;
    const double u0 = u01_53(w0.x, w0.y), u1 = u01_53(w0.z, w0.w);
    const double u2 = u01_53(w1.x, w1.y), u3 = u01_53(w1.z, w1.w);
    if (a.noise == GPAT_NOISE_UNIFORM) {
        const double sqrt3 = sqrt(3.0);
        r[0] = (2.0 * u0 - 1.0) * sqrt3;
        r[1] = (2.0 * u1 - 1.0) * sqrt3;
        r[2] = (2.0 * u2 - 1.0) * sqrt3;
        r[3] = (2.0 * u3 - 1.0) * sqrt3;
    } else {
        const double twopi = 6.283185307179586;
        const double ra = sqrt(-2.0 * log(1.0 - u0)), rb = sqrt(-2.0 * log(1.0 - u2));
        r[0] = ra * cos(twopi * u1);
        r[1] = ra * sin(twopi * u1);
        r[2] = rb * cos(twopi * u3);
        r[3] = rb * sin(twopi * u3);
    }
}

__device__ __forceinline__ bool in_acc_region(const MoverArgs &a, const State &s, int ndim) {
    const double xn = (s.x - a.cfg_xmin) / a.cfg_lx;
    bool in = (xn >= a.acc_region[0]) && (xn <= a.acc_region[1]);
    if (ndim > 1) {
        const double yn = (s.y - a.cfg_ymin) / a.cfg_ly;
        in = in && (yn >= a.acc_region[2]) && (yn <= a.acc_region[3]);
    }
    if (ndim == 3) {
        const double zn = (s.z - a.cfg_zmin) / a.cfg_lz;
        in = in && (zn >= a.acc_region[4]) && (zn <= a.acc_region[5]);
    }
    return in;
}

__device__ __forceinline__ double vdrift_prefactor(const MoverArgs &a, double p) {
    const float q = __fdiv_rn(1.0f, (float)(3 * a.charge));
    const double t1 = a.drift1 * a.p0 / p;
    const double t2 = a.drift2 * (a.p0 * a.p0) / (p * p);
    return (double)q / sqrt(t1 * t1 + t2 * t2);
}

__device__ __forceinline__ void push_momentum(const MoverArgs &a, State &s, double dp_dt,
                                              double sdt, double ranp, int ndim, double &deltap) {
    const double dpp = 0.0;
    double dP = dp_dt * s.dt + ranp * sqrt(2.0 * dpp) * sdt;
    if (a.acc_region_flag == 1) {
        if (in_acc_region(a, s, ndim)) s.p = s.p + dP;
        else dP = 0.0;
    } else {
        s.p = s.p + dP;
    }
    const double pfloor = 0.25 * a.p0;
    if (s.p < pfloor) {
        s.p = s.p - dP;
        dP = pfloor - s.p;
        s.p = pfloor;
    }
    deltap = dP;
}

// Kappa (norms, square roots) shared by both dimensions.
struct KBase {
    double kpara, kperp, skpara, skperp, skpp, kpp, b, ib1, ib2, ib3;
};

__device__ __forceinline__ KBase kappa_base(const MoverArgs &a, double p, double bx, double by,
                                            double bz) {
    KBase k;
    k.b = sqrt(bx * bx + by * by + bz * bz);
    k.ib1 = (k.b < DBL_EPSILON) ? 1.0 : 1.0 / k.b;
    k.ib2 = k.ib1 * k.ib1;
    k.ib3 = k.ib1 * k.ib2;
    double knorm_para = 1.0, knorm;
    if (a.mag_dependency == 1) knorm_para = knorm_para * pow(k.b, a.gamma_turb - 2.0);
    if (a.momentum_dependency == 1) knorm = knorm_para * pow(p / a.p0, a.pindex);
    else knorm = knorm_para;
    k.kpara = a.kpara0 * knorm;
    k.kperp = k.kpara * a.kret;
    k.skpara = sqrt(2.0 * k.kpara);
    k.skperp = sqrt(2.0 * k.kperp);
    k.skpp = sqrt(2.0 * (k.kpara - k.kperp));
    k.kpp = k.kpara - k.kperp;
    return k;
}

__device__ __forceinline__ void push2d(const MoverArgs &a, State &s, const double *f, bool fixed_dt,
                                       double &dX_o, double &dY_o, double &dZ_o, double &dP_o) {
    const double bx = f[A_BX], by = f[A_BY], bz = f[A_BZ];
    const KBase k = kappa_base(a, s.p, bx, by, bz);
    // kappa gradients, 2D branch (:2351-2388)
    const double dbx_dx = f[A_DBXDX], dbx_dy = f[A_DBXDY], dby_dx = f[A_DBYDX], dby_dy = f[A_DBYDY];
    const double db_dx = f[A_DBDX], db_dy = f[A_DBDY];
    double dkdx = 0.0, dkdy = 0.0;
    if (a.mag_dependency == 1) {
        dkdx = db_dx * k.ib1 * (a.gamma_turb - 2.0);
        dkdy = db_dy * k.ib1 * (a.gamma_turb - 2.0);
    }
    const double b = k.b, kpp = k.kpp, kperp = k.kperp;
    const double ib2k = k.ib2, ib3k = k.ib3;
    const double dkxx_dx = kperp * dkdx + kpp * dkdx * (bx * bx) * ib2k +
                           2.0 * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3k;
    const double dkyy_dy = kperp * dkdy + kpp * dkdy * (by * by) * ib2k +
                           2.0 * kpp * by * (dby_dy * b - by * db_dy) * ib3k;
    const double dkxy_dx = kpp * dkdx * bx * by * ib2k +
                           kpp * ((dbx_dx * by + bx * dby_dx) * ib2k - 2.0 * bx * by * db_dx * ib3k);
    const double dkxy_dy = kpp * dkdy * bx * by * ib2k +
                           kpp * ((dbx_dy * by + bx * dby_dy) * ib2k - 2.0 * bx * by * db_dy * ib3k);
    // push_particle_2d (:3358-3606)
    const double vx = f[A_VX], vy = f[A_VY];
    const double dvx_dx = f[A_DVXDX], dvy_dy = f[A_DVYDY];
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    const double dbz_dx = f[A_DBZDX], dbz_dy = f[A_DBZDY];
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor(a, s.p);
    const double vdx = vdp * (dbz_dy * ib2 - 2.0 * bz * db_dy * ib3);
    const double vdy = vdp * (-(dbz_dx * ib2) + 2.0 * bz * db_dx * ib3);
    double vdz = 0.0;
    if (a.check_drift_2d)
        vdz = vdp * ((dby_dx - dbx_dy) * ib2 - 2.0 * (by * db_dx - bx * db_dy) * ib3);
    const double dx_dt = vx + vdx + dkxx_dx + dkxy_dy;
    const double dy_dt = vy + vdy + dkxy_dx + dkyy_dy;
    const double dz_dt = vdz;
    const double divv = dvx_dx + dvy_dy;
    const double dp_dt = -(s.p * divv / 3.0);
    const double skpara = k.skpara, skperp = k.skperp;
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double q = 0.5 * a.dx / skpara, m = q * q;
            q = 0.5 * a.dy / skpara; if (q * q < m) m = q * q;
            q = sk / dx_dt; if (q * q < m) m = q * q;
            q = sk / dy_dt; if (q * q < m) m = q * q;
            q = (double)0.1f * s.p / fabs(dp_dt); if (q < m) m = q;
            s.dt = m;
        } else {
            s.dt = a.dt_min;
        }
        if (s.dt < a.dt_min) s.dt = a.dt_min;
        if (s.dt > a.dt_max) s.dt = a.dt_max;
    }
    const double sdt = sqrt(s.dt);
    double r[4];
    noise4(a, s, r);
    const double skpp = k.skpp;
    const double dX = dx_dt * s.dt + r[0] * skperp * sdt + r[2] * skpp * sdt * bx * ib;
    const double dY = dy_dt * s.dt + r[1] * skperp * sdt + r[2] * skpp * sdt * by * ib;
    const double dZ = dz_dt * s.dt;
    s.x = s.x + dX;
    s.y = s.y + dY;
    s.z = s.z + dZ;
    s.t = s.t + s.dt;
    dX_o = dX; dY_o = dY; dZ_o = dZ;
    push_momentum(a, s, dp_dt, sdt, r[3], 2, dP_o);
}

__device__ __forceinline__ void push3d(const MoverArgs &a, State &s, const double *f, bool fixed_dt,
                                       double &dX_o, double &dY_o, double &dZ_o, double &dP_o) {
    const double bx = f[B_BX], by = f[B_BY], bz = f[B_BZ];
    const KBase k = kappa_base(a, s.p, bx, by, bz);
    // kappa gradients, 3D branch (:2389-2449); no 1/B in dkdx (reference).
    const double dbx_dx = f[B_DBXDX], dbx_dy = f[B_DBXDY], dbx_dz = f[B_DBXDZ];
    const double dby_dx = f[B_DBYDX], dby_dy = f[B_DBYDY], dby_dz = f[B_DBYDZ];
    const double dbz_dx = f[B_DBZDX], dbz_dy = f[B_DBZDY], dbz_dz = f[B_DBZDZ];
    const double db_dx = f[B_DBDX], db_dy = f[B_DBDY], db_dz = f[B_DBDZ];
    double dkdx = 0.0, dkdy = 0.0, dkdz = 0.0;
    if (a.mag_dependency == 1) {
        dkdx = db_dx * (a.gamma_turb - 2.0);
        dkdy = db_dy * (a.gamma_turb - 2.0);
        dkdz = db_dz * (a.gamma_turb - 2.0);
    }
    const double b = k.b, kpp = k.kpp, kperp = k.kperp;
    const double ib2k = k.ib2, ib3k = k.ib3;
    const double dkxx_dx = kperp * dkdx + kpp * dkdx * (bx * bx) * ib2k +
                           2.0 * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3k;
    const double dkyy_dy = kperp * dkdy + kpp * dkdy * (by * by) * ib2k +
                           2.0 * kpp * by * (dby_dy * b - by * db_dy) * ib3k;
    const double dkzz_dz = kperp * dkdz + kpp * dkdz * (bz * bz) * ib2k +
                           2.0 * kpp * bz * (dbz_dz * b - bz * db_dz) * ib3k;
    const double dkxy_dx = kpp * dkdx * bx * by * ib2k +
                           kpp * ((dbx_dx * by + bx * dby_dx) * ib2k - 2.0 * bx * by * db_dx * ib3k);
    const double dkxy_dy = kpp * dkdy * bx * by * ib2k +
                           kpp * ((dbx_dy * by + bx * dby_dy) * ib2k - 2.0 * bx * by * db_dy * ib3k);
    const double dkxz_dx = kpp * dkdx * bx * bz * ib2k +
                           kpp * ((dbx_dx * bz + bx * dbz_dx) * ib2k - 2.0 * bx * bz * db_dx * ib3k);
    const double dkxz_dz = kpp * dkdz * bx * bz * ib2k +
                           kpp * ((dbx_dz * bz + bx * dbz_dz) * ib2k - 2.0 * bx * bz * db_dz * ib3k);
    const double dkyz_dy = kpp * dkdy * by * bz * ib2k +
                           kpp * ((dby_dy * bz + by * dbz_dy) * ib2k - 2.0 * by * bz * db_dy * ib3k);
    const double dkyz_dz = kpp * dkdz * by * bz * ib2k +
                           kpp * ((dby_dz * bz + by * dbz_dz) * ib2k - 2.0 * by * bz * db_dz * ib3k);
    // push_particle_3d (:4625-4907)
    const double vx = f[B_VX], vy = f[B_VY], vz = f[B_VZ];
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    const double bxn = bx * ib, byn = by * ib, bzn = bz * ib;
    const double bxyn = sqrt(bxn * bxn + byn * byn);
    const double ibxyn = (bxyn < DBL_EPSILON) ? 0.0 : 1.0 / bxyn;
    const double dvx_dx = f[B_DVXDX], dvy_dy = f[B_DVYDY], dvz_dz = f[B_DVZDZ];
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor(a, s.p);
    const double vdx = vdp * ((dbz_dy - dby_dz) * ib2 - 2.0 * (bz * db_dy - by * db_dz) * ib3);
    const double vdy = vdp * ((dbx_dz - dbz_dx) * ib2 - 2.0 * (bx * db_dz - bz * db_dx) * ib3);
    const double vdz = vdp * ((dby_dx - dbx_dy) * ib2 - 2.0 * (by * db_dx - bx * db_dy) * ib3);
    const double dx_dt = vx + vdx + dkxx_dx + dkxy_dy + dkxz_dz;
    const double dy_dt = vy + vdy + dkxy_dx + dkyy_dy + dkyz_dz;
    const double dz_dt = vz + vdz + dkxz_dx + dkyz_dy + dkzz_dz;
    const double divv = dvx_dx + dvy_dy + dvz_dz;
    const double dp_dt = -(s.p * divv / 3.0);
    const double skpara = k.skpara, skperp = k.skperp;
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double q = 0.5 * a.dx / skpara, m = q * q;
            q = 0.5 * a.dy / skpara; if (q * q < m) m = q * q;
            q = 0.5 * a.dz / skpara; if (q * q < m) m = q * q;
            q = sk / dx_dt; if (q * q < m) m = q * q;
            q = sk / dy_dt; if (q * q < m) m = q * q;
            q = sk / dz_dt; if (q * q < m) m = q * q;
            q = (double)0.1f * s.p / fabs(dp_dt); if (q < m) m = q;
            s.dt = m;
        } else {
            s.dt = a.dt_min;
        }
        if (s.dt < a.dt_min) s.dt = a.dt_min;
        if (s.dt > a.dt_max) s.dt = a.dt_max;
    }
    const double sdt = sqrt(s.dt);
    double r[4];
    noise4(a, s, r);
    const double dX = dx_dt * s.dt +
        (bxn * skpara * r[0] - bxn * bzn * skperp * ibxyn * r[1] - byn * skperp * ibxyn * r[2]) * sdt;
    const double dY = dy_dt * s.dt +
        (byn * skpara * r[0] - byn * bzn * skperp * ibxyn * r[1] + bxn * skperp * ibxyn * r[2]) * sdt;
    const double dZ = dz_dt * s.dt + (bzn * skpara * r[0] + bxyn * skperp * r[1]) * sdt;
    s.x = s.x + dX;
    s.y = s.y + dY;
    s.z = s.z + dZ;
    s.t = s.t + s.dt;
    dX_o = dX; dY_o = dY; dZ_o = dZ;
    push_momentum(a, s, dp_dt, sdt, r[3], 3, dP_o);
}

template <int NDIM>
__device__ __forceinline__ void boundary(const MoverArgs &a, State &s, double xlo, double xhi,
                                         double ylo, double yhi, double zlo, double zhi, Acc &acc) {
    if (s.x < xlo && s.flag == 1) {
        if (a.pbcx) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -1; }
        else s.x = s.x - xlo + xhi;
    } else if (s.x > xhi && s.flag == 1) {
        if (a.pbcx) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -2; }
        else s.x = s.x - xhi + xlo;
    }
    if (s.y < ylo && s.flag == 1) {
        if (a.pbcy) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -3; }
        else s.y = s.y - ylo + yhi;
    } else if (s.y > yhi && s.flag == 1) {
        if (a.pbcy) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -4; }
        else s.y = s.y - yhi + ylo;
    }
    if (NDIM == 3) {
        if (s.z < zlo && s.flag == 1) {
            if (a.pbcz) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -5; }
            else s.z = s.z - zlo + zhi;
        } else if (s.z > zhi && s.flag == 1) {
            if (a.pbcz) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -6; }
            else s.z = s.z - zhi + zlo;
        }
    }
}

template <int NDIM>
__device__ __forceinline__ void negp_or_boundary(const MoverArgs &a, State &s, Acc &acc) {
    if (s.p < 0.0) {
        s.flag = 0;
        acc_add(acc.negp_h, acc.negp_l, s.w);
    } else {
        boundary<NDIM>(a, s, a.xmin1, a.xmax1, a.ymin1, a.ymax1, a.zmin1, a.zmax1, acc);
    }
}

template <int NDIM>
__device__ __forceinline__ bool do_push(const MoverArgs &a, State &s, bool fixed_dt, double &dX,
                                        double &dY, double &dZ, double &dP) {
    constexpr int NV = (NDIM == 2) ? 15 : 21;
    double f[NV];
    if (!interp<NDIM, NV>(a, s, f)) return false;
    if (NDIM == 2) push2d(a, s, f, fixed_dt, dX, dY, dZ, dP);
    else push3d(a, s, f, fixed_dt, dX, dY, dZ, dP);
    if (!isfinite(s.x) || !isfinite(s.y) || !isfinite(s.z) || !isfinite(s.p) || !isfinite(s.t)) {
        set_status(a.cnt, kStatusNonFinite);
        return false;
    }
    return true;
}

template <int NDIM>
__global__ void __launch_bounds__(128) mover_fp64_kernel(const MoverArgs a) {
    Acc acc = {0, 0, 0, 0, 0};
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n) {
        State s;
        s.x = a.P.x[i]; s.y = a.P.y[i]; s.z = a.P.z[i]; s.p = a.P.p[i];
        s.t = a.P.t[i]; s.dt = a.P.dt[i]; s.w = a.P.weight[i];
        s.flag = a.P.count_flag[i];
        s.nsteps_pushed = a.P.nsteps_pushed[i];
        s.tag_inj = a.P.tag_injected[i];
        s.tag_spl = a.P.tag_splitted[i];
        s.ctr = a.P.rng_ctr[i];
        const double t0 = a.t0, dt_fine = a.dt_fine;
        double deltax = 0.0, deltay = 0.0, deltaz = 0.0, deltap = 0.0;
        const double step = ceil((s.t - t0) / dt_fine);
        double dt_target = (step <= 0.0) ? dt_fine : step * dt_fine;
        if (dt_target > a.dtf) dt_target = a.dtf;
        if (s.p < 0.0 && s.flag == 1) {
            s.flag = 0;
            acc_add(acc.negp_h, acc.negp_l, s.w);
        } else {
            boundary<NDIM>(a, s, a.xmin1, a.xmax1, a.ymin1, a.ymax1, a.zmin1, a.zmax1, acc);
        }
        uint32_t pushes = 0;
        bool alive = (s.flag == 1);
        while (alive && dt_target < a.limit) {
            if (s.flag != 1) break;
            while ((s.t - t0) < dt_target && s.flag == 1) {
                negp_or_boundary<NDIM>(a, s, acc);
                if (s.flag != 1) break;
                if (pushes >= a.max_pushes) { set_status(a.cnt, kStatusStepLimit); alive = false; break; }
                if (!do_push<NDIM>(a, s, false, deltax, deltay, deltaz, deltap)) {
                    s.flag = 0; alive = false; break;
                }
                ++pushes;
                s.nsteps_pushed = (s.nsteps_pushed + 1) % a.nsteps_interval;
            }
            if (!alive) break;
            if ((s.t - t0) > dt_target && s.flag == 1) {
                s.x = s.x - deltax;
                s.y = s.y - deltay;
                s.z = s.z - deltaz;
                s.p = s.p - deltap;
                s.t = s.t - s.dt;
                const double dt_old = s.dt;
                s.dt = t0 + dt_target - s.t;
                if (s.dt > 0.0) {
                    s.nsteps_pushed = s.nsteps_pushed - 1;
                    if (!do_push<NDIM>(a, s, true, deltax, deltay, deltaz, deltap)) {
                        s.flag = 0; alive = false; break;
                    }
                    ++pushes;
                    s.nsteps_pushed = (s.nsteps_pushed + 1) % a.nsteps_interval;
                }
                s.dt = dt_old;
                negp_or_boundary<NDIM>(a, s, acc);
            }
            dt_target = dt_target + dt_fine;
        }
        // End-of-interval boundary pass on the exact box (:1959-1973); it
        // only acts on particles still in the box.
        if (s.flag == 1)
            boundary<NDIM>(a, s, a.xmin, a.xmax, a.ymin, a.ymax, a.zmin, a.zmax, acc);
        acc.steps = pushes;
        a.P.x[i] = s.x; a.P.y[i] = s.y; a.P.z[i] = s.z; a.P.p[i] = s.p;
        a.P.t[i] = s.t; a.P.dt[i] = s.dt;
        a.P.count_flag[i] = (int8_t)s.flag;
        a.P.nsteps_pushed[i] = s.nsteps_pushed;
        a.P.nsteps_tracked[i] = 1;
        a.P.rng_ctr[i] = s.ctr;
    }
    // Warp-aggregated counters.
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

cudaError_t launch_mover_fp64(const MoverArgs &a, int sm_count, cudaStream_t s) {
    (void)sm_count;
    if (a.n <= 0) return cudaSuccess;
    const int threads = 128;
    const int64_t blocks = (a.n + threads - 1) / threads;
    if (a.ndim == 2) mover_fp64_kernel<2><<<(unsigned)blocks, threads, 0, s>>>(a);
    else mover_fp64_kernel<3><<<(unsigned)blocks, threads, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace gpat
