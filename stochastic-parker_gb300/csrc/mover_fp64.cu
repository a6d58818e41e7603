// FP64 particle mover: the reference's Parker path with its exact operation
// order.  This translation unit is compiled with -fmad=false so every
// +, -, *, / and sqrt is a single IEEE-rounded operation, which makes the
// trajectories bit-identical to a CPU FP64 evaluation of the same formulas
// (only pow() -- momentum/|B|-dependent kappa, focused transport's D_mumu --
// is library-dependent).
//
// Follows particle_mover_one_cycle (particle_module.f90:1481-1833),
// get_interp_paramters (:642-674), interp_fields (mhd_data_parallel.f90:
// 1751-1804), calc_spatial_diffusion_coefficients (:2208-2450) and its NLGC
// variant (:2464-2771), push_particle_2d (:3358-3606), push_particle_3d
// (:4625-4907), the focused-transport pushes push_particle_2d_ft
// (:3626-3964) and push_particle_3d_ft (:4930-5324) with calc_duu
// (:3116-3155), and particle_boundary_condition (:1984-2129) on one rank.
#include <cfloat>

#include "device_common.cuh"
#include "grid_common.cuh"
#include "track_common.cuh"

namespace gpat {
namespace {

// Packed record slots (fields.cu).
enum R2 { A_VX, A_VY, A_BX, A_BY, A_BZ, A_DVXDX, A_DVYDY, A_DBXDX, A_DBXDY, A_DBYDX, A_DBYDY,
          A_DBZDX, A_DBZDY, A_DBDX, A_DBDY };
enum R3 { B_VX, B_VY, B_VZ, B_BX, B_BY, B_BZ, B_DVXDX, B_DVYDY, B_DVZDZ, B_DBXDX, B_DBXDY,
          B_DBXDZ, B_DBYDX, B_DBYDY, B_DBYDZ, B_DBZDX, B_DBZDY, B_DBZDZ, B_DBDX, B_DBDY, B_DBDZ };

struct State {
    double x, y, z, p, v, mu, t, dt, w;
    double h1, h2;   // acceleration-surface heights at the push's start
    int flag;
    int32_t nsteps_pushed, tag_inj, tag_spl;
    uint32_t ctr;
};

// deltax, deltay, deltaz, deltap, deltav, deltamu of particle_mover_one_cycle.
struct Delta {
    double x, y, z, p, v, mu;
};

struct Acc {
    unsigned long long leak_h, leak_l, negp_h, negp_l, steps;
};

__device__ __forceinline__ void acc_add(unsigned long long &h, unsigned long long &l, double w) {
    unsigned long long bh, bl;
    fixed_split(w, bh, bl);
    add_u128(h, l, bh, bl);
}

// NV variables of records of R floats interpolated with corner (ix, iy, iz)
// and weights w, time-interpolated between the two frames.
template <int NDIM, int NV, int R>
__device__ __forceinline__ void interp_at(const MoverArgs &a, const float *rec1, const float *rec2,
                                          const State &s, int ix, int iy, int iz, const double *w,
                                          double f[NV]);

// get_interp_paramters on the uniform grid: the lower corner (memory
// indices) and the 8 weights; false outside the ghost cells.
template <int NDIM>
__device__ __forceinline__ bool uniform_cell(const MoverArgs &a, const State &s, int &ix, int &iy,
                                             int &iz, double w[8]);

// Interpolated fields at the particle: NV variables of records of R floats.
template <int NDIM, int NV, int R>
__device__ __forceinline__ bool interp(const MoverArgs &a, const float *rec1, const float *rec2,
                                       const State &s, double f[NV]) {
    int ix, iy, iz;
    double w[8];
    if (!uniform_cell<NDIM>(a, s, ix, iy, iz, w)) return false;
    interp_at<NDIM, NV, R>(a, rec1, rec2, s, ix, iy, iz, w, f);
    return true;
}

template <int NDIM>
__device__ __forceinline__ bool uniform_cell(const MoverArgs &a, const State &s, int &ix, int &iy,
                                             int &iz, double w[8]) {
    const double px = (s.x - a.xmin) / a.dx;
    const double py = (s.y - a.ymin) / a.dy;
    const double pz = (s.z - a.zmin) / a.dz;
    const int nx = a.nxg - 4, ny = a.nyg - 4, nz = a.nzg - 4;
    if (!(px >= -1.0 && px < nx + 1.0) || (NDIM > 1 && !(py >= -1.0 && py < ny + 1.0)) ||
        (NDIM == 3 && !(pz >= -1.0 && pz < nz + 1.0))) {
        set_status(a.cnt, kStatusIndexGuard);
        return false;
    }
    // get_interp_paramters: pos = floor(p) + 1 (Fortran), r = p - pos + 1;
    // 1D: pos = (floor(px) + 1, 1, 1), ry = rz = 0 (:649-652).
    const int fx = (int)floor(px), fy = (NDIM > 1) ? (int)floor(py) : -2;
    const int fz = (NDIM == 3) ? (int)floor(pz) : 0;
    const double rx = (px - (double)(fx + 1)) + 1.0;
    const double ry = (NDIM > 1) ? (py - (double)(fy + 1)) + 1.0 : 0.0;
    const double rz = (NDIM == 3) ? (pz - (double)(fz + 1)) + 1.0 : 0.0;
    const double rx1 = 1.0 - rx, ry1 = 1.0 - ry, rz1 = 1.0 - rz;
    w[0] = rx1 * ry1 * rz1;
    w[1] = rx * ry1 * rz1;
    w[2] = rx1 * ry * rz1;
    w[3] = rx * ry * rz1;
    w[4] = rx1 * ry1 * rz;
    w[5] = rx * ry1 * rz;
    w[6] = rx1 * ry * rz;
    w[7] = rx * ry * rz;
    ix = fx + 2;
    iy = fy + 2;   // 0 in 1D, whose arrays have one y node
    iz = (NDIM == 3) ? fz + 2 : 0;
    return true;
}

template <int NDIM, int NV, int R>
__device__ __forceinline__ void interp_at(const MoverArgs &a, const float *rec1, const float *rec2,
                                          const State &s, int ix, int iy, int iz, const double *w,
                                          double f[NV]) {
    double f2[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) { f[v] = 0.0; f2[v] = 0.0; }
    const double rt = (s.t - a.t0) / a.dtf;
#pragma unroll
    for (int k = 0; k < (NDIM == 3 ? 2 : 1); ++k)
#pragma unroll
        for (int j = 0; j < (NDIM >= 2 ? 2 : 1); ++j)
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const double wc = w[k * 4 + j * 2 + i];
                const size_t cell = (size_t)(ix + i) +
                                    (size_t)a.nxg * ((size_t)(iy + j) + (size_t)a.nyg * (size_t)(iz + k));
                const float4 *r4 = reinterpret_cast<const float4 *>(rec1 + (size_t)R * cell);
#pragma unroll
                for (int q = 0; q < (NV + 3) / 4; ++q) {
                    const float4 v4 = __ldg(r4 + q);
                    const float vv[4] = {v4.x, v4.y, v4.z, v4.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        if (4 * q + e < NV) f[4 * q + e] = f[4 * q + e] + (double)vv[e] * wc;
                }
                if (a.time_interp) {
                    const float4 *s4 = reinterpret_cast<const float4 *>(rec2 + (size_t)R * cell);
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
}

// Field values at the particle under the reference's names.
struct Fld {
    double vx, vy, vz, rho, bx, by, bz;
    double dvx_dx, dvx_dy, dvx_dz, dvy_dx, dvy_dy, dvy_dz, dvz_dx, dvz_dy, dvz_dz;
    double dbx_dx, dbx_dy, dbx_dz, dby_dx, dby_dy, dby_dz, dbz_dx, dbz_dy, dbz_dz;
    double db_dx, db_dy, db_dz;
};

// From the full 32-variable layout (interp_fields order, 0-based).
__device__ __forceinline__ Fld named_full(const double *f) {
    Fld q;
    q.vx = f[0]; q.vy = f[1]; q.vz = f[2]; q.rho = f[3]; q.bx = f[4]; q.by = f[5]; q.bz = f[6];
    q.dvx_dx = f[8]; q.dvx_dy = f[9]; q.dvx_dz = f[10];
    q.dvy_dx = f[11]; q.dvy_dy = f[12]; q.dvy_dz = f[13];
    q.dvz_dx = f[14]; q.dvz_dy = f[15]; q.dvz_dz = f[16];
    q.dbx_dx = f[20]; q.dbx_dy = f[21]; q.dbx_dz = f[22];
    q.dby_dx = f[23]; q.dby_dy = f[24]; q.dby_dz = f[25];
    q.dbz_dx = f[26]; q.dbz_dy = f[27]; q.dbz_dz = f[28];
    q.db_dx = f[29]; q.db_dy = f[30]; q.db_dz = f[31];
    return q;
}

// From the packed records, which hold what the Parker pushes read.
template <int NDIM>
__device__ __forceinline__ Fld named_packed(const double *f) {
    Fld q = {};
    if (NDIM == 2) {
        q.vx = f[A_VX]; q.vy = f[A_VY]; q.bx = f[A_BX]; q.by = f[A_BY]; q.bz = f[A_BZ];
        q.dvx_dx = f[A_DVXDX]; q.dvy_dy = f[A_DVYDY];
        q.dbx_dx = f[A_DBXDX]; q.dbx_dy = f[A_DBXDY]; q.dby_dx = f[A_DBYDX]; q.dby_dy = f[A_DBYDY];
        q.dbz_dx = f[A_DBZDX]; q.dbz_dy = f[A_DBZDY]; q.db_dx = f[A_DBDX]; q.db_dy = f[A_DBDY];
    } else {
        q.vx = f[B_VX]; q.vy = f[B_VY]; q.vz = f[B_VZ];
        q.bx = f[B_BX]; q.by = f[B_BY]; q.bz = f[B_BZ];
        q.dvx_dx = f[B_DVXDX]; q.dvy_dy = f[B_DVYDY]; q.dvz_dz = f[B_DVZDZ];
        q.dbx_dx = f[B_DBXDX]; q.dbx_dy = f[B_DBXDY]; q.dbx_dz = f[B_DBXDZ];
        q.dby_dx = f[B_DBYDX]; q.dby_dy = f[B_DBYDY]; q.dby_dz = f[B_DBYDZ];
        q.dbz_dx = f[B_DBZDX]; q.dbz_dy = f[B_DBZDY]; q.dbz_dz = f[B_DBZDZ];
        q.db_dx = f[B_DBDX]; q.db_dy = f[B_DBDY]; q.db_dz = f[B_DBDZ];
    }
    return q;
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

// noise4 plus r[4], r[5] from a third Philox block of the same push (the 3D
// spherical focused-transport push draws five numbers).
__device__ __forceinline__ void noise6(const MoverArgs &a, State &s, double r[6]) {
    const uint4 w2 = philox4x32_10(make_uint4(s.ctr, 2u, (uint32_t)s.tag_inj, (uint32_t)s.tag_spl),
                                   a.key0, a.key1);
    const double u4 = u01_53(w2.x, w2.y), u5 = u01_53(w2.z, w2.w);
    if (a.noise == GPAT_NOISE_UNIFORM) {
        r[4] = (2.0 * u4 - 1.0) * sqrt(3.0);
        r[5] = (2.0 * u5 - 1.0) * sqrt(3.0);
    } else {
        const double rc = sqrt(-2.0 * log(1.0 - u4));
        r[4] = rc * cos(6.283185307179586 * u5);
        r[5] = rc * sin(6.283185307179586 * u5);
    }
    noise4(a, s, r);
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
        if (a.surf_on) {
            // check_above_acc_surface (acc_region_surface.f90:343-383), as
            // push_particle_3d / _3d_ft apply it (:4889-4893)
            const double xyz[3] = {s.x, s.y, s.z};
            double ph = xyz[a.surf_axis[0]];
            bool up = a.surf_sign[0] > 0 ? ph > s.h1 : ph < s.h1;
            if (a.surf_has2) {
                ph = xyz[a.surf_axis[1]];
                const bool up2 = a.surf_sign[1] > 0 ? ph > s.h2 : ph < s.h2;
                up = a.surf_inter ? (up && up2) : (up || up2);
            }
            in = in && up;
        }
    }
    return in;
}

// interp_acc_surface (acc_region_surface.f90:255-335): the 3D weights
// summed along the surface normal, corners summed in Fortran's order.
__device__ __forceinline__ double surface_height(const MoverArgs &a, int k, int ix, int iy,
                                                 int iz, const double *w, double rt) {
    const int ax = a.surf_axis[k];
    int i1, j1;
    double w2[4];
    if (ax == 0) {
        i1 = iy; j1 = iz;
        w2[0] = w[0] + w[1]; w2[1] = w[2] + w[3]; w2[2] = w[4] + w[5]; w2[3] = w[6] + w[7];
    } else if (ax == 1) {
        i1 = ix; j1 = iz;
        w2[0] = w[0] + w[2]; w2[1] = w[1] + w[3]; w2[2] = w[4] + w[6]; w2[3] = w[5] + w[7];
    } else {
        i1 = ix; j1 = iy;
        w2[0] = w[0] + w[4]; w2[1] = w[1] + w[5]; w2[2] = w[2] + w[6]; w2[3] = w[3] + w[7];
    }
    const size_t ld = (size_t)a.surf_ld[k];
    double hs[2] = {0.0, 0.0};
    for (int t = 0; t < (a.time_interp ? 2 : 1); ++t) {
        const double *h = a.surf[k][t];
        double sum = 0.0;
        sum = sum + __ldg(h + (size_t)i1 + ld * (size_t)j1) * w2[0];
        sum = sum + __ldg(h + (size_t)i1 + 1 + ld * (size_t)j1) * w2[1];
        sum = sum + __ldg(h + (size_t)i1 + ld * (size_t)(j1 + 1)) * w2[2];
        sum = sum + __ldg(h + (size_t)i1 + 1 + ld * (size_t)(j1 + 1)) * w2[3];
        hs[t] = sum;
    }
    return a.time_interp ? hs[0] * (1.0 - rt) + hs[1] * rt : hs[0];
}

__device__ __forceinline__ void surface_heights(const MoverArgs &a, State &s, int ix, int iy,
                                                int iz, const double *w) {
    const double rt = (s.t - a.t0) / a.dtf;
    s.h1 = surface_height(a, 0, ix, iy, iz, w, rt);
    s.h2 = a.surf_has2 ? surface_height(a, 1, ix, iy, iz, w, rt) : 0.0;
}

// 1 / (3 pcharge) (Parker) or 1 / pcharge (focused transport) is single
// precision in the reference.
__device__ __forceinline__ double vdrift_prefactor(const MoverArgs &a, double p, int qmul) {
    const float q = __fdiv_rn(1.0f, (float)(qmul * a.charge));
    const double t1 = a.drift1 * a.p0 / p;
    const double t2 = a.drift2 * (a.p0 * a.p0) / (p * p);
    return (double)q / sqrt(t1 * t1 + t2 * t2);
}

__device__ __forceinline__ void push_momentum(const MoverArgs &a, State &s, double dp_dt,
                                              double dpp, double sdt, double ranp, int ndim,
                                              double &deltap) {
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

// calc_spatial_diffusion_coefficients (:2208-2450) or its NLGC variant
// (:2464-2771).  The gradient terms are written as
//   dkii_di = T_i + A_i bi^2 / B^2 + 2 kpp bi (dbi_di B - bi dB_di) / B^3
//   dkij_dk = A_k bi bj / B^2 + kpp ((dbi_dk bj + bi dbj_dk) / B^2 - 2 bi bj dB_dk / B^3)
// with T_i = kperp dk_i, A_i = kpp dk_i (fixed ratio) or T_i = kperp dkperp_i,
// A_i = kpara dkpara_i - kperp dkperp_i (NLGC), each in the reference's order.
struct Kap {
    double knorm_para, kpara, kperp, skpara, skperp, skpp;
    double dkxx_dx, dkyy_dy, dkzz_dz, dkxy_dx, dkxy_dy, dkxz_dx, dkxz_dz, dkyz_dy, dkyz_dz;
    double kxx, kyy, kzz, kxy, kxz, kyz;   // read by the spherical pushes
};

// aux: interpolated {db2_slab, db2_2d, lc_slab, lc_2d} x {value, d/dx, d/dy,
// d/dz}, or nullptr; read when deltab_flag / correlation_flag are on.
// I3 (with NDIM = 3): include_3rd_dim of a 2D run, the 3D tensor with the z
// derivatives zero and the 2D gradient terms (:2293-2350, :2564-2640).
template <int NDIM, bool FT, bool I3 = false>
__device__ __forceinline__ Kap kappa(const MoverArgs &a, double p, double mu, const Fld &f,
                                     const double *aux) {
    const bool dbf = a.deltab_flag && aux, lcf = a.correlation_flag && aux;
    const double *s2 = aux, *d2 = aux + 4, *l1 = aux + 8, *l2 = aux + 12;
    const double bx = f.bx, by = f.by, bz = f.bz;
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double ib1 = (b < DBL_EPSILON) ? 1.0 : 1.0 / b;
    const double ib2 = ib1 * ib1;
    const double ib3 = ib1 * ib2;
    double kpara, kperp, knorm_para = 1.0;
    if (!a.nlgc) {
        double knorm;
        if (a.mag_dependency == 1) knorm_para = knorm_para * pow(b, a.gamma_turb - 2.0);
        if (dbf) knorm_para = knorm_para / s2[0];
        if (lcf) knorm_para = knorm_para * pow(l1[0], a.gamma_turb - 1.0);
        if (a.momentum_dependency == 1) knorm = knorm_para * pow(p / a.p0, a.pindex);
        else knorm = knorm_para;
        kpara = a.kpara0 * knorm;
        kperp = kpara * a.kret;
    } else {
        double knorm_perp = 1.0, kn_para, kn_perp;
        if (a.mag_dependency == 1) {
            knorm_para = knorm_para * pow(b, a.gamma_turb - 2.0);
            knorm_perp = knorm_perp * pow(b, (a.gamma_turb - 2.0) / 3.0);
        }
        if (dbf) {
            knorm_para = knorm_para / s2[0];
            knorm_perp = knorm_perp * pow(s2[0], -1.0 / 3.0) * pow(d2[0], 2.0 / 3.0);
        }
        if (lcf) {
            knorm_para = knorm_para * pow(l1[0], a.gamma_turb - 1.0);
            knorm_perp = knorm_perp * pow(l1[0], (a.gamma_turb - 1.0) / 3.0) *
                         pow(l2[0], 2.0 / 3.0);
        }
        if (a.momentum_dependency == 1) {
            kn_para = knorm_para * pow(p / a.p0, a.pindex);
            kn_perp = knorm_perp * pow(p / a.p0, (5.0 - a.gamma_turb) / 3.0);
        } else {
            kn_para = knorm_para;
            kn_perp = knorm_perp;
        }
        kpara = a.kpara0 * kn_para;
        kperp = a.kpara0 * a.kperp_kpara * kn_perp * (mu * mu);
    }
    Kap k;
    k.knorm_para = knorm_para;
    k.kpara = kpara;
    k.kperp = kperp;
    k.skpara = sqrt(2.0 * kpara);
    k.skperp = sqrt(2.0 * kperp);
    k.skpp = sqrt(2.0 * (kpara - kperp));
    const double kpp = FT ? -kperp : kpara - kperp;
    if (NDIM == 1) {
        // the 1D branches (:2270-2291, :2536-2562): dkxx_dx, and kxx for
        // spherical coordinates
        double dk = 0.0, dkperp = 0.0;
        if (a.mag_dependency == 1) {
            dk = f.db_dx * ib1 * (a.gamma_turb - 2.0);
            dkperp = f.db_dx * ib1 * (a.gamma_turb - 2.0) / 3.0;
        }
        if (dbf) {
            dk = dk - s2[1] / s2[0];
            dkperp = dkperp - s2[1] / s2[0] / 3.0 + 2.0 * d2[1] / d2[0] / 3.0;
        }
        if (lcf) {
            dk = dk + (a.gamma_turb - 1.0) * l1[1] / l1[0];
            dkperp = dkperp + (a.gamma_turb - 1.0) * l1[1] / l1[0] / 3.0 +
                     2.0 * l2[1] / l2[0] / 3.0;
        }
        if (!a.nlgc) dkperp = dk;
        k.dkxx_dx = FT ? kperp * dkperp : kpara * dk;
        k.kxx = a.spherical ? (FT ? kperp : kpara) : 0.0;
        k.dkyy_dy = 0.0; k.dkzz_dz = 0.0; k.dkxy_dx = 0.0; k.dkxy_dy = 0.0;
        k.dkxz_dx = 0.0; k.dkxz_dz = 0.0; k.dkyz_dy = 0.0; k.dkyz_dz = 0.0;
        k.kyy = 0.0; k.kzz = 0.0; k.kxy = 0.0; k.kxz = 0.0; k.kyz = 0.0;
        return k;
    }
    const double db[3] = {f.db_dx, f.db_dy, f.db_dz};
    const double g2 = a.gamma_turb - 2.0;
    double T[3] = {0.0, 0.0, 0.0}, A[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < (I3 ? 2 : NDIM); ++d) {
        if (!a.nlgc) {
            double dk = 0.0;
            // the fixed-ratio 3D branch has no 1/B factor (:2406-2408)
            if (a.mag_dependency == 1) dk = (NDIM == 3 && !I3) ? db[d] * g2 : db[d] * ib1 * g2;
            if (dbf) dk = dk - s2[1 + d] / s2[0];
            if (lcf) dk = dk + (a.gamma_turb - 1.0) * l1[1 + d] / l1[0];
            T[d] = kperp * dk;
            A[d] = kpp * dk;
        } else {
            double dkpara = 0.0, dkperp = 0.0;
            if (a.mag_dependency == 1) {
                dkpara = db[d] * ib1 * g2;
                dkperp = db[d] * ib1 * g2 / 3.0;
            }
            if (dbf) {
                dkpara = dkpara - s2[1 + d] / s2[0];
                dkperp = dkperp - s2[1 + d] / s2[0] / 3.0 + 2.0 * d2[1 + d] / d2[0] / 3.0;
            }
            if (lcf) {
                dkpara = dkpara + (a.gamma_turb - 1.0) * l1[1 + d] / l1[0];
                dkperp = dkperp + (a.gamma_turb - 1.0) * l1[1 + d] / l1[0] / 3.0 +
                         2.0 * l2[1 + d] / l2[0] / 3.0;
            }
            T[d] = kperp * dkperp;
            A[d] = kpara * dkpara - kperp * dkperp;
        }
    }
    k.dkxx_dx = T[0] + A[0] * (bx * bx) * ib2 + 2.0 * kpp * bx * (f.dbx_dx * b - bx * f.db_dx) * ib3;
    k.dkyy_dy = T[1] + A[1] * (by * by) * ib2 + 2.0 * kpp * by * (f.dby_dy * b - by * f.db_dy) * ib3;
    k.dkxy_dx = A[0] * bx * by * ib2 +
                kpp * ((f.dbx_dx * by + bx * f.dby_dx) * ib2 - 2.0 * bx * by * f.db_dx * ib3);
    k.dkxy_dy = A[1] * bx * by * ib2 +
                kpp * ((f.dbx_dy * by + bx * f.dby_dy) * ib2 - 2.0 * bx * by * f.db_dy * ib3);
    k.kxx = kperp + kpp * bx * bx * ib2;
    k.kyy = kperp + kpp * by * by * ib2;
    k.kxy = kpp * bx * by * ib2;
    k.kzz = (NDIM == 3) ? kperp + kpp * bz * bz * ib2 : 0.0;
    k.kxz = (NDIM == 3) ? kpp * bx * bz * ib2 : 0.0;
    k.kyz = (NDIM == 3) ? kpp * by * bz * ib2 : 0.0;
    if (NDIM == 3) {
        k.dkzz_dz = T[2] + A[2] * (bz * bz) * ib2 +
                    2.0 * kpp * bz * (f.dbz_dz * b - bz * f.db_dz) * ib3;
        k.dkxz_dx = A[0] * bx * bz * ib2 +
                    kpp * ((f.dbx_dx * bz + bx * f.dbz_dx) * ib2 - 2.0 * bx * bz * f.db_dx * ib3);
        k.dkxz_dz = A[2] * bx * bz * ib2 +
                    kpp * ((f.dbx_dz * bz + bx * f.dbz_dz) * ib2 - 2.0 * bx * bz * f.db_dz * ib3);
        k.dkyz_dy = A[1] * by * bz * ib2 +
                    kpp * ((f.dby_dy * bz + by * f.dbz_dy) * ib2 - 2.0 * by * bz * f.db_dy * ib3);
        k.dkyz_dz = A[2] * by * bz * ib2 +
                    kpp * ((f.dby_dz * bz + by * f.dbz_dz) * ib2 - 2.0 * by * bz * f.db_dz * ib3);
    } else {
        k.dkzz_dz = 0.0; k.dkxz_dx = 0.0; k.dkxz_dz = 0.0; k.dkyz_dy = 0.0; k.dkyz_dz = 0.0;
    }
    return k;
}

// calc_dpp_wave_scattering (:2918-2931) and calc_dpp_flow_shear
// (:2946-2979) as the pushes call them (:3479-3496, :4764-4788): they add to
// dp_dt and return dpp.
template <int NDIM>
__device__ __forceinline__ double dpp_terms(const MoverArgs &a, double p, const Fld &f,
                                            const Kap &k, double b, double divv,
                                            double &dp_dt) {
    double dpp = 0.0;
    if (a.dpp_wave) {
        const double va = b / sqrt(f.rho);
        if (a.momentum_dependency == 1) dp_dt = dp_dt + (8.0 * p / (27.0 * k.kpara)) * (va * va);
        else dp_dt = dp_dt + (4.0 * p / (9.0 * k.kpara)) * (va * va);
        dpp = dpp + (p * va) * (p * va) / (9.0 * k.kpara);
    }
    if (a.dpp_shear) {
        const double sxx = f.dvx_dx - divv / 3.0;
        const double syy = f.dvy_dy - divv / 3.0;
        const double szz = (NDIM == 3) ? f.dvz_dz - divv / 3.0 : -(divv / 3.0);
        // the 1D pushes pass zero off-diagonal shear (:3052-3057)
        const double sxy = (NDIM > 1) ? (f.dvx_dy + f.dvy_dx) / 2.0 : 0.0;
        const double sxz = (NDIM == 3) ? (f.dvx_dz + f.dvz_dx) / 2.0 : 0.0;
        const double syz = (NDIM == 3) ? (f.dvy_dz + f.dvz_dy) / 2.0 : 0.0;
        const double bx = f.bx, by = f.by, bz = f.bz;
        double gshear;
        if (a.weak_scattering) {
            const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
            double bbs = sxx * (bx * bx) + syy * (by * by) + szz * (bz * bz) +
                         2.0 * (sxy * bx * by + sxz * bx * bz + syz * by * bz);
            bbs = bbs * ib * ib;
            gshear = bbs * bbs / 5.0;
        } else {
            gshear = 2.0 * (sxx * sxx + syy * syy + szz * szz +
                            2.0 * (sxy * sxy + sxz * sxz + syz * syz)) / 15.0;
        }
        if (gshear > 0.0) {
            const double p0f = pow(a.p0, 2.0 - a.pindex);
            dp_dt = dp_dt + (2.0 + a.pindex) * gshear * a.tau0 * k.knorm_para *
                    pow(p, a.pindex - 1.0) * p0f;
            dpp = dpp + gshear * a.tau0 * k.knorm_para * pow(p, a.pindex) * p0f;
        }
    }
    return dpp;
}

// Cell sizes a push sees: mhd_config's dx, dy, dz on a uniform grid, the
// searched cell's spans on a non-uniform one (:3400-3408, :4689-4700).
struct Geo {
    double dxm, dym, dzm;
};

// Metric factors of spherical coordinates (x = r, y = theta, z = phi) set at
// the top of every spherical push (:3420-3427, :4707-4713).
struct Sph {
    double ctheta, istheta, cot_theta, ir, ir2;
};

__device__ __forceinline__ Sph spherical_terms(const State &s) {
    Sph g;
    g.ctheta = cos(s.y);
    g.istheta = 1.0 / sin(s.y);
    g.cot_theta = g.ctheta * g.istheta;
    g.ir = 1.0 / s.x;
    g.ir2 = 1.0 / (s.x * s.x);
    return g;
}

// Position noise of the 2D spherical pushes: the eigen-decomposition of the
// (r, theta) diffusion tensor (:3559-3580, :3905-3925).
__device__ __forceinline__ void spherical_noise_2d(const Kap &k, const Sph &g, double r1, double r2,
                                                   double sdt, double &nx, double &ny) {
    const double a1 = k.kxx;
    const double b1 = k.kxy * g.ir;
    const double c1 = k.kyy * g.ir2;
    const double amc = a1 - c1;
    const double atmp = sqrt(amc * amc + 4.0 * (b1 * b1));
    const double Qpp = atmp + (a1 + c1);
    double Qmp = atmp - (a1 + c1);
    const double Qpm = atmp + (a1 - c1);
    const double Qmm = atmp - (a1 - c1);
    if (Qmp > 0.0) Qmp = 0.0;
    const double qtmp1 = sqrt(-Qmp / (Qmm * Qmm + 4.0 * (b1 * b1)));
    const double qtmp2 = sqrt(Qpp / (Qpm * Qpm + 4.0 * (b1 * b1)));
    nx = (-(Qmm * qtmp1 * r1) + Qpm * qtmp2 * r2) * sdt;
    ny = (2.0 * b1 * qtmp1 * r1 + 2.0 * b1 * qtmp2 * r2) * sdt;
}

// The 3D spherical noise matrix P (upper triangular, P P^T = 2 K in the
// metric): p11 p12 p13 p22 p23 p33.  CLAMP: the focused-transport push's
// guards against small negative radicands (:5253-5278), absent from the
// Parker push (:4852-4863).
template <bool CLAMP>
__device__ __forceinline__ void spherical_noise_3d(const Kap &k, const Sph &g, double p[6]) {
    const double kxx = k.kxx, kyy = k.kyy, kzz = k.kzz, kxy = k.kxy, kxz = k.kxz, kyz = k.kyz;
    const double num = kxx * (kyz * kyz) + kyy * (kxz * kxz) + kzz * (kxy * kxy) -
                       2.0 * kxy * kxz * kyz - kxx * kyy * kzz;
    const double den = kyz * kyz - kyy * kzz;
    double q = 2.0 * num / den;
    if (CLAMP && q < 0.0) q = 0.0;
    p[0] = sqrt(q);
    q = 2.0 * (kyy - kyz * kyz / kzz);
    if (CLAMP && q < 0.0) q = 0.0;
    p[1] = (kxz * kyz - kxy * kzz) * sqrt(q) / den;
    p[3] = sqrt(q) * g.ir;
    if (CLAMP && kzz <= 0.0) {
        p[2] = 0.0; p[4] = 0.0; p[5] = 0.0;
    } else {
        p[2] = sqrt(2.0 / kzz) * kxz;
        p[4] = sqrt(2.0 / kzz) * kyz * g.ir;
        p[5] = sqrt(2.0 * kzz) * g.istheta * g.ir;
    }
}

// push_particle_2d (:3358-3606), Cartesian or spherical (SPH).
template <bool SPH>
__device__ __forceinline__ void push2d(const MoverArgs &a, State &s, const Fld &f, const Kap &k,
                                       const Geo &geo, bool fixed_dt, Delta &d) {
    const double bx = f.bx, by = f.by, bz = f.bz;
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    Sph g = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (SPH) g = spherical_terms(s);
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor(a, s.p, 3);
    double vdx, vdy, gbr = 0.0, gbt = 0.0;
    if (SPH) {
        gbr = f.db_dx;
        gbt = f.db_dy * g.ir;
        vdx = vdp * ((f.dbz_dy + g.cot_theta * bz) * g.ir * ib2 - gbt * bz * 2.0 * ib3);
        vdy = vdp * (-((f.dbz_dx + bz * g.ir) * ib2) + gbr * bz * 2.0 * ib3);
    } else {
        vdx = vdp * (f.dbz_dy * ib2 - 2.0 * bz * f.db_dy * ib3);
        vdy = vdp * (-(f.dbz_dx * ib2) + 2.0 * bz * f.db_dx * ib3);
    }
    double vdz = 0.0;
    if (a.check_drift_2d) {
        if (SPH)
            vdz = vdp * ((f.dby_dx + by * g.ir - f.dbx_dy * g.ir) * ib2 -
                         (gbr * by - gbt * bx * g.ir) * 2.0 * ib3);
        else
            vdz = vdp * ((f.dby_dx - f.dbx_dy) * ib2 - 2.0 * (by * f.db_dx - bx * f.db_dy) * ib3);
    }
    double dx_dt, dy_dt, dz_dt, divv;
    if (SPH) {
        dx_dt = f.vx + vdx + k.dkxx_dx + (2.0 * k.kxx + k.dkxy_dy + k.kxy * g.cot_theta) * g.ir;
        dy_dt = (f.vy + vdy + k.dkxy_dx) * g.ir + (k.kxy + k.dkyy_dy + k.kyy * g.cot_theta) * g.ir2;
        dz_dt = vdz * g.istheta * g.ir;
        divv = f.dvx_dx + (2.0 * f.vx + f.dvy_dy + f.vy * g.ctheta * g.istheta) * g.ir;
    } else {
        dx_dt = f.vx + vdx + k.dkxx_dx + k.dkxy_dy;
        dy_dt = f.vy + vdy + k.dkxy_dx + k.dkyy_dy;
        dz_dt = vdz;
        divv = f.dvx_dx + f.dvy_dy;
    }
    double dp_dt = -(s.p * divv / 3.0);
    const double dpp = dpp_terms<2>(a, s.p, f, k, b, divv, dp_dt);
    const double skpara = k.skpara, skperp = k.skperp;
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double q = 0.5 * geo.dxm / skpara, m = q * q;
            if (SPH) {
                q = 0.5 * geo.dym * s.x / skpara; if (q * q < m) m = q * q;
                q = sk / dx_dt; if (q * q < m) m = q * q;
                q = sk * g.ir / dy_dt; if (q * q < m) m = q * q;
            } else {
                q = 0.5 * geo.dym / skpara; if (q * q < m) m = q * q;
                q = sk / dx_dt; if (q * q < m) m = q * q;
                q = sk / dy_dt; if (q * q < m) m = q * q;
            }
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
    double dX, dY;
    if (SPH) {
        double nx, ny;
        spherical_noise_2d(k, g, r[0], r[1], sdt, nx, ny);
        dX = dx_dt * s.dt + nx;
        dY = dy_dt * s.dt + ny;
    } else {
        const double skpp = k.skpp;
        dX = dx_dt * s.dt + r[0] * skperp * sdt + r[2] * skpp * sdt * bx * ib;
        dY = dy_dt * s.dt + r[1] * skperp * sdt + r[2] * skpp * sdt * by * ib;
    }
    const double dZ = dz_dt * s.dt;
    s.x = s.x + dX;
    s.y = s.y + dY;
    s.z = s.z + dZ;
    s.t = s.t + s.dt;
    // deltaz is local to push_particle_2d: the mover's copy stays 0.
    d.x = dX; d.y = dY; d.z = 0.0; d.v = 0.0; d.mu = 0.0;
    push_momentum(a, s, dp_dt, dpp, sdt, r[3], 2, d.p);
}

// push_particle_3d (:4625-4907), Cartesian or spherical (SPH); I3:
// push_particle_2d_include_3rd (:3979-4266), the same with 2D field data
// (z derivatives zero), the 2D time-step limits and the 2D acceleration
// region.
template <bool SPH, bool I3 = false>
__device__ __forceinline__ void push3d(const MoverArgs &a, State &s, const Fld &f, const Kap &k,
                                       const Geo &geo, bool fixed_dt, Delta &d) {
    const double bx = f.bx, by = f.by, bz = f.bz;
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    const double bxn = bx * ib, byn = by * ib, bzn = bz * ib;
    const double bxyn = sqrt(bxn * bxn + byn * byn);
    const double ibxyn = (bxyn < DBL_EPSILON) ? 0.0 : 1.0 / bxyn;
    Sph g = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (SPH) g = spherical_terms(s);
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor(a, s.p, 3);
    double vdx, vdy, vdz;
    if (SPH) {
        const double gbr = f.db_dx, gbt = f.db_dy * g.ir, gbp = f.db_dz * g.ir * g.istheta;
        vdx = vdp * ((f.dbz_dy + bz * g.ctheta * g.istheta - f.dby_dz * g.istheta) * g.ir * ib2 -
                     (gbt * bz - gbp * by) * 2.0 * ib3);
        vdy = vdp * ((f.dbx_dz * g.istheta * g.ir - f.dbz_dx - bz * g.ir) * ib2 -
                     (gbp * bx - gbr * bz) * 2.0 * ib3);
        vdz = vdp * ((f.dby_dx + by * g.ir - f.dbx_dy * g.ir) * ib2 -
                     (gbr * by - gbt * bx) * 2.0 * ib3);
    } else {
        vdx = vdp * ((f.dbz_dy - f.dby_dz) * ib2 - 2.0 * (bz * f.db_dy - by * f.db_dz) * ib3);
        vdy = vdp * ((f.dbx_dz - f.dbz_dx) * ib2 - 2.0 * (bx * f.db_dz - bz * f.db_dx) * ib3);
        vdz = vdp * ((f.dby_dx - f.dbx_dy) * ib2 - 2.0 * (by * f.db_dx - bx * f.db_dy) * ib3);
    }
    double dx_dt, dy_dt, dz_dt, divv;
    if (SPH) {
        dx_dt = f.vx + vdx + k.dkxx_dx +
                (2.0 * k.kxx + k.dkxy_dy + k.kxy * g.ctheta * g.istheta + k.dkxz_dz * g.istheta) * g.ir;
        dy_dt = (f.vy + vdy + k.dkxy_dx) * g.ir +
                (k.kxy + k.dkyy_dy + k.kyy * g.ctheta * g.istheta + k.dkyz_dz * g.istheta) * g.ir2;
        dz_dt = (f.vz + vdz + k.dkxz_dx) * g.istheta * g.ir +
                (k.kxz + k.dkyz_dy + k.dkzz_dz * g.istheta) * g.istheta * g.ir2;
        divv = f.dvx_dx +
               (2.0 * f.vx + f.dvy_dy + f.vy * g.ctheta * g.istheta + f.dvz_dz * g.istheta) * g.ir;
    } else {
        dx_dt = f.vx + vdx + k.dkxx_dx + k.dkxy_dy + k.dkxz_dz;
        dy_dt = f.vy + vdy + k.dkxy_dx + k.dkyy_dy + k.dkyz_dz;
        dz_dt = f.vz + vdz + k.dkxz_dx + k.dkyz_dy + k.dkzz_dz;
        divv = f.dvx_dx + f.dvy_dy + f.dvz_dz;
    }
    double dp_dt = -(s.p * divv / 3.0);
    const double dpp = dpp_terms<3>(a, s.p, f, k, b, divv, dp_dt);
    const double skpara = k.skpara, skperp = k.skperp;
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double q = 0.5 * geo.dxm / skpara, m = q * q;
            if (SPH) {
                q = 0.5 * geo.dym * s.x / skpara; if (q * q < m) m = q * q;
                if (!I3) { q = 0.5 * geo.dzm * s.x * sin(s.y) / skpara; if (q * q < m) m = q * q; }
                q = sk / dx_dt; if (q * q < m) m = q * q;
                q = sk * g.ir / dy_dt; if (q * q < m) m = q * q;
                if (!I3) { q = sk * g.ir * g.istheta / dz_dt; if (q * q < m) m = q * q; }
            } else {
                q = 0.5 * geo.dym / skpara; if (q * q < m) m = q * q;
                if (!I3) { q = 0.5 * geo.dzm / skpara; if (q * q < m) m = q * q; }
                q = sk / dx_dt; if (q * q < m) m = q * q;
                q = sk / dy_dt; if (q * q < m) m = q * q;
                if (!I3) { q = sk / dz_dt; if (q * q < m) m = q * q; }
            }
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
    double dX, dY, dZ;
    if (SPH) {
        double P[6];
        spherical_noise_3d<false>(k, g, P);
        dX = dx_dt * s.dt + (P[0] * r[0] + P[1] * r[1] + P[2] * r[2]) * sdt;
        dY = dy_dt * s.dt + (P[3] * r[1] + P[4] * r[2]) * sdt;
        dZ = dz_dt * s.dt + P[5] * r[2] * sdt;
    } else {
        dX = dx_dt * s.dt +
            (bxn * skpara * r[0] - bxn * bzn * skperp * ibxyn * r[1] - byn * skperp * ibxyn * r[2]) * sdt;
        dY = dy_dt * s.dt +
            (byn * skpara * r[0] - byn * bzn * skperp * ibxyn * r[1] + bxn * skperp * ibxyn * r[2]) * sdt;
        dZ = dz_dt * s.dt + (bzn * skpara * r[0] + bxyn * skperp * r[1]) * sdt;
    }
    s.x = s.x + dX;
    s.y = s.y + dY;
    s.z = s.z + dZ;
    s.t = s.t + s.dt;
    d.x = dX; d.y = dY; d.z = dZ; d.v = 0.0; d.mu = 0.0;
    push_momentum(a, s, dp_dt, dpp, sdt, r[3], I3 ? 2 : 3, d.p);
}

// calc_duu (:3116-3155) without delta-B or correlation length.
__device__ __forceinline__ void calc_duu(const MoverArgs &a, const State &s, double b,
                                         const double *aux, double div_bnorm, double divv,
                                         double bb_gradv, double bv_gradv, double mu2,
                                         double &dmu_dt, double &duu) {
    double dm = s.v * div_bnorm + s.mu * divv - 3.0 * s.mu * bb_gradv - 2.0 * bv_gradv / s.v;
    dm = dm * (1.0 - mu2) * 0.5;
    const double h0 = (double)0.2f;
    const double dtmp = pow(fabs(s.mu), a.gamma_turb - 1.0) + h0;
    double u = a.duu0 * (1.0 - mu2) * dtmp;
    double ud;
    if (s.mu > 0.0)
        ud = a.duu0 * (-(2.0 * s.mu * dtmp) + (1.0 - mu2) * pow(fabs(s.mu), a.gamma_turb - 2.0));
    else if (s.mu < 0.0)
        ud = a.duu0 * (-(2.0 * s.mu * dtmp) - (1.0 - mu2) * pow(fabs(s.mu), a.gamma_turb - 2.0));
    else
        ud = 0.0;
    double norm = 1.0;
    if (a.mag_dependency == 1) norm = norm * pow(b, 2.0 - a.gamma_turb);
    if (a.deltab_flag && aux) norm = norm * aux[0];
    if (a.correlation_flag && aux) norm = norm * pow(aux[8], 1.0 - a.gamma_turb);
    if (a.momentum_dependency == 1) norm = norm * pow(s.p / a.p0, a.gamma_turb - 1.0);
    ud = ud * norm;
    u = u * norm;
    dmu_dt = dm + ud;
    duu = u;
}

// Adaptive step of the focused-transport pushes (:3850-3905, :5170-5230);
// in spherical coordinates the theta and phi limits carry r and r sin(theta).
template <int NDIM, bool SPH>
__device__ __forceinline__ void ft_time_step(const MoverArgs &a, State &s, const Kap &k,
                                             const Geo &geo, const Sph &g, double dx_dt,
                                             double dy_dt, double dz_dt, double dp_dt,
                                             double dmu_dt, double duu) {
    const bool nonzero = dx_dt != 0.0 && dy_dt != 0.0 && (NDIM < 3 || dz_dt != 0.0) &&
                         dp_dt != 0.0 && dmu_dt != 0.0;
    if (nonzero) {
        const double sk = (k.skperp > 0.0) ? k.skperp : k.skpara;
        double q = 0.5 * geo.dxm / sk, m = q * q;
        if (SPH) {
            q = 0.5 * geo.dym * s.x / sk; if (q * q < m) m = q * q;
            if (NDIM == 3) { q = 0.5 * geo.dzm * s.x * sin(s.y) / sk; if (q * q < m) m = q * q; }
            q = sk / dx_dt; if (q * q < m) m = q * q;
            q = sk * g.ir / dy_dt; if (q * q < m) m = q * q;
            if (NDIM == 3) { q = sk * g.ir * g.istheta / dz_dt; if (q * q < m) m = q * q; }
        } else {
            q = 0.5 * geo.dym / sk; if (q * q < m) m = q * q;
            if (NDIM == 3) { q = 0.5 * geo.dzm / sk; if (q * q < m) m = q * q; }
            q = sk / dx_dt; if (q * q < m) m = q * q;
            q = sk / dy_dt; if (q * q < m) m = q * q;
            if (NDIM == 3) { q = sk / dz_dt; if (q * q < m) m = q * q; }
        }
        q = (double)0.1f * s.p / fabs(dp_dt); if (q < m) m = q;
        q = (double)0.1f / fabs(dmu_dt); if (q < m) m = q;
        q = 2.0 * duu / (dmu_dt * dmu_dt); if (q < m) m = q;
        s.dt = m;
    } else {
        s.dt = a.dt_min;
    }
    if (s.dt < a.dt_min) s.dt = a.dt_min;
    if (s.dt > a.dt_max) s.dt = a.dt_max;
}

// Shared tail of push_particle_2d_ft / push_particle_3d_ft (:3920-3963,
// :5280-5323); r[2] drives momentum diffusion, r[3] pitch-angle scattering.
template <int NDIM, int ACC_NDIM = NDIM>
__device__ __forceinline__ void push_ft_tail(const MoverArgs &a, State &s, double dX, double dY,
                                             double dZ, double dp_dt, double dpp, double dmu_dt,
                                             double duu, double sdt, const double r[4], Delta &d) {
    double dP = dp_dt * s.dt + r[2] * sqrt(2.0 * dpp) * sdt;
    double dV = s.v * dP / s.p;
    double dMu = dmu_dt * s.dt + r[3] * sqrt(2.0 * duu) * sdt;
    s.x = s.x + dX;
    s.y = s.y + dY;
    s.z = s.z + dZ;
    s.mu = s.mu + dMu;
    s.t = s.t + s.dt;
    const double mu_max = (double)0.99f;
    if (s.mu > mu_max) {
        dMu = mu_max - (s.mu - dMu);
        s.mu = mu_max;
    } else if (s.mu < -mu_max) {
        dMu = -mu_max - (s.mu - dMu);
        s.mu = -mu_max;
    }
    if (a.acc_region_flag == 1) {
        if (in_acc_region(a, s, ACC_NDIM)) {
            s.p = s.p + dP;
            s.v = s.v + dV;
        } else {
            dP = 0.0;
            dV = 0.0;
        }
    } else {
        s.p = s.p + dP;
        s.v = s.v + dV;
    }
    const double pfloor = 0.25 * a.p0;
    if (s.p < pfloor) {
        s.v = s.v - dV;
        dV = s.v * 0.25 * a.p0 / s.p - s.v;
        s.v = s.v + dV;
        s.p = s.p - dP;
        dP = pfloor - s.p;
        s.p = pfloor;
    }
    // deltaz is local to push_particle_2d_ft: the mover's copy stays 0.
    d.x = dX; d.y = dY; d.z = (NDIM == 3) ? dZ : 0.0; d.p = dP; d.v = dV; d.mu = dMu;
}

// push_particle_2d_ft (:3626-3964) and push_particle_3d_ft (:4930-5324),
// Cartesian or spherical (SPH).  The 3D spherical position noise draws a
// third number (ran3), taken from the push's third Philox block.  I3 (with
// NDIM = 3): push_particle_2d_include_3rd_ft (:4267-4610), the 3D push on 2D
// field data with the 2D time-step limits, cot(theta) in the spherical r and
// theta rates and no radicand guards in the spherical noise.
template <int NDIM, bool SPH, bool I3 = false>
__device__ __forceinline__ void push_ft(const MoverArgs &a, State &s, const Fld &f,
                                        const double *aux, const Kap &k, const Geo &geo,
                                        bool fixed_dt, Delta &d) {
    const double bx = f.bx, by = f.by, bz = f.bz;
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    Sph g = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (SPH) g = spherical_terms(s);
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor(a, s.p, 1);
    const double mu2 = s.mu * s.mu;
    const double muf1 = 0.5 * (1.0 - mu2);
    const double muf2 = 0.5 * (3.0 * mu2 - 1.0);
    double kx, ky, kz, bdot_curvb, vdx, vdy, vdz = 0.0;
    if (NDIM == 2) {
        double gbr = 0.0, gbt = 0.0;
        if (SPH) {
            const double ir = g.ir, cot = g.cot_theta;
            gbr = f.db_dx;
            gbt = f.db_dy * ir;
            kx = bx * f.dbx_dx + by * f.dbx_dy * ir - (by * by + bz * bz) * ir;
            ky = bx * f.dby_dx + by * f.dby_dy * ir + (bx * by - cot * (bz * bz)) * ir;
            kz = bx * f.dbz_dx + by * f.dbz_dy * ir + (bx * bz + cot * by * bz) * ir;
            bdot_curvb = bx * (f.dbz_dy + cot * bz) * ir + by * (-f.dbz_dx - bz * ir) +
                         bz * (f.dby_dx + by * ir - f.dbx_dy * ir);
            vdx = vdp * (muf1 * (-(bz * gbt)) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                         muf1 * bx * bdot_curvb * ib3);
            vdy = vdp * (muf1 * (bz * gbr) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                         muf1 * by * bdot_curvb * ib3);
        } else {
            kx = bx * f.dbx_dx + by * f.dbx_dy;
            ky = bx * f.dby_dx + by * f.dby_dy;
            kz = bx * f.dbz_dx + by * f.dbz_dy;
            bdot_curvb = bx * f.dbz_dy - by * f.dbz_dx + bz * (f.dby_dx - f.dbx_dy);
            vdx = vdp * (muf1 * (-(bz * f.db_dy)) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                         muf1 * bx * bdot_curvb * ib3);
            vdy = vdp * (muf1 * (bz * f.db_dx) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                         muf1 * by * bdot_curvb * ib3);
        }
        if (a.check_drift_2d) {
            if (SPH)
                vdz = vdp * (muf1 * (bx * gbt - by * gbr) * ib2 + mu2 * (bx * ky - by * kx) * ib3 +
                             muf1 * bz * bdot_curvb * ib3);
            else
                vdz = vdp * (muf1 * (bx * f.db_dy - by * f.db_dx) * ib2 +
                             mu2 * (bx * ky - by * kx) * ib3 + muf1 * bz * bdot_curvb * ib3);
        }
    } else {
        if (SPH) {
            const double ir = g.ir, ist = g.istheta, cot = g.cot_theta;
            const double gbr = f.db_dx, gbt = f.db_dy * ir, gbp = f.db_dz * ir * ist;
            kx = bx * f.dbx_dx + ir * (by * f.dbx_dy + bz * f.dbx_dz * ist - (by * by + bz * bz));
            ky = bx * f.dby_dx + ir * (by * f.dby_dy + bz * f.dby_dz * ist + (bx * by - cot * (bz * bz)));
            kz = bx * f.dbz_dx + ir * (by * f.dbz_dy + bz * f.dbz_dz * ist + (bx * bz + cot * by * bz));
            bdot_curvb = bx * (f.dbz_dy + cot * bz - f.dby_dz * ist) * ir +
                         by * (f.dbx_dz * ist * ir - f.dbz_dx - bz * ir) +
                         bz * (f.dby_dx + by * ir - f.dbx_dy * ir);
            vdx = vdp * (muf1 * (by * gbp - bz * gbt) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                         muf1 * bx * bdot_curvb * ib3);
            vdy = vdp * (muf1 * (bz * gbr - bx * gbp) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                         muf1 * by * bdot_curvb * ib3);
            vdz = vdp * (muf1 * (bx * gbt - by * gbr) * ib2 + mu2 * (bx * ky - by * kx) * ib3 +
                         muf1 * bz * bdot_curvb * ib3);
        } else {
            kx = bx * f.dbx_dx + by * f.dbx_dy + bz * f.dbx_dz;
            ky = bx * f.dby_dx + by * f.dby_dy + bz * f.dby_dz;
            kz = bx * f.dbz_dx + by * f.dbz_dy + bz * f.dbz_dz;
            bdot_curvb = bx * (f.dbz_dy - f.dby_dz) + by * (f.dbx_dz - f.dbz_dx) + bz * (f.dby_dx - f.dbx_dy);
            vdx = vdp * (muf1 * (by * f.db_dz - bz * f.db_dy) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                         muf1 * bx * bdot_curvb * ib3);
            vdy = vdp * (muf1 * (bz * f.db_dx - bx * f.db_dz) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                         muf1 * by * bdot_curvb * ib3);
            vdz = vdp * (muf1 * (bx * f.db_dy - by * f.db_dx) * ib2 + mu2 * (bx * ky - by * kx) * ib3 +
                         muf1 * bz * bdot_curvb * ib3);
        }
    }
    double vbx = s.v * s.mu * ib;
    const double vby = vbx * by;
    const double vbz = vbx * bz;
    vbx = vbx * bx;
    double dx_dt, dy_dt, dz_dt, divv, bb_gradv, bv_gradv, div_bnorm;
    if (NDIM == 2) {
        if (SPH) {
            const double ir = g.ir, cot = g.cot_theta;
            const double vx = f.vx, vy = f.vy, vz = f.vz;
            dx_dt = vx + vdx + vbx + k.dkxx_dx + (2.0 * k.kxx + k.dkxy_dy + k.kxy * cot) * ir;
            dy_dt = (vy + vdy + vby + k.dkxy_dx) * ir + (k.kxy + k.dkyy_dy + k.kyy * cot) * g.ir2;
            dz_dt = vdz * g.istheta * ir;
            divv = f.dvx_dx + (2.0 * vx + f.dvy_dy + vy * cot) * ir;
            bb_gradv = (bx * bx * f.dvx_dx + bx * by * f.dvx_dy * ir - bx * (by * vy + bz * vz) * ir +
                        by * bx * f.dvy_dx + by * by * f.dvy_dy * ir + by * (by * vx - cot * bz * vz) * ir +
                        bz * bx * f.dvz_dx + bz * by * f.dvz_dy * ir + (bz * bz) * (vx + cot * vy) * ir) * ib2;
            bv_gradv = (bx * vx * f.dvx_dx + bx * vy * f.dvx_dy * ir - bx * (vy * vy + vz * vz) * ir +
                        by * vx * f.dvy_dx + by * vy * f.dvy_dy * ir + by * (vy * vx - cot * vz * vz) * ir +
                        bz * vx * f.dvz_dx + bz * vy * f.dvz_dy * ir + bz * vz * (vx + cot * vy) * ir) * ib;
            div_bnorm = -((bx * f.db_dx + by * f.db_dy * ir) * ib2);
        } else {
            dx_dt = f.vx + vdx + vbx + k.dkxx_dx + k.dkxy_dy;
            dy_dt = f.vy + vdy + vby + k.dkxy_dx + k.dkyy_dy;
            dz_dt = vdz;
            divv = f.dvx_dx + f.dvy_dy;
            bb_gradv = (bx * (bx * f.dvx_dx + by * f.dvx_dy) + by * (bx * f.dvy_dx + by * f.dvy_dy) +
                        bz * (bx * f.dvz_dx + by * f.dvz_dy)) * ib2;
            bv_gradv = (bx * (f.vx * f.dvx_dx + f.vy * f.dvx_dy) + by * (f.vx * f.dvy_dx + f.vy * f.dvy_dy) +
                        bz * (f.vx * f.dvz_dx + f.vy * f.dvz_dy)) * ib;
            div_bnorm = -((bx * f.db_dx + by * f.db_dy) * ib2);
        }
    } else {
        if (SPH) {
            const double ir = g.ir, ist = g.istheta, cot = g.cot_theta;
            const double vx = f.vx, vy = f.vy, vz = f.vz;
            if (I3) {
                dx_dt = vx + vbx + vdx + k.dkxx_dx + (2.0 * k.kxx + k.dkxy_dy + k.kxy * cot) * ir;
                dy_dt = (vy + vby + vdy + k.dkxy_dx) * ir + (k.kxy + k.dkyy_dy + k.kyy * cot) * g.ir2;
            } else {
                dx_dt = vx + vbx + vdx + k.dkxx_dx +
                        (2.0 * k.kxx + k.dkxy_dy + k.kxy * g.ctheta * ist + k.dkxz_dz * ist) * ir;
                dy_dt = (vy + vby + vdy + k.dkxy_dx) * ir +
                        (k.kxy + k.dkyy_dy + k.kyy * g.ctheta * ist + k.dkyz_dz * ist) * g.ir2;
            }
            dz_dt = (vz + vbz + vdz + k.dkxz_dx) * ist * ir +
                    (k.kxz + k.dkyz_dy + k.dkzz_dz * ist) * ist * g.ir2;
            divv = f.dvx_dx + (2.0 * vx + f.dvy_dy + vy * cot + f.dvz_dz * ist) * ir;
            const double dtmp = ist * ir;
            bb_gradv = (bx * bx * f.dvx_dx + bx * by * f.dvx_dy * ir + bx * bz * f.dvx_dz * dtmp -
                        bx * (by * vy + bz * vz) * ir +
                        by * bx * f.dvy_dx + by * by * f.dvy_dy * ir + by * bz * f.dvy_dz * dtmp +
                        by * (by * vx - cot * bz * vz) * ir +
                        bz * bx * f.dvz_dx + bz * by * f.dvz_dy * ir + bz * bz * f.dvz_dz * dtmp +
                        (bz * bz) * (vx + cot * vy) * ir) * ib2;
            bv_gradv = (bx * vx * f.dvx_dx + bx * vy * f.dvx_dy * ir + bx * vz * f.dvx_dz * dtmp -
                        bx * (vy * vy + vz * vz) * ir +
                        by * vx * f.dvy_dx + by * vy * f.dvy_dy * ir + by * vz * f.dvy_dz * dtmp +
                        by * (vy * vx - cot * vz * vz) * ir +
                        bz * vx * f.dvz_dx + bz * vy * f.dvz_dy * ir + bz * vz * f.dvz_dz * dtmp +
                        bz * vz * (vx + cot * vy) * ir) * ib;
            div_bnorm = -((bx * f.db_dx + by * f.db_dy * ir + bz * f.db_dz * ir * ist) * ib2);
        } else {
            dx_dt = f.vx + vbx + vdx + k.dkxx_dx + k.dkxy_dy + k.dkxz_dz;
            dy_dt = f.vy + vby + vdy + k.dkxy_dx + k.dkyy_dy + k.dkyz_dz;
            dz_dt = f.vz + vbz + vdz + k.dkxz_dx + k.dkyz_dy + k.dkzz_dz;
            divv = f.dvx_dx + f.dvy_dy + f.dvz_dz;
            bb_gradv = (bx * (bx * f.dvx_dx + by * f.dvx_dy + bz * f.dvx_dz) +
                        by * (bx * f.dvy_dx + by * f.dvy_dy + bz * f.dvy_dz) +
                        bz * (bx * f.dvz_dx + by * f.dvz_dy + bz * f.dvz_dz)) * ib2;
            bv_gradv = (bx * (f.vx * f.dvx_dx + f.vy * f.dvx_dy + f.vz * f.dvx_dz) +
                        by * (f.vx * f.dvy_dx + f.vy * f.dvy_dy + f.vz * f.dvy_dz) +
                        bz * (f.vx * f.dvz_dx + f.vy * f.dvz_dy + f.vz * f.dvz_dz)) * ib;
            div_bnorm = -((bx * f.db_dx + by * f.db_dy + bz * f.db_dz) * ib2);
        }
    }
    const double acc_rate = -(muf1 * divv + muf2 * bb_gradv + s.mu * bv_gradv / s.v);
    double dp_dt = s.p * acc_rate;
    const double dpp = dpp_terms<NDIM>(a, s.p, f, k, b, divv, dp_dt);
    double dmu_dt, duu;
    calc_duu(a, s, b, aux, div_bnorm, divv, bb_gradv, bv_gradv, mu2, dmu_dt, duu);
    if (!fixed_dt)
        ft_time_step<I3 ? 2 : NDIM, SPH>(a, s, k, geo, g, dx_dt, dy_dt, dz_dt, dp_dt, dmu_dt, duu);
    const double sdt = sqrt(s.dt);
    double r[6];
    if (SPH && NDIM == 3) noise6(a, s, r);
    else noise4(a, s, r);
    const double bxn = bx * ib, byn = by * ib, bzn = bz * ib;
    const double skperp = k.skperp;
    double dX, dY, dZ;
    if (NDIM == 2) {
        if (SPH) {
            double nx, ny;
            spherical_noise_2d(k, g, r[0], r[1], sdt, nx, ny);
            dX = dx_dt * s.dt + nx;
            dY = dy_dt * s.dt + ny;
        } else {
            // by and bx (not byn, bxn) in the second terms, as the reference.
            const double ibxyn = 1.0 / sqrt(bxn * bxn + byn * byn);
            dX = dx_dt * s.dt + skperp * ibxyn * sdt * (-(bxn * bzn * r[0]) - by * r[1]);
            dY = dy_dt * s.dt + skperp * ibxyn * sdt * (-(byn * bzn * r[0]) + bx * r[1]);
        }
        dZ = dz_dt * s.dt;
    } else if (SPH) {
        double P[6];
        spherical_noise_3d<!I3>(k, g, P);
        dX = dx_dt * s.dt + (P[0] * r[0] + P[1] * r[1] + P[2] * r[4]) * sdt;
        dY = dy_dt * s.dt + (P[3] * r[1] + P[4] * r[4]) * sdt;
        dZ = dz_dt * s.dt + P[5] * r[4] * sdt;
    } else {
        const double bxyn = sqrt(bxn * bxn + byn * byn);
        const double ibxyn = (bxyn < DBL_EPSILON) ? 0.0 : 1.0 / bxyn;
        dX = dx_dt * s.dt + (-(bxn * bzn * skperp * ibxyn * r[0]) - byn * skperp * ibxyn * r[1]) * sdt;
        dY = dy_dt * s.dt + (-(byn * bzn * skperp * ibxyn * r[0]) + bxn * skperp * ibxyn * r[1]) * sdt;
        dZ = dz_dt * s.dt + bxyn * skperp * r[0] * sdt;
    }
    push_ft_tail<NDIM, I3 ? 2 : NDIM>(a, s, dX, dY, dZ, dp_dt, dpp, dmu_dt, duu, sdt, r, d);
}

// After the reference's one-period wrap: a push longer than a period (a
// drift at dt_min where kappa's gradient is steep) leaves the particle
// outside even so, where the reference would index outside its arrays.
// Whole periods more bring it back; inside the box this is the identity, so
// every case the reference defines is unchanged.
__device__ __forceinline__ double wrap_rest(double x, double lo, double hi) {
    const double per = hi - lo;
    if (x < lo) x += per * ceil((lo - x) / per);
    else if (x > hi) x -= per * ceil((x - hi) / per);
    return x;
}

template <int NDIM>
__device__ __forceinline__ void boundary(const MoverArgs &a, State &s, double xlo, double xhi,
                                         double ylo, double yhi, double zlo, double zhi, Acc &acc) {
    if (s.x < xlo && s.flag == 1) {
        if (a.pbcx) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -1; }
        else s.x = wrap_rest(s.x - xlo + xhi, xlo, xhi);
    } else if (s.x > xhi && s.flag == 1) {
        if (a.pbcx) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -2; }
        else s.x = wrap_rest(s.x - xhi + xlo, xlo, xhi);
    }
    if (NDIM > 1) {
        if (s.y < ylo && s.flag == 1) {
            if (a.pbcy) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -3; }
            else s.y = wrap_rest(s.y - ylo + yhi, ylo, yhi);
        } else if (s.y > yhi && s.flag == 1) {
            if (a.pbcy) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -4; }
            else s.y = wrap_rest(s.y - yhi + ylo, ylo, yhi);
        }
    }
    if (NDIM == 3 || a.include_3rd) {   // z too for include_3rd_dim runs (:2084)
        if (s.z < zlo && s.flag == 1) {
            if (a.pbcz) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -5; }
            else s.z = wrap_rest(s.z - zlo + zhi, zlo, zhi);
        } else if (s.z > zhi && s.flag == 1) {
            if (a.pbcz) { acc_add(acc.leak_h, acc.leak_l, s.w); s.flag = -6; }
            else s.z = wrap_rest(s.z - zhi + zlo, zlo, zhi);
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

// push_particle_1d (:2993-3110), Cartesian or spherical (x = r); r[0]
// drives x, r[3] momentum.
template <bool SPH>
__device__ __forceinline__ void push1d(const MoverArgs &a, State &s, const Fld &f, const Kap &k,
                                       const Geo &geo, bool fixed_dt, Delta &d) {
    const double bx = f.bx, by = f.by, bz = f.bz;
    const double b = sqrt(bx * bx + by * by + bz * bz);
    double dx_dt, divv;
    if (SPH) {
        dx_dt = f.vx + k.dkxx_dx + 2.0 * k.kxx / s.x;
        divv = f.dvx_dx + 2.0 * f.vx / s.x;
    } else {
        dx_dt = f.vx + k.dkxx_dx;
        divv = f.dvx_dx;
    }
    double dp_dt = -(s.p * divv / 3.0);
    const double dpp = dpp_terms<1>(a, s.p, f, k, b, divv, dp_dt);
    const double skpara = k.skpara, skperp = k.skperp;
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double q = 0.5 * geo.dxm / skpara, m = q * q;
            q = sk / dx_dt; if (q * q < m) m = q * q;
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
    const double dX = dx_dt * s.dt + r[0] * skpara * sdt;
    s.x = s.x + dX;
    s.t = s.t + s.dt;
    d.x = dX; d.y = 0.0; d.z = 0.0; d.v = 0.0; d.mu = 0.0;
    push_momentum(a, s, dp_dt, dpp, sdt, r[3], 1, d.p);
}

// push_particle_1d_ft (:3174-3357).  The reference computes the x rate into
// dv_dt and then reads dx_dt, which it never sets; the computed rate is
// used.  r[0] drives x, r[2] momentum, r[3] pitch angle.
template <bool SPH>
__device__ __forceinline__ void push_ft1d(const MoverArgs &a, State &s, const Fld &f,
                                          const double *aux, const Kap &k, const Geo &geo,
                                          bool fixed_dt, Delta &d) {
    const double vx = f.vx, vy = f.vy, vz = f.vz, bx = f.bx, by = f.by, bz = f.bz;
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double dvx_dx = f.dvx_dx, dvy_dx = f.dvy_dx, dvz_dx = f.dvz_dx;
    double dx_dt, divv, bb_gradv, bv_gradv;
    if (SPH) {
        const double ir = 1.0 / s.x;
        dx_dt = vx + s.v * s.mu + k.dkxx_dx + 2.0 * k.kxx * ir;
        const double cot = 1.0 / tan(s.y);
        divv = dvx_dx + 2.0 * vx * ir;
        bb_gradv = (bx * bx * dvx_dx - bx * (by * vy + bz * vz) * ir + by * bx * dvy_dx +
                    by * (by * vx - cot * bz * vz) * ir + bz * bx * dvz_dx +
                    (bz * bz) * (vx + cot * vy) * ir) / (b * b);
        bv_gradv = (bx * vx * dvx_dx - bx * (vy * vy + vz * vz) * ir + by * vx * dvy_dx +
                    by * (vy * vx - cot * vz * vz) * ir + bz * vx * dvz_dx +
                    bz * vz * (vx + cot * vy) * ir) / (b * b);
    } else {
        dx_dt = vx + s.v * s.mu + k.dkxx_dx;
        divv = dvx_dx;
        bb_gradv = (bx * bx * dvx_dx + by * bx * dvy_dx + bz * bx * dvz_dx) / (b * b);
        bv_gradv = (bx * vx * dvx_dx + by * vx * dvy_dx + bz * vx * dvz_dx) / b;
    }
    const double mu2 = s.mu * s.mu;
    const double acc_rate = -(0.5 * (1.0 - mu2) * divv + 0.5 * (3.0 * mu2 - 1.0) * bb_gradv +
                              s.mu * bv_gradv / s.v);
    double dp_dt = s.p * acc_rate;
    const double dpp = dpp_terms<1>(a, s.p, f, k, b, divv, dp_dt);
    const double div_bnorm = -(bx * f.db_dx / (b * b));
    double dmu_dt, duu;
    calc_duu(a, s, b, aux, div_bnorm, divv, bb_gradv, bv_gradv, mu2, dmu_dt, duu);
    const double skpara = k.skpara, skperp = k.skperp;
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dp_dt != 0.0 && dmu_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double q = 0.5 * geo.dxm / sk, m = q * q;
            q = sk / dx_dt; if (q * q < m) m = q * q;
            q = (double)0.1f * s.p / fabs(dp_dt); if (q < m) m = q;
            q = (double)0.1f / fabs(dmu_dt); if (q < m) m = q;
            q = 2.0 * duu / (dmu_dt * dmu_dt); if (q < m) m = q;
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
    const double dX = dx_dt * s.dt + r[0] * skpara * sdt;
    push_ft_tail<1>(a, s, dX, 0.0, 0.0, dp_dt, dpp, dmu_dt, duu, sdt, r, d);
}

// kappa and the push for interpolated fields f: NDIM-dimensional, or the 3D
// push on 2D data for include_3rd_dim runs (I3).
template <int NDIM, bool FT, bool SPH, bool I3>
__device__ __forceinline__ void run_push(const MoverArgs &a, State &s, const Fld &f,
                                         const double *aux, const Geo &geo, bool fixed_dt,
                                         Delta &d) {
    if (I3) {
        const Kap k = kappa<3, FT, true>(a, s.p, s.mu, f, aux);
        if (FT) push_ft<3, SPH, true>(a, s, f, aux, k, geo, fixed_dt, d);
        else push3d<SPH, true>(a, s, f, k, geo, fixed_dt, d);
    } else if (NDIM == 1) {
        const Kap k = kappa<1, FT>(a, s.p, s.mu, f, aux);
        if (FT) push_ft1d<SPH>(a, s, f, aux, k, geo, fixed_dt, d);
        else push1d<SPH>(a, s, f, k, geo, fixed_dt, d);
    } else {
        const Kap k = kappa<NDIM, FT>(a, s.p, s.mu, f, aux);
        if (FT) push_ft<NDIM, SPH>(a, s, f, aux, k, geo, fixed_dt, d);
        else if (NDIM == 2) push2d<SPH>(a, s, f, k, geo, fixed_dt, d);
        else push3d<SPH>(a, s, f, k, geo, fixed_dt, d);
    }
}

template <int NDIM, bool FT, bool FULL, bool GRID, bool I3>
__device__ __forceinline__ bool do_push(const MoverArgs &a, State &s, bool fixed_dt, Delta &d) {
    Fld f;
    double av[16];
    const double *aux = nullptr;
    if (GRID) {
        // Spherical or non-uniform grid: corner and weights from the node
        // positions (:1615-1630), all 32 variables.
        GridCell c;
        if (!grid_cell(NDIM, a.spherical, a.xpos, a.nxg, a.ypos, a.nyg, a.zpos, a.nzg, s.x, s.y,
                       s.z, c)) {
            set_status(a.cnt, kStatusIndexGuard);
            return false;
        }
        double v[32];
        interp_at<NDIM, 32, 32>(a, a.full1, a.full2, s, c.ix, c.iy, c.iz, c.w, v);
        f = named_full(v);
        if (NDIM == 3 && a.surf_on) surface_heights(a, s, c.ix, c.iy, c.iz, c.w);
        if (a.aux1 && (a.deltab_flag || a.correlation_flag)) {
            interp_at<NDIM, 16, 16>(a, a.aux1, a.aux2, s, c.ix, c.iy, c.iz, c.w, av);
            aux = av;
        }
        Geo geo = {a.dx, a.dy, a.dz};
        if (a.nonuniform) {
            // the pushes' own search (no offset shift): X[k] - X[k - 1]
            geo.dxm = __ldg(a.xpos + c.kx) - __ldg(a.xpos + c.kx - 1);
            if (NDIM > 1) geo.dym = __ldg(a.ypos + c.ky) - __ldg(a.ypos + c.ky - 1);
            if (NDIM == 3) geo.dzm = __ldg(a.zpos + c.kz) - __ldg(a.zpos + c.kz - 1);
        }
        if (a.spherical) run_push<NDIM, FT, true, I3>(a, s, f, aux, geo, fixed_dt, d);
        else run_push<NDIM, FT, false, I3>(a, s, f, aux, geo, fixed_dt, d);
        if (!isfinite(s.x) || !isfinite(s.y) || !isfinite(s.z) || !isfinite(s.p) ||
            !isfinite(s.t) || (FT && (!isfinite(s.v) || !isfinite(s.mu)))) {
            set_status(a.cnt, kStatusNonFinite);
            return false;
        }
        return true;
    }
    if (FULL) {
        double v[32];
        int ix, iy, iz;
        double w[8];
        if (!uniform_cell<NDIM>(a, s, ix, iy, iz, w)) return false;
        interp_at<NDIM, 32, 32>(a, a.full1, a.full2, s, ix, iy, iz, w, v);
        f = named_full(v);
        if (NDIM == 3 && a.surf_on) surface_heights(a, s, ix, iy, iz, w);
        if (a.aux1 && (a.deltab_flag || a.correlation_flag)) {
            if (!interp<NDIM, 16, 16>(a, a.aux1, a.aux2, s, av)) return false;
            aux = av;
        }
    } else {
        constexpr int NV = (NDIM == 2) ? 15 : 21;
        constexpr int R = (NDIM == 2) ? kRec2D : kRec3D;
        double v[NV];
        if (!interp<NDIM, NV, R>(a, a.rec1, a.rec2, s, v)) return false;
        f = named_packed<NDIM>(v);
    }
    const Geo geo = {a.dx, a.dy, a.dz};
    run_push<NDIM, FT, false, I3>(a, s, f, aux, geo, fixed_dt, d);
    if (!isfinite(s.x) || !isfinite(s.y) || !isfinite(s.z) || !isfinite(s.p) || !isfinite(s.t) ||
        (FT && (!isfinite(s.v) || !isfinite(s.mu)))) {
        set_status(a.cnt, kStatusNonFinite);
        return false;
    }
    return true;
}

// Particle tracking after a push (particle_module.f90:1697-1703 and
// :1806-1812): a tracked particle (tag_splitted < 0) whose push count wraps
// to 0 appends its state to its columns of particles_tracked.  The columns
// are searched once per call (they depend on tags and split_times only).
template <bool FT>
__device__ __forceinline__ void track_push(const MoverArgs &a, const State &s, int64_t i,
                                           int32_t &ntrk, int &lo, int &hi, int &found) {
    if (!a.trk.tags || s.tag_spl >= 0 || s.nsteps_pushed != 0) return;
    if (found == 0)
        found = trk_select(a.trk, a.P.origin[i], s.tag_inj, a.P.split_times[i], s.tag_spl, lo,
                           hi) ? 1 : 2;
    ntrk += 1;
    if (found != 1) return;
    TrkRecord r;
    r.x = s.x; r.y = s.y; r.z = s.z; r.p = s.p;
    r.v = FT ? s.v : a.P.v[i];
    r.mu = s.mu; r.w = s.w; r.t = s.t; r.dt = s.dt;
    r.split_times = a.P.split_times[i]; r.count_flag = s.flag;
    r.origin = a.P.origin[i]; r.nsteps_tracked = ntrk; r.nsteps_pushed = s.nsteps_pushed;
    r.tag_inj = s.tag_inj; r.tag_spl = s.tag_spl; r.ctr = s.ctr;
    trk_write(a.trk, ntrk, lo, hi, r, a.cnt);
}

// FT: focused transport.  FULL: interpolate all 32 variables (focused
// transport and momentum diffusion read velocity gradients and density that
// the packed records leave out).  GRID: spherical coordinates or non-uniform
// node positions.  I3: a 2D run with transport along z (include_3rd_dim).
template <int NDIM, bool FT, bool FULL, bool GRID, bool I3>
__global__ void __launch_bounds__(128) mover_fp64_kernel(const MoverArgs a) {
    Acc acc = {0, 0, 0, 0, 0};
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n) {
        State s;
        s.x = a.P.x[i]; s.y = a.P.y[i]; s.z = a.P.z[i]; s.p = a.P.p[i];
        s.v = FT ? a.P.v[i] : 0.0;
        s.mu = a.P.mu[i];
        s.t = a.P.t[i]; s.dt = a.P.dt[i]; s.w = a.P.weight[i];
        s.flag = a.P.count_flag[i];
        s.nsteps_pushed = a.P.nsteps_pushed[i];
        s.tag_inj = a.P.tag_injected[i];
        s.tag_spl = a.P.tag_splitted[i];
        s.ctr = a.P.rng_ctr[i];
        const double t0 = a.t0, dt_fine = a.dt_fine;
        Delta dl = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
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
        // nsteps_tracked restarts at 1 every call (particle_mover :1910-1913)
        int32_t ntrk = 1;
        int trk_lo = 0, trk_hi = -1, trk_found = 0;
        bool alive = (s.flag == 1);
        while (alive && dt_target < a.limit) {
            if (s.flag != 1) break;
            while ((s.t - t0) < dt_target && s.flag == 1) {
                negp_or_boundary<NDIM>(a, s, acc);
                if (s.flag != 1) break;
                if (pushes >= a.max_pushes) { set_status(a.cnt, kStatusStepLimit); alive = false; break; }
                if (!do_push<NDIM, FT, FULL, GRID, I3>(a, s, false, dl)) {
                    s.flag = 0; alive = false; break;
                }
                ++pushes;
                s.nsteps_pushed = (s.nsteps_pushed + 1) % a.nsteps_interval;
                track_push<FT>(a, s, i, ntrk, trk_lo, trk_hi, trk_found);
            }
            if (!alive) break;
            if ((s.t - t0) > dt_target && s.flag == 1) {
                s.x = s.x - dl.x;
                s.y = s.y - dl.y;
                s.z = s.z - dl.z;
                s.p = s.p - dl.p;
                if (FT) {
                    s.v = s.v - dl.v;
                    s.mu = s.mu - dl.mu;
                }
                s.t = s.t - s.dt;
                const double dt_old = s.dt;
                s.dt = t0 + dt_target - s.t;
                if (s.dt > 0.0) {
                    // a tracked particle whose undone push was recorded takes
                    // the record back (:1716-1722)
                    if (s.tag_spl < 0 && s.nsteps_pushed == 0) {
                        ntrk -= 1;
                        s.nsteps_pushed = a.nsteps_interval - 2;
                    } else {
                        s.nsteps_pushed = s.nsteps_pushed - 1;
                    }
                    if (!do_push<NDIM, FT, FULL, GRID, I3>(a, s, true, dl)) {
                        s.flag = 0; alive = false; break;
                    }
                    ++pushes;
                    s.nsteps_pushed = (s.nsteps_pushed + 1) % a.nsteps_interval;
                    track_push<FT>(a, s, i, ntrk, trk_lo, trk_hi, trk_found);
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
        if (FT) { a.P.v[i] = s.v; a.P.mu[i] = s.mu; }
        a.P.t[i] = s.t; a.P.dt[i] = s.dt;
        a.P.count_flag[i] = (int8_t)s.flag;
        a.P.nsteps_pushed[i] = s.nsteps_pushed;
        a.P.nsteps_tracked[i] = ntrk;
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
    const bool ft = a.focused_transport != 0;
    const bool full = ft || a.dpp_wave || a.dpp_shear || a.deltab_flag || a.correlation_flag ||
                      a.surf_on;
    const bool grid = a.spherical || a.nonuniform;
    const unsigned g = (unsigned)blocks;
    if (a.ndim == 1) {
        // 1D runs always interpolate all 32 variables
        if (grid && ft) mover_fp64_kernel<1, true, true, true, false><<<g, threads, 0, s>>>(a);
        else if (grid) mover_fp64_kernel<1, false, true, true, false><<<g, threads, 0, s>>>(a);
        else if (ft) mover_fp64_kernel<1, true, true, false, false><<<g, threads, 0, s>>>(a);
        else mover_fp64_kernel<1, false, true, false, false><<<g, threads, 0, s>>>(a);
    } else if (a.ndim == 2 && a.include_3rd) {
        // 2D data, 3D transport: all 32 variables (the pushes read vz and
        // the in-plane gradients of bz and vz)
        if (grid && ft) mover_fp64_kernel<2, true, true, true, true><<<g, threads, 0, s>>>(a);
        else if (grid) mover_fp64_kernel<2, false, true, true, true><<<g, threads, 0, s>>>(a);
        else if (ft) mover_fp64_kernel<2, true, true, false, true><<<g, threads, 0, s>>>(a);
        else mover_fp64_kernel<2, false, true, false, true><<<g, threads, 0, s>>>(a);
    } else if (a.ndim == 2) {
        if (grid && ft) mover_fp64_kernel<2, true, true, true, false><<<g, threads, 0, s>>>(a);
        else if (grid) mover_fp64_kernel<2, false, true, true, false><<<g, threads, 0, s>>>(a);
        else if (ft) mover_fp64_kernel<2, true, true, false, false><<<g, threads, 0, s>>>(a);
        else if (full) mover_fp64_kernel<2, false, true, false, false><<<g, threads, 0, s>>>(a);
        else mover_fp64_kernel<2, false, false, false, false><<<g, threads, 0, s>>>(a);
    } else {
        if (grid && ft) mover_fp64_kernel<3, true, true, true, false><<<g, threads, 0, s>>>(a);
        else if (grid) mover_fp64_kernel<3, false, true, true, false><<<g, threads, 0, s>>>(a);
        else if (ft) mover_fp64_kernel<3, true, true, false, false><<<g, threads, 0, s>>>(a);
        else if (full) mover_fp64_kernel<3, false, true, false, false><<<g, threads, 0, s>>>(a);
        else mover_fp64_kernel<3, false, false, false, false><<<g, threads, 0, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace gpat
