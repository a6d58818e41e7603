/*
 * gpat_oracle.c -- CPU FP64 restatement of the reference's Parker mover.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline; see
 * gpat_oracle.h).  Parity is unpinned by reference tests: the reference has
 * none and cannot be built here.
 *
 * Every routine cites the Fortran routine it restates (paths relative to the
 * reference project root).  Expressions keep Fortran's left-to-right order;
 * build with -ffp-contract=off.
 */
#include "gpat_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Counter-based RNG: Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).    */
/* ------------------------------------------------------------------------ */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        uint64_t m0 = (uint64_t)0xD2511F53u * c0;
        uint64_t m1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(m0 >> 32), lo0 = (uint32_t)m0;
        uint32_t hi1 = (uint32_t)(m1 >> 32), lo1 = (uint32_t)m1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* 53-bit uniform on [0,1) from two 32-bit words. The reference draws
 * genrand_double1 (closed [0,1]); random_number_generator.f90:97-101. */
double orc_u01(uint32_t a, uint32_t b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

/* ------------------------------------------------------------------------ */
/* Exact weight sums: unsigned 128-bit fixed point, 64 fraction bits.       */
/* ------------------------------------------------------------------------ */
static void fixed_split(double w, uint64_t *h, uint64_t *l)
{
    double fl = floor(w);
    *h = (uint64_t)fl;
    *l = (uint64_t)((w - fl) * 18446744073709551616.0);
}

void orc_fixed_add(uint64_t *hi, uint64_t *lo, double w)
{
    uint64_t h, l;
    if (w >= 0.0) {
        fixed_split(w, &h, &l);
        uint64_t old = *lo;
        *lo = old + l;
        *hi += h + (*lo < old ? 1u : 0u);
    } else {
        fixed_split(-w, &h, &l);
        uint64_t old = *lo;
        *lo = old - l;
        *hi -= h + (old < l ? 1u : 0u);
    }
}

double orc_fixed_to_double(uint64_t hi, uint64_t lo)
{
    return (double)hi + (double)lo * (1.0 / 18446744073709551616.0);
}

/* ------------------------------------------------------------------------ */
/* Field gradients: mhd_data_parallel.f90:504-610 (calc_fields_gradients).   */
/* farray is (32, nxg, nyg, nzg) with the variable index fastest; the first  */
/* 8 variables are vx vy vz rho bx by bz |B|; variable v's d/dx, d/dy, d/dz  */
/* go to 8+3v, 8+3v+1, 8+3v+2.  Differences are single precision, scaled by */
/* the double 0.5/dx and rounded back to single.                            */
/* ------------------------------------------------------------------------ */
#define GA(a, v, i, j, k) (a)[(size_t)(v) + (size_t)stride * ((size_t)(i) + (size_t)nxg * ((size_t)(j) + (size_t)nyg * (size_t)(k)))]

/* One gradient component of variable v along an axis with node spacing
 * `step` (in records) at index `i` of `n`: central inside, one-sided 2nd
 * order at the two outermost nodes; FP32 differences scaled by the FP64
 * half inverse spacing, as the reference's real(sp) arrays. */
static float grad_axis(const float *a, size_t c, size_t step, int i, int n, double ih)
{
    if (i == 0) {
        float t = -(3.0f * a[c]);
        t = t + 4.0f * a[c + step];
        t = t - a[c + 2 * step];
        return (float)((double)t * ih);
    }
    if (i == n - 1) {
        float t = 3.0f * a[c];
        t = t - 4.0f * a[c - step];
        t = t + a[c - 2 * step];
        return (float)((double)t * ih);
    }
    const float t = a[c + step] - a[c - step];
    return (float)((double)t * ih);
}

/* Gradients of nvar variables (value at v * vstride of each record of
 * `stride` floats) into gbase + v * gstep + axis; the z component only in
 * 3D (in 2D it keeps whatever it held). */
static void grad_generic(float *a, int stride, int nvar, int vstride, int gbase, int gstep,
                         int ndim, int nxg, int nyg, int nzg, double dx, double dy, double dz,
                         const double *ihx, const double *ihy, const double *ihz)
{
    /* ih*: per-node inverse spans of a non-uniform grid (NULL: 0.5/d). */
    const double idxh = 0.5 / dx, idyh = 0.5 / dy, idzh = 0.5 / dz;
    const size_t sx = (size_t)stride, sy = sx * (size_t)nxg, sz = sy * (size_t)nyg;
    for (int k = 0; k < nzg; ++k)
        for (int j = 0; j < nyg; ++j)
            for (int i = 0; i < nxg; ++i)
                for (int v = 0; v < nvar; ++v) {
                    const size_t c = (size_t)v * vstride + sx * (size_t)i + sy * (size_t)j +
                                     sz * (size_t)k;
                    GA(a, gbase + v * gstep, i, j, k) =
                        grad_axis(a, c, sx, i, nxg, ihx ? ihx[i] : idxh);
                    if (nyg > 1)
                        GA(a, gbase + v * gstep + 1, i, j, k) =
                            grad_axis(a, c, sy, j, nyg, ihy ? ihy[j] : idyh);
                    if (nzg > 1 && ndim == 3)
                        GA(a, gbase + v * gstep + 2, i, j, k) =
                            grad_axis(a, c, sz, k, nzg, ihz ? ihz[k] : idzh);
                }
}

/* calc_fields_gradients (mhd_data_parallel.f90:504-610): 8 variables of
 * the 32-float records, gradients at 8 + 3 v + axis. */
void orc_calc_fields_gradients(float *a, int ndim, int nxg, int nyg, int nzg,
                               double dx, double dy, double dz)
{
    grad_generic(a, 32, 8, 1, 8, 3, ndim, nxg, nyg, nzg, dx, dy, dz, NULL, NULL, NULL);
}

/* calc_grad_sigma2_slab / _2d and calc_grad_lc_slab / _2d
 * (mhd_data_parallel.f90:771-1604) on the 16-float fluctuation records
 * {db2_slab, db2_2d, lc_slab, lc_2d} x {value, d/dx, d/dy, d/dz}. */
void orc_calc_aux_gradients(float *a, int ndim, int nxg, int nyg, int nzg,
                            double dx, double dy, double dz)
{
    grad_generic(a, 16, 4, 4, 1, 4, ndim, nxg, nyg, nzg, dx, dy, dz, NULL, NULL, NULL);
}

/* ------------------------------------------------------------------------ */
/* Grid positions for spherical and non-uniform grids.                      */
/* ------------------------------------------------------------------------ */
static struct {
    double *pos[3];   /* node positions, ghost nodes included               */
    double *ih[3];    /* idxh_grid: inverse spans for the gradients         */
    int n[3];
} g_grid;

/* set_local_grid_positions (mhd_data_parallel.f90:2153-2190) on one rank:
 * 1 / (x[i+1] - x[i-1]) inside, the one-sided spans at the two ends. */
static void inverse_spans(const double *x, int n, double *ih)
{
    if (n < 3) {
        for (int i = 0; i < n; ++i) ih[i] = 0.0;
        return;
    }
    for (int i = 1; i < n - 1; ++i) ih[i] = 1.0 / (x[i + 1] - x[i - 1]);
    ih[0] = 1.0 / (-(3.0 * x[0]) + 4.0 * x[1] - x[2]);
    ih[n - 1] = 1.0 / (3.0 * x[n - 1] - 4.0 * x[n - 2] + x[n - 3]);
}

void orc_set_grid_positions(const double *xpos, const double *ypos, const double *zpos,
                            int nxg, int nyg, int nzg)
{
    const double *src[3] = {xpos, ypos, zpos};
    const int n[3] = {nxg, nyg, nzg};
    for (int a = 0; a < 3; ++a) {
        free(g_grid.pos[a]);
        free(g_grid.ih[a]);
        g_grid.pos[a] = NULL;
        g_grid.ih[a] = NULL;
        g_grid.n[a] = 0;
        if (!src[a] || n[a] <= 0) continue;
        g_grid.pos[a] = (double *)malloc(sizeof(double) * (size_t)n[a]);
        g_grid.ih[a] = (double *)malloc(sizeof(double) * (size_t)n[a]);
        memcpy(g_grid.pos[a], src[a], sizeof(double) * (size_t)n[a]);
        inverse_spans(g_grid.pos[a], n[a], g_grid.ih[a]);
        g_grid.n[a] = n[a];
    }
}

void orc_uniform_grid_positions(int n, double d, double xmin, double *pos)
{
    for (int j = 0; j < n; ++j) pos[j] = d * (double)(j - 2) + xmin;
}

int orc_binary_search(const double *a, int n, double v)
{
    /* For increasing nodes the recursion of binarySearch_R returns the
     * count of nodes <= v; this is the same count by bisection. */
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = lo + (hi - lo) / 2;
        if (a[mid] > v) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

void orc_calc_fields_gradients_nonuniform(float *a, int ndim, int nxg, int nyg, int nzg)
{
    grad_generic(a, 32, 8, 1, 8, 3, ndim, nxg, nyg, nzg, 1.0, 1.0, 1.0, g_grid.ih[0],
                 g_grid.ih[1], g_grid.ih[2]);
}

void orc_calc_aux_gradients_nonuniform(float *a, int ndim, int nxg, int nyg, int nzg)
{
    grad_generic(a, 16, 4, 4, 1, 4, ndim, nxg, nyg, nzg, 1.0, 1.0, 1.0, g_grid.ih[0],
                 g_grid.ih[1], g_grid.ih[2]);
}

/* The node count along an axis, checked: the particle must lie between the
 * first and the last ghost node (the engine reports such a particle as an
 * index-guard error). */
static int grid_count(int axis, double v)
{
    const int n = g_grid.n[axis];
    const double *x = g_grid.pos[axis];
    if (!x || !(v >= x[1] && v < x[n - 1])) {
        fprintf(stderr, "oracle: position %.17g outside the grid along axis %d\n", v, axis);
        abort();
    }
    return orc_binary_search(x, n, v);
}

/* get_interp_paramters_spherical: particle_module.f90:705-775 (2D and 3D). */
static void spherical_weights(int ndim, double x, double y, double z, int32_t pos[3], double w[8])
{
    const double *X = g_grid.pos[0], *Y = g_grid.pos[1], *Z = g_grid.pos[2];
    pos[0] = grid_count(0, x) - 2;
    pos[1] = (ndim > 1) ? grid_count(1, y) - 2 : 1;
    pos[2] = (ndim == 3) ? grid_count(2, z) - 2 : 1;
    /* xpos_local(i) is X[i + 1]. */
    const double one_third = 1.0 / 3.0;
    const double x3 = x * x * x * one_third;
    const double xa = X[pos[0] + 1], xb = X[pos[0] + 2];
    const double x3_1 = xa * xa * xa * one_third;
    const double x3_2 = xb * xb * xb * one_third;
    const double rx = x3 - x3_1, rx1 = x3_2 - x3;
    double ry = 0.0, ry1 = 1.0;
    if (ndim > 1) {
        const double ctheta1 = cos(Y[pos[1] + 1]);
        const double ctheta2 = cos(Y[pos[1] + 2]);
        const double ctheta = cos(y);
        ry = ctheta1 - ctheta;
        ry1 = ctheta - ctheta2;
    }
    /* rz = 0, rz1 = 1 below 3D (1D leaves them unset in the reference) */
    double rz = 0.0, rz1 = 1.0;
    if (ndim == 3) {
        rz = z - Z[pos[2] + 1];
        rz1 = Z[pos[2] + 2] - z;
    }
    const double dv = (x3_2 - x3_1) * (ry + ry1) * (rz + rz1);
    w[0] = rx1 * ry1 * rz1;
    w[1] = rx * ry1 * rz1;
    w[2] = rx1 * ry * rz1;
    w[3] = rx * ry * rz1;
    w[4] = rx1 * ry1 * rz;
    w[5] = rx * ry1 * rz;
    w[6] = rx1 * ry * rz;
    w[7] = rx * ry * rz;
    for (int k = 0; k < 8; ++k) w[k] = w[k] / dv;
}

void orc_grid_interp_paramters(const orc_params *pr, const orc_mhd_config *cfg, double x,
                               double y, double z, int32_t pos[3], double w[8])
{
    const int ndim = pr->ndim;
    if (pr->spherical_coord) {
        spherical_weights(ndim, x, y, z, pos, w);
        return;
    }
    if (!pr->nonuniform_grid) {
        orc_get_interp_paramters(ndim, (x - cfg->xmin) / cfg->dx, (y - cfg->ymin) / cfg->dy,
                                 (z - cfg->zmin) / cfg->dz, pos, w);
        return;
    }
    /* :1620-1625 computes the offset inside the cell found by the search
     * and get_interp_paramters then places the corner at floor(offset) + 1,
     * i.e. at the first cell whatever the search found.  The corner is
     * shifted to the searched cell here (the reference's weights, the
     * intended cell). */
    const double *X = g_grid.pos[0], *Y = g_grid.pos[1], *Z = g_grid.pos[2];
    const int ix = grid_count(0, x) - 2;
    const int iy = (ndim > 1) ? grid_count(1, y) - 2 : 1;
    const int iz = (ndim == 3) ? grid_count(2, z) - 2 : 1;
    const double px = (x - X[ix + 1]) / (X[ix + 2] - X[ix + 1]);
    const double py = (ndim > 1) ? (y - Y[iy + 1]) / (Y[iy + 2] - Y[iy + 1]) : 0.0;
    const double pz = (ndim == 3) ? (z - Z[iz + 1]) / (Z[iz + 2] - Z[iz + 1]) : 0.0;
    orc_get_interp_paramters(ndim, px, py, pz, pos, w);
    pos[0] += ix - 1;
    if (ndim > 1) pos[1] += iy - 1;
    if (ndim == 3) pos[2] += iz - 1;
    const int hi[3] = {g_grid.n[0] - 3, g_grid.n[1] - 3, (ndim == 3) ? g_grid.n[2] - 3 : 1};
    for (int a = 0; a < ndim; ++a)
        if (pos[a] > hi[a]) {
            fprintf(stderr, "oracle: interpolation corner outside the grid along axis %d\n", a);
            abort();
        }
}

/* ------------------------------------------------------------------------ */
/* get_interp_paramters: particle_module.f90:642-674.  pos is returned as   */
/* the reference's 1-based Fortran index (ghost cells start at -1).         */
/* ------------------------------------------------------------------------ */
void orc_get_interp_paramters(int ndim, double px, double py, double pz,
                              int32_t pos[3], double w[8])
{
    double rx, ry, rz;
    pos[0] = (int32_t)floor(px) + 1;
    if (ndim == 1) {
        pos[1] = 1;
        pos[2] = 1;
        ry = 0.0;
        rz = 0.0;
    } else if (ndim == 2) {
        pos[1] = (int32_t)floor(py) + 1;
        pos[2] = 1;
        ry = (py - (double)pos[1]) + 1.0;
        rz = 0.0;
    } else {
        pos[1] = (int32_t)floor(py) + 1;
        pos[2] = (int32_t)floor(pz) + 1;
        ry = (py - (double)pos[1]) + 1.0;
        rz = (pz - (double)pos[2]) + 1.0;
    }
    rx = (px - (double)pos[0]) + 1.0;
    double rx1 = 1.0 - rx, ry1 = 1.0 - ry, rz1 = 1.0 - rz;
    w[0] = rx1 * ry1 * rz1;
    w[1] = rx * ry1 * rz1;
    w[2] = rx1 * ry * rz1;
    w[3] = rx * ry * rz1;
    w[4] = rx1 * ry1 * rz;
    w[5] = rx * ry1 * rz;
    w[6] = rx1 * ry * rz;
    w[7] = rx * ry * rz;
}

/* ------------------------------------------------------------------------ */
/* interp_fields: mhd_data_parallel.f90:1751-1804.  Fortran index i maps to */
/* C index i+1 in x and y; z is i+1 in 3D and 0 in 2D (declared 1:1).       */
/* ------------------------------------------------------------------------ */
void orc_interp_fields(const float *f1, const float *f2, int time_interp, int ndim,
                       int nxg, int nyg, const int32_t pos[3], const double w[8],
                       double rt, double fields[32])
{
    /* 1D arrays are declared (-1:nx+2, 1, 1): y is index 0 there */
    const int ix = pos[0] + 1, iy = (ndim > 1) ? pos[1] + 1 : 0;
    const int iz = (ndim == 3) ? pos[2] + 1 : 0;
    const int ze = (ndim == 3) ? 1 : 0, ye = (ndim > 1) ? 1 : 0;
    double fields2[32];
    for (int v = 0; v < 32; ++v) { fields[v] = 0.0; fields2[v] = 0.0; }
    for (int k = 0; k <= ze; ++k)
        for (int j = 0; j <= ye; ++j)
            for (int i = 0; i <= 1; ++i) {
                const int idx = k * 4 + j * 2 + i;
                const size_t c = 32u * ((size_t)(ix + i) + (size_t)nxg * ((size_t)(iy + j) + (size_t)nyg * (size_t)(iz + k)));
                for (int v = 0; v < 32; ++v) fields[v] = fields[v] + (double)f1[c + v] * w[idx];
                if (time_interp)
                    for (int v = 0; v < 32; ++v) fields2[v] = fields2[v] + (double)f2[c + v] * w[idx];
            }
    if (time_interp)
        for (int v = 0; v < 32; ++v) fields[v] = fields[v] * (1.0 - rt) + fields2[v] * rt;
}

/* interp_magnetic_fluctuation / interp_correlation_length
 * (mhd_data_parallel.f90:1806-1915): the 16-float fluctuation records with
 * the same weights and time interpolation as the fields. */
void orc_interp_aux(const float *a1, const float *a2, int time_interp, int ndim, int nxg,
                    int nyg, const int32_t pos[3], const double w[8], double rt, double out[16])
{
    const int ix = pos[0] + 1, iy = (ndim > 1) ? pos[1] + 1 : 0;
    const int iz = (ndim == 3) ? pos[2] + 1 : 0;
    const int ze = (ndim == 3) ? 1 : 0, ye = (ndim > 1) ? 1 : 0;
    double o2[16];
    for (int v = 0; v < 16; ++v) { out[v] = 0.0; o2[v] = 0.0; }
    for (int k = 0; k <= ze; ++k)
        for (int j = 0; j <= ye; ++j)
            for (int i = 0; i <= 1; ++i) {
                const int idx = k * 4 + j * 2 + i;
                const size_t c = 16u * ((size_t)(ix + i) + (size_t)nxg * ((size_t)(iy + j) + (size_t)nyg * (size_t)(iz + k)));
                for (int v = 0; v < 16; ++v) out[v] = out[v] + (double)a1[c + v] * w[idx];
                if (time_interp)
                    for (int v = 0; v < 16; ++v) o2[v] = o2[v] + (double)a2[c + v] * w[idx];
            }
    if (time_interp)
        for (int v = 0; v < 16; ++v) out[v] = out[v] * (1.0 - rt) + o2[v] * rt;
}

/* ------------------------------------------------------------------------ */
/* calc_spatial_diffusion_coefficients (particle_module.f90:2208-2450) and   */
/* calc_spatial_diffusion_coefficients_nlgc (:2464-2771) without delta-B or */
/* correlation-length inputs.  kappa follows kappa_type (:93-104):          */
/* knorm_para knorm_perp kpara kperp skpara skperp skpara_perp kxx kyy kzz  */
/* kxy kxz kyz dkxx_dx dkyy_dy dkzz_dz dkxy_dx dkxy_dy dkxz_dx dkxz_dz      */
/* dkyz_dy dkyz_dz.  Focused transport keeps only the perpendicular part    */
/* (kpp = -kperp).                                                          */
/* ------------------------------------------------------------------------ */
enum { K_KNORM_PARA, K_KNORM_PERP, K_KPARA, K_KPERP, K_SKPARA, K_SKPERP, K_SKPARA_PERP,
       K_KXX, K_KYY, K_KZZ, K_KXY, K_KXZ, K_KYZ, K_DKXX_DX, K_DKYY_DY, K_DKZZ_DZ,
       K_DKXY_DX, K_DKXY_DY, K_DKXZ_DX, K_DKXZ_DZ, K_DKYZ_DY, K_DKYZ_DZ };

/* Both variants write the gradient terms as
 *   dkii_di = T_i + A_i * bi^2 / B^2 + 2 kpp bi (dbi_di B - bi dB_di) / B^3
 *   dkij_dk = A_k * bi bj / B^2 + kpp ((dbi_dk bj + bi dbj_dk) / B^2 - 2 bi bj dB_dk / B^3)
 * with T_i = kperp dk_i, A_i = kpp dk_i for the fixed ratio (:2351-2449)
 * and T_i = kperp dkperp_i, A_i = kpara dkpara_i - kperp dkperp_i for NLGC
 * (:2583-2770); the operation order of each is the reference's. */
void orc_calc_spatial_diffusion_coefficients(const orc_params *pr, double p, double mu,
                                             const double f[32], const double *aux,
                                             double kap[22])
{
    /* aux: interpolated {db2_slab, db2_2d, lc_slab, lc_2d} x {value, d/dx,
     * d/dy, d/dz} (interp_magnetic_fluctuation, interp_correlation_length);
     * only read when deltab_flag / correlation_flag are on. */
    const double *s2 = aux, *d2 = aux ? aux + 4 : NULL, *l1 = aux ? aux + 8 : NULL;
    const double *l2 = aux ? aux + 12 : NULL;
    const int dbf = pr->deltab_flag && aux, lcf = pr->correlation_flag && aux;
    const double bx = f[4], by = f[5], bz = f[6];
    const double b = sqrt(bx * bx + by * by + bz * bz);
    double ib1 = (b < DBL_EPSILON) ? 1.0 : 1.0 / b;
    const double ib2 = ib1 * ib1;
    const double ib3 = ib1 * ib2;
    /* include_3rd_dim (2D data, 3D transport): the 3D tensor with the z
     * derivatives zero and the 2D gradient terms (:2293-2350, :2564-2640). */
    const int d3 = (pr->ndim == 3) || (pr->ndim == 2 && pr->include_3rd_dim);
    const int full3 = (pr->ndim == 3);
    double kpara, kperp;
    double knorm_para = 1.0, knorm_perp = 1.0;
    if (!pr->nlgc) {
        double knorm;
        if (pr->mag_dependency == 1) knorm_para = knorm_para * pow(b, pr->gamma_turb - 2.0);
        if (dbf) knorm_para = knorm_para / s2[0];
        if (lcf) knorm_para = knorm_para * pow(l1[0], pr->gamma_turb - 1.0);
        if (pr->momentum_dependency == 1) knorm = knorm_para * pow(p / pr->p0, pr->pindex);
        else knorm = knorm_para;
        knorm_perp = knorm_para;
        kpara = pr->kpara0 * knorm;
        kperp = kpara * pr->kret;
    } else {
        double kn_para, kn_perp;
        if (pr->mag_dependency == 1) {
            knorm_para = knorm_para * pow(b, pr->gamma_turb - 2.0);
            knorm_perp = knorm_perp * pow(b, (pr->gamma_turb - 2.0) / 3.0);
        }
        if (dbf) {
            knorm_para = knorm_para / s2[0];
            knorm_perp = knorm_perp * pow(s2[0], -1.0 / 3.0) * pow(d2[0], 2.0 / 3.0);
        }
        if (lcf) {
            knorm_para = knorm_para * pow(l1[0], pr->gamma_turb - 1.0);
            knorm_perp = knorm_perp * pow(l1[0], (pr->gamma_turb - 1.0) / 3.0) *
                         pow(l2[0], 2.0 / 3.0);
        }
        if (pr->momentum_dependency == 1) {
            kn_para = knorm_para * pow(p / pr->p0, pr->pindex);
            kn_perp = knorm_perp * pow(p / pr->p0, (5.0 - pr->gamma_turb) / 3.0);
        } else {
            kn_para = knorm_para;
            kn_perp = knorm_perp;
        }
        kpara = pr->kpara0 * kn_para;
        kperp = pr->kpara0 * pr->kperp_kpara * kn_perp * (mu * mu);
    }
    kap[K_KNORM_PARA] = knorm_para;
    kap[K_KNORM_PERP] = knorm_perp;
    kap[K_KPARA] = kpara;
    kap[K_KPERP] = kperp;
    kap[K_SKPARA] = sqrt(2.0 * kpara);
    kap[K_SKPERP] = sqrt(2.0 * kperp);
    kap[K_SKPARA_PERP] = sqrt(2.0 * (kpara - kperp));
    const double kpp = pr->focused_transport ? -kperp : kpara - kperp;
    if (pr->ndim == 1) {
        /* the 1D branches (:2270-2291, :2536-2562): only dkxx_dx, and kxx
         * for spherical coordinates */
        for (int k = K_KXX; k <= K_DKYZ_DZ; ++k) kap[k] = 0.0;
        const double dbdx = f[29];
        double dk = 0.0, dkperp = 0.0;
        if (pr->mag_dependency == 1) {
            dk = dbdx * ib1 * (pr->gamma_turb - 2.0);
            dkperp = dbdx * ib1 * (pr->gamma_turb - 2.0) / 3.0;
        }
        if (dbf) {
            dk = dk - s2[1] / s2[0];
            dkperp = dkperp - s2[1] / s2[0] / 3.0 + 2.0 * d2[1] / d2[0] / 3.0;
        }
        if (lcf) {
            dk = dk + (pr->gamma_turb - 1.0) * l1[1] / l1[0];
            dkperp = dkperp + (pr->gamma_turb - 1.0) * l1[1] / l1[0] / 3.0 +
                     2.0 * l2[1] / l2[0] / 3.0;
        }
        if (!pr->nlgc) dkperp = dk;   /* the fixed-ratio branch has one dkdx */
        if (pr->focused_transport) {
            kap[K_DKXX_DX] = kperp * dkperp;
            if (pr->spherical_coord) kap[K_KXX] = kperp;
        } else {
            kap[K_DKXX_DX] = kpara * dk;
            if (pr->spherical_coord) kap[K_KXX] = kpara;
        }
        return;
    }

    const double dbx_dx = f[20], dbx_dy = f[21], dbx_dz = f[22];
    const double dby_dx = f[23], dby_dy = f[24], dby_dz = f[25];
    const double dbz_dx = f[26], dbz_dy = f[27], dbz_dz = f[28];
    const double db_dx = f[29], db_dy = f[30], db_dz = f[31];
    double T[3] = {0.0, 0.0, 0.0}, A[3] = {0.0, 0.0, 0.0};
    const double db[3] = {db_dx, db_dy, db_dz};
    const double g2 = pr->gamma_turb - 2.0;
    for (int k = 0; k < 2 + full3; ++k) {
        if (!pr->nlgc) {
            double dk = 0.0;
            if (pr->mag_dependency == 1)
                /* the fixed-ratio 3D branch has no 1/B factor (:2406-2408) */
                dk = full3 ? db[k] * g2 : db[k] * ib1 * g2;
            if (dbf) dk = dk - s2[1 + k] / s2[0];
            if (lcf) dk = dk + (pr->gamma_turb - 1.0) * l1[1 + k] / l1[0];
            T[k] = kperp * dk;
            A[k] = kpp * dk;
        } else {
            double dkpara = 0.0, dkperp = 0.0;
            if (pr->mag_dependency == 1) {
                dkpara = db[k] * ib1 * g2;
                dkperp = db[k] * ib1 * g2 / 3.0;
            }
            if (dbf) {
                dkpara = dkpara - s2[1 + k] / s2[0];
                dkperp = dkperp - s2[1 + k] / s2[0] / 3.0 + 2.0 * d2[1 + k] / d2[0] / 3.0;
            }
            if (lcf) {
                dkpara = dkpara + (pr->gamma_turb - 1.0) * l1[1 + k] / l1[0];
                dkperp = dkperp + (pr->gamma_turb - 1.0) * l1[1 + k] / l1[0] / 3.0 +
                         2.0 * l2[1 + k] / l2[0] / 3.0;
            }
            T[k] = kperp * dkperp;
            A[k] = kpara * dkpara - kperp * dkperp;
        }
    }
    kap[K_DKXX_DX] = T[0] + A[0] * (bx * bx) * ib2 + 2.0 * kpp * bx * (dbx_dx * b - bx * db_dx) * ib3;
    kap[K_DKYY_DY] = T[1] + A[1] * (by * by) * ib2 + 2.0 * kpp * by * (dby_dy * b - by * db_dy) * ib3;
    kap[K_DKXY_DX] = A[0] * bx * by * ib2 +
                     kpp * ((dbx_dx * by + bx * dby_dx) * ib2 - 2.0 * bx * by * db_dx * ib3);
    kap[K_DKXY_DY] = A[1] * bx * by * ib2 +
                     kpp * ((dbx_dy * by + bx * dby_dy) * ib2 - 2.0 * bx * by * db_dy * ib3);
    kap[K_KXX] = kperp + kpp * bx * bx * ib2;
    kap[K_KYY] = kperp + kpp * by * by * ib2;
    kap[K_KXY] = kpp * bx * by * ib2;
    if (!d3) {
        kap[K_KZZ] = 0.0; kap[K_KXZ] = 0.0; kap[K_KYZ] = 0.0;
        kap[K_DKZZ_DZ] = 0.0; kap[K_DKXZ_DX] = 0.0; kap[K_DKXZ_DZ] = 0.0;
        kap[K_DKYZ_DY] = 0.0; kap[K_DKYZ_DZ] = 0.0;
    } else {
        kap[K_DKZZ_DZ] = T[2] + A[2] * (bz * bz) * ib2 +
                         2.0 * kpp * bz * (dbz_dz * b - bz * db_dz) * ib3;
        kap[K_DKXZ_DX] = A[0] * bx * bz * ib2 +
                         kpp * ((dbx_dx * bz + bx * dbz_dx) * ib2 - 2.0 * bx * bz * db_dx * ib3);
        kap[K_DKXZ_DZ] = A[2] * bx * bz * ib2 +
                         kpp * ((dbx_dz * bz + bx * dbz_dz) * ib2 - 2.0 * bx * bz * db_dz * ib3);
        kap[K_DKYZ_DY] = A[1] * by * bz * ib2 +
                         kpp * ((dby_dy * bz + by * dbz_dy) * ib2 - 2.0 * by * bz * db_dy * ib3);
        kap[K_DKYZ_DZ] = A[2] * by * bz * ib2 +
                         kpp * ((dby_dz * bz + by * dbz_dz) * ib2 - 2.0 * by * bz * db_dz * ib3);
        kap[K_KZZ] = kperp + kpp * bz * bz * ib2;
        kap[K_KXZ] = kpp * bx * bz * ib2;
        kap[K_KYZ] = kpp * by * bz * ib2;
    }
}

/* ------------------------------------------------------------------------ */
/* Mover.                                                                    */
/* ------------------------------------------------------------------------ */
typedef struct mover_ctx {
    const orc_params *pr;
    const float *f1, *f2;
    const float *aux1, *aux2;      /* 16-float fluctuation records, or NULL */
    int time_interp, ndim, nxg, nyg;
    double dx, dy, dz;
    double xmin, ymin, zmin;                   /* fconfig box (exact)      */
    double xmin1, xmax1, ymin1, ymax1, zmin1, zmax1;  /* half-cell-extended */
    double cfg_xmin, cfg_ymin, cfg_zmin, cfg_lx, cfg_ly, cfg_lz;
    double dt_min, dt_max, t0, dtf;
    uint32_t key[2];
    int sph, nonuni;       /* spherical_coord, nonuniform_grid             */
    int i3;                /* include_3rd_dim of a 2D run                  */
} mover_ctx;

typedef struct ptl_state {
    double x, y, z, p, v, mu, t, dt, weight;
    double h1, h2;   /* acceleration-surface heights at the push's start */
    int flag, split_times;
    int32_t nsteps_pushed, tag_injected, tag_splitted, origin, nsteps_tracked;
    uint32_t rng_ctr;
} ptl_state;

/* ------------------------------------------------------------------------ */
/* Particle tracking (particle_module.f90:144-150, 5825-6030): the table    */
/* tags_tracking(nrows, n) and the records particles_tracked(nsteps_max, n), */
/* both Fortran order, owned by the caller.                                 */
/* ------------------------------------------------------------------------ */
typedef struct {
    const int32_t *tags;
    int nrows, n;
    int64_t nsteps_max;
    orc_particles rec;
    int64_t dropped;
} orc_tracking;
static orc_tracking g_trk;

void orc_set_tracking(const int32_t *tags, int nrows, int n, int64_t nsteps_max,
                      const orc_particles *rec)
{
    memset(&g_trk, 0, sizeof g_trk);
    if (!tags) return;
    g_trk.tags = tags; g_trk.nrows = nrows; g_trk.n = n; g_trk.nsteps_max = nsteps_max;
    g_trk.rec = *rec;
}

int64_t orc_tracking_dropped(void) { return g_trk.dropped; }

/* nsteps_tracking_max = ceiling((1.0 / dt_min_rel) / nsteps_interval) + 1
 * (:5874). */
int64_t orc_nsteps_tracking_max(double dt_min_rel, int nsteps_interval)
{
    return (int64_t)ceil((1.0 / dt_min_rel) / (double)nsteps_interval) + 1;
}

/* findloc(tags_tracking(row, from:to), v [, back]) as a 1-based column
 * (0: none); row and columns 1-based. */
static int trk_findloc(int row, int32_t v, int from, int to, int back)
{
    const int32_t *T = g_trk.tags;
    if (!back) {
        for (int j = from; j <= to; ++j)
            if (T[(size_t)(j - 1) * g_trk.nrows + (row - 1)] == v) return j;
    } else {
        for (int j = to; j >= from; --j)
            if (T[(size_t)(j - 1) * g_trk.nrows + (row - 1)] == v) return j;
    }
    return 0;
}

/* is_particle_selected (:5923-5963) with 1-based iptl_lo / iptl_hi.
 * locate_particle (:5971-5994) is the same search for a tracked particle,
 * whose split count never exceeds the table's; one that is not listed
 * (out-of-range indexing in the reference) records nothing here. */
static int trk_selected(int32_t origin, int32_t tag_inj, int nsplit, int32_t tag_spl,
                        int *lo, int *hi)
{
    const int split_times_max = g_trk.nrows - 2;
    *lo = -1; *hi = -1;
    if (nsplit > split_times_max || nsplit < 0) return 0;
    const int i1 = trk_findloc(1, origin, 1, g_trk.n, 0);
    if (i1 == 0) return 0;
    const int i2 = trk_findloc(1, origin, 1, g_trk.n, 1);
    const int32_t ai = tag_inj < 0 ? -tag_inj : tag_inj;
    const int i3 = trk_findloc(2, ai, i1, i2, 0);
    if (i3 == 0) return 0;
    const int i4 = trk_findloc(2, ai, i1, i2, 1);
    if (nsplit > 0) {
        const int32_t as = tag_spl < 0 ? -tag_spl : tag_spl;
        const int i5 = trk_findloc(nsplit + 2, as, i3, i4, 0);
        if (i5 == 0) return 0;
        *lo = i5;
        *hi = trk_findloc(nsplit + 2, as, i3, i4, 1);
    } else {
        *lo = i3;
        *hi = i4;
    }
    return 1;
}

/* particles_tracked(row, lo:hi) = ptl (1-based); a row past nsteps_max is
 * counted instead of written. */
static void trk_write(int64_t row, int lo, int hi, const orc_particles *S, int64_t i,
                      const ptl_state *s)
{
    if (row < 1 || row > g_trk.nsteps_max) {
#ifdef _OPENMP
#pragma omp atomic
#endif
        g_trk.dropped += 1;
        return;
    }
    const orc_particles *D = &g_trk.rec;
    for (int j = lo; j <= hi; ++j) {
        const size_t e = (size_t)(row - 1) + (size_t)g_trk.nsteps_max * (size_t)(j - 1);
        if (s) {
            D->x[e] = s->x; D->y[e] = s->y; D->z[e] = s->z; D->p[e] = s->p;
            D->v[e] = s->v; D->mu[e] = s->mu; D->weight[e] = s->weight;
            D->t[e] = s->t; D->dt[e] = s->dt;
            D->split_times[e] = (int8_t)s->split_times; D->count_flag[e] = (int8_t)s->flag;
            D->origin[e] = s->origin; D->nsteps_tracked[e] = s->nsteps_tracked;
            D->nsteps_pushed[e] = s->nsteps_pushed;
            D->tag_injected[e] = s->tag_injected; D->tag_splitted[e] = s->tag_splitted;
            D->rng_ctr[e] = s->rng_ctr;
        } else {
            D->x[e] = S->x[i]; D->y[e] = S->y[i]; D->z[e] = S->z[i]; D->p[e] = S->p[i];
            D->v[e] = S->v[i]; D->mu[e] = S->mu[i]; D->weight[e] = S->weight[i];
            D->t[e] = S->t[i]; D->dt[e] = S->dt[i];
            D->split_times[e] = S->split_times[i]; D->count_flag[e] = S->count_flag[i];
            D->origin[e] = S->origin[i]; D->nsteps_tracked[e] = S->nsteps_tracked[i];
            D->nsteps_pushed[e] = S->nsteps_pushed[i];
            D->tag_injected[e] = S->tag_injected[i]; D->tag_splitted[e] = S->tag_splitted[i];
            D->rng_ctr[e] = S->rng_ctr[i];
        }
    }
}

/* The mover's record after a push (:1697-1703, :1806-1812). */
static void trk_after_push(ptl_state *s)
{
    if (!g_trk.tags) return;
    if (s->tag_splitted < 0 && s->nsteps_pushed == 0) {
        int lo, hi;
        const int found = trk_selected(s->origin, s->tag_injected, s->split_times,
                                       s->tag_splitted, &lo, &hi);
        s->nsteps_tracked = s->nsteps_tracked + 1;
        if (found) trk_write(s->nsteps_tracked, lo, hi, NULL, 0, s);
    }
}

/* inject_one_particle's tracking block (:434-440, :622-628) for the new
 * particle c. */
static void trk_injected(orc_particles *P, int64_t c)
{
    int lo, hi;
    if (!g_trk.tags) return;
    if (!trk_selected(P->origin[c], P->tag_injected[c], P->split_times[c], P->tag_splitted[c],
                      &lo, &hi))
        return;
    P->nsteps_tracked[c] = 1;
    P->tag_injected[c] = -P->tag_injected[c];
    P->tag_splitted[c] = -1;
    trk_write(1, lo, hi, P, c, NULL);
}

/* sync_tracked_particles on one rank (:5994-6030): per column, the records
 * with tag_splitted < 0 shifted to the front in order, the rest zeroed
 * (the MPI_SCAN offset is 0 and the reductions are copies). */
void orc_sync_tracked(void)
{
    const orc_particles *D = &g_trk.rec;
    for (int c = 0; c < g_trk.n; ++c) {
        const size_t base = (size_t)g_trk.nsteps_max * (size_t)c;
        int64_t j = 0;
        for (int64_t i = 0; i < g_trk.nsteps_max; ++i) {
            const size_t a = base + (size_t)i, b = base + (size_t)j;
            if (D->tag_splitted[a] < 0) {
                D->x[b] = D->x[a]; D->y[b] = D->y[a]; D->z[b] = D->z[a]; D->p[b] = D->p[a];
                D->v[b] = D->v[a]; D->mu[b] = D->mu[a]; D->weight[b] = D->weight[a];
                D->t[b] = D->t[a]; D->dt[b] = D->dt[a];
                D->split_times[b] = D->split_times[a]; D->count_flag[b] = D->count_flag[a];
                D->origin[b] = D->origin[a]; D->nsteps_tracked[b] = D->nsteps_tracked[a];
                D->nsteps_pushed[b] = D->nsteps_pushed[a];
                D->tag_injected[b] = D->tag_injected[a];
                D->tag_splitted[b] = D->tag_splitted[a];
                D->rng_ctr[b] = D->rng_ctr[a];
                j += 1;
            }
        }
        for (int64_t i = j; i < g_trk.nsteps_max; ++i) {
            const size_t b = base + (size_t)i;
            D->x[b] = 0.0; D->y[b] = 0.0; D->z[b] = 0.0; D->p[b] = 0.0; D->v[b] = 0.0;
            D->mu[b] = 0.0; D->weight[b] = 0.0; D->t[b] = 0.0; D->dt[b] = 0.0;
            D->split_times[b] = 0; D->count_flag[b] = 0; D->origin[b] = 0;
            D->nsteps_tracked[b] = 0; D->nsteps_pushed[b] = 0;
            D->tag_injected[b] = 0; D->tag_splitted[b] = 0; D->rng_ctr[b] = 0;
        }
    }
}

typedef struct thread_acc {
    uint64_t leak_hi, leak_lo, negp_hi, negp_lo, steps;
} thread_acc;

/* Four unit-variance increments for one push, drawn in the reference's order
 * ran1, ran2, ran3 (position) then ran1 again (momentum); :3546-3590. */
static void push_noise_n(const mover_ctx *c, ptl_state *s, double *r, int n6)
{
    uint32_t w[8];
    uint32_t ctr[4] = {s->rng_ctr, 0u, (uint32_t)s->tag_injected, (uint32_t)s->tag_splitted};
    orc_philox4x32_10(ctr, c->key, w);
    ctr[1] = 1u;
    orc_philox4x32_10(ctr, c->key, w + 4);
    if (n6) {
        /* A third block for pushes that draw five numbers (3D spherical
         * focused transport); r[4] and r[5] come from it. */
        uint32_t w3[4];
        ctr[1] = 2u;
        orc_philox4x32_10(ctr, c->key, w3);
        const double u4 = orc_u01(w3[0], w3[1]), u5 = orc_u01(w3[2], w3[3]);
        if (c->pr->noise == 0) {
            r[4] = (2.0 * u4 - 1.0) * sqrt(3.0);
            r[5] = (2.0 * u5 - 1.0) * sqrt(3.0);
        } else {
            const double rc = sqrt(-2.0 * log(1.0 - u4));
            r[4] = rc * cos(6.283185307179586 * u5);
            r[5] = rc * sin(6.283185307179586 * u5);
        }
    }
    s->rng_ctr += 1u;
    const double u0 = orc_u01(w[0], w[1]), u1 = orc_u01(w[2], w[3]);
    const double u2 = orc_u01(w[4], w[5]), u3 = orc_u01(w[6], w[7]);
    if (c->pr->noise == 0) {
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

static void push_noise(const mover_ctx *c, ptl_state *s, double r[4])
{
    push_noise_n(c, s, r, 0);
}

/* Metric factors of spherical coordinates (x = r, y = theta, z = phi) set
 * at the top of every push (:3420-3427, :4707-4713). */
typedef struct sph_terms {
    double ctheta, istheta, cot_theta, ir, ir2;
} sph_terms;

static sph_terms spherical_terms(const ptl_state *s)
{
    sph_terms t;
    t.ctheta = cos(s->y);
    t.istheta = 1.0 / sin(s->y);
    t.cot_theta = t.ctheta * t.istheta;
    t.ir = 1.0 / s->x;
    t.ir2 = 1.0 / (s->x * s->x);
    return t;
}

/* The position noise of the 2D spherical pushes: eigen-decomposition of
 * the (r, theta) diffusion tensor (:3559-3580, :3905-3925). */
static void spherical_noise_2d(const double *kap, const sph_terms *g, double r1, double r2,
                               double sdt, double *nx, double *ny)
{
    const double a1 = kap[K_KXX];
    const double b1 = kap[K_KXY] * g->ir;
    const double c1 = kap[K_KYY] * g->ir2;
    const double amc = a1 - c1;
    const double atmp = sqrt(amc * amc + 4.0 * (b1 * b1));
    const double Qpp = atmp + (a1 + c1);
    double Qmp = atmp - (a1 + c1);
    const double Qpm = atmp + (a1 - c1);
    const double Qmm = atmp - (a1 - c1);
    if (Qmp > 0.0) Qmp = 0.0;
    const double qtmp1 = sqrt(-Qmp / (Qmm * Qmm + 4.0 * (b1 * b1)));
    const double qtmp2 = sqrt(Qpp / (Qpm * Qpm + 4.0 * (b1 * b1)));
    *nx = (-(Qmm * qtmp1 * r1) + Qpm * qtmp2 * r2) * sdt;
    *ny = (2.0 * b1 * qtmp1 * r1 + 2.0 * b1 * qtmp2 * r2) * sdt;
}

/* The 3D spherical noise matrix (upper triangular, P P^T = 2 K in the
 * metric); `clamp` adds the focused-transport pushes' guards against
 * small negative radicands (:5253-5278) that the Parker push lacks
 * (:4852-4863). */
static void spherical_noise_3d(const double *kap, const sph_terms *g, int clamp, double p[6])
{
    const double kxx = kap[K_KXX], kyy = kap[K_KYY], kzz = kap[K_KZZ];
    const double kxy = kap[K_KXY], kxz = kap[K_KXZ], kyz = kap[K_KYZ];
    const double num = kxx * (kyz * kyz) + kyy * (kxz * kxz) + kzz * (kxy * kxy) -
                       2.0 * kxy * kxz * kyz - kxx * kyy * kzz;
    const double den = kyz * kyz - kyy * kzz;
    double d = 2.0 * num / den;
    if (clamp && d < 0.0) d = 0.0;
    p[0] = sqrt(d);                                            /* p11 */
    d = 2.0 * (kyy - kyz * kyz / kzz);
    if (clamp && d < 0.0) d = 0.0;
    p[1] = (kxz * kyz - kxy * kzz) * sqrt(d) / den;            /* p12 */
    p[3] = sqrt(d) * g->ir;                                    /* p22 */
    if (clamp && kzz <= 0.0) {
        p[2] = 0.0; p[4] = 0.0; p[5] = 0.0;
    } else {
        p[2] = sqrt(2.0 / kzz) * kxz;                          /* p13 */
        p[4] = sqrt(2.0 / kzz) * kyz * g->ir;                  /* p23 */
        p[5] = sqrt(2.0 * kzz) * g->istheta * g->ir;           /* p33 */
    }
}

/* particle_in_acceleration_region: particle_module.f90:2885-2906. */
/* ------------------------------------------------------------------------ */
/* Surfaces separating the acceleration region in 3D runs                    */
/* (acc_region_surface.f90): heights over the plane normal to one axis,      */
/* ghost-padded, the first index fastest.                                    */
/* ------------------------------------------------------------------------ */
static struct {
    int on, has2, intersection;
    int axis[2], sign[2];      /* normal axis 0/1/2; +1: the region is above */
    int ld[2];                 /* leading dimension of each surface array     */
    double *h[2][2];           /* [surface][slot]                             */
} g_surf;

static int surf_ld(int axis, int nxg, int nyg)
{
    return axis == 0 ? nyg : nxg;   /* x: (nyg, nzg); y: (nxg, nzg); z: (nxg, nyg) */
}

void orc_set_acc_surface(int axis1, int sign1, int axis2, int sign2, int has2, int intersection,
                         const double *s11, const double *s12, const double *s21,
                         const double *s22, int nxg, int nyg, int nzg)
{
    for (int k = 0; k < 2; ++k)
        for (int t = 0; t < 2; ++t) {
            free(g_surf.h[k][t]);
            g_surf.h[k][t] = NULL;
        }
    g_surf.on = s11 != NULL;
    if (!g_surf.on) return;
    g_surf.has2 = has2 && s21;
    g_surf.intersection = intersection;
    g_surf.axis[0] = axis1; g_surf.sign[0] = sign1;
    g_surf.axis[1] = axis2; g_surf.sign[1] = sign2;
    const int n[3] = {nxg, nyg, nzg};
    const double *src[2][2] = {{s11, s12}, {s21, s22}};
    for (int k = 0; k < 1 + g_surf.has2; ++k) {
        const int ax = g_surf.axis[k];
        g_surf.ld[k] = surf_ld(ax, nxg, nyg);
        const size_t cnt = (size_t)g_surf.ld[k] * (size_t)(ax == 2 ? n[1] : n[2]);
        for (int t = 0; t < 2; ++t) {
            const double *q = src[k][t] ? src[k][t] : src[k][0];
            g_surf.h[k][t] = (double *)malloc(sizeof(double) * cnt);
            memcpy(g_surf.h[k][t], q, sizeof(double) * cnt);
        }
    }
}

/* interp_acc_surface (acc_region_surface.f90:255-335): the 3D weights
 * summed along the normal, Fortran sum order over the 2 x 2 corners. */
static double surface_height(int k, const int32_t pos[3], const double w[8], double rt,
                             int time_interp)
{
    const int ax = g_surf.axis[k];
    int i1, j1;
    double w2[4];   /* (1,1) (2,1) (1,2) (2,2) */
    if (ax == 0) {
        i1 = pos[1] + 1; j1 = pos[2] + 1;
        w2[0] = w[0] + w[1]; w2[1] = w[2] + w[3]; w2[2] = w[4] + w[5]; w2[3] = w[6] + w[7];
    } else if (ax == 1) {
        i1 = pos[0] + 1; j1 = pos[2] + 1;
        w2[0] = w[0] + w[2]; w2[1] = w[1] + w[3]; w2[2] = w[4] + w[6]; w2[3] = w[5] + w[7];
    } else {
        i1 = pos[0] + 1; j1 = pos[1] + 1;
        w2[0] = w[0] + w[4]; w2[1] = w[1] + w[5]; w2[2] = w[2] + w[6]; w2[3] = w[3] + w[7];
    }
    double hs[2];
    for (int t = 0; t < 1 + (time_interp != 0); ++t) {
        const double *a = g_surf.h[k][t];
        const size_t ld = (size_t)g_surf.ld[k];
        double sum = 0.0;
        sum = sum + a[(size_t)i1 + ld * (size_t)j1] * w2[0];
        sum = sum + a[(size_t)i1 + 1 + ld * (size_t)j1] * w2[1];
        sum = sum + a[(size_t)i1 + ld * (size_t)(j1 + 1)] * w2[2];
        sum = sum + a[(size_t)i1 + 1 + ld * (size_t)(j1 + 1)] * w2[3];
        hs[t] = sum;
    }
    return time_interp ? hs[0] * (1.0 - rt) + hs[1] * rt : hs[0];
}

/* check_above_acc_surface (acc_region_surface.f90:343-383). */
static int above_surfaces(const ptl_state *s)
{
    const double xyz[3] = {s->x, s->y, s->z};
    double ph = xyz[g_surf.axis[0]];
    int in = g_surf.sign[0] > 0 ? ph > s->h1 : ph < s->h1;
    if (g_surf.has2) {
        ph = xyz[g_surf.axis[1]];
        const int in2 = g_surf.sign[1] > 0 ? ph > s->h2 : ph < s->h2;
        in = g_surf.intersection ? (in && in2) : (in || in2);
    }
    return in;
}

static int in_acc_region(const mover_ctx *c, const ptl_state *s)
{
    const double *a = c->pr->acc_region;
    const double xn = (s->x - c->cfg_xmin) / c->cfg_lx;
    int in = (xn >= a[0]) && (xn <= a[1]);
    if (c->ndim > 1) {
        const double yn = (s->y - c->cfg_ymin) / c->cfg_ly;
        in = in && (yn >= a[2]) && (yn <= a[3]);
    }
    if (c->ndim == 3) {
        const double zn = (s->z - c->cfg_zmin) / c->cfg_lz;
        in = in && (zn >= a[4]) && (zn <= a[5]);
        /* push_particle_3d / _3d_ft with acc_by_surface (:4889-4893) */
        if (g_surf.on) in = in && above_surfaces(s);
    }
    return in;
}

static double vdrift_prefactor(const orc_params *pr, double p)
{
    /* 1.0 / (3 * pcharge) is single precision in the reference. */
    const float q = 1.0f / (float)(3 * pr->charge);
    const double t1 = pr->drift1 * pr->p0 / p;
    const double t2 = pr->drift2 * (pr->p0 * pr->p0) / (p * p);
    return (double)q / sqrt(t1 * t1 + t2 * t2);
}

/* calc_dpp_wave_scattering (:2918-2931) and calc_dpp_flow_shear
 * (:2946-2979) as called by the pushes (:3479-3496, :4764-4788): they add
 * to dp_dt and return dpp.  Shear tensor sigma_ij = (dvi/dj + dvj/di)/2 -
 * delta_ij divv/3 (dvz/dz = 0 and no xz, yz terms in 2D). */
static double dpp_terms(const orc_params *pr, double p, const double *f, const double *kap,
                        double b, double divv, double *dp_dt)
{
    double dpp = 0.0;
    if (pr->dpp_wave) {
        const double va = b / sqrt(f[3]);
        if (pr->momentum_dependency == 1)
            *dp_dt = *dp_dt + (8.0 * p / (27.0 * kap[K_KPARA])) * (va * va);
        else
            *dp_dt = *dp_dt + (4.0 * p / (9.0 * kap[K_KPARA])) * (va * va);
        dpp = dpp + (p * va) * (p * va) / (9.0 * kap[K_KPARA]);
    }
    if (pr->dpp_shear) {
        const int d3 = (pr->ndim == 3) || pr->include_3rd_dim;
        const double sxx = f[8] - divv / 3.0;
        const double syy = f[12] - divv / 3.0;
        const double szz = d3 ? f[16] - divv / 3.0 : -(divv / 3.0);
        /* the 1D pushes pass zero off-diagonal shear (:3052-3057) */
        const double sxy = pr->ndim > 1 ? (f[9] + f[11]) / 2.0 : 0.0;
        const double sxz = d3 ? (f[10] + f[14]) / 2.0 : 0.0;
        const double syz = d3 ? (f[13] + f[15]) / 2.0 : 0.0;
        const double bx = f[4], by = f[5], bz = f[6];
        double gshear;
        if (pr->weak_scattering) {
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
            const double kn = kap[K_KNORM_PARA];
            const double p0f = pow(pr->p0, 2.0 - pr->pindex);
            *dp_dt = *dp_dt + (2.0 + pr->pindex) * gshear * pr->tau0 * kn *
                     pow(p, pr->pindex - 1.0) * p0f;
            dpp = dpp + gshear * pr->tau0 * kn * pow(p, pr->pindex) * p0f;
        }
    }
    return dpp;
}

/* Momentum update, acceleration-region mask and the 0.25 p0 floor, shared
 * by the 2D and 3D pushes (:3591-3605, :4885-4906). */
static void push_momentum(const mover_ctx *c, ptl_state *s, double dp_dt, double dpp, double sdt,
                          double ranp, double *deltap)
{
    double dP = dp_dt * s->dt + ranp * sqrt(2.0 * dpp) * sdt;
    if (c->pr->acc_region_flag == 1) {
        if (in_acc_region(c, s)) s->p = s->p + dP;
        else dP = 0.0;
    } else {
        s->p = s->p + dP;
    }
    const double pfloor = (double)0.25f * c->pr->p0;
    if (s->p < pfloor) {
        s->p = s->p - dP;
        dP = pfloor - s->p;
        s->p = pfloor;
    }
    *deltap = dP;
}

/* Cell sizes seen by a push: mhd_config's dx, dy, dz on a uniform grid,
 * the searched cell's spans on a non-uniform one (:3400-3408, :4689-4700). */
typedef struct cell_size {
    double dxm, dym, dzm;
} cell_size;

/* push_particle_2d: particle_module.f90:3358-3606, Cartesian and
 * spherical (x = r, y = theta). */
static void push_2d(const mover_ctx *c, ptl_state *s, const double *f, const double *kap,
                    const cell_size *cs, int fixed_dt, double d[6])
{
    const orc_params *pr = c->pr;
    const double vx = f[0], vy = f[1], bx = f[4], by = f[5], bz = f[6];
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double dvx_dx = f[8], dvy_dy = f[12];
    const double dxm = cs->dxm, dym = cs->dym;
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    sph_terms g = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (c->sph) g = spherical_terms(s);
    const double dbz_dx = f[26], dbz_dy = f[27], db_dx = f[29], db_dy = f[30];
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor(pr, s->p);
    double vdx, vdy, gbr = 0.0, gbt = 0.0;
    if (c->sph) {
        gbr = db_dx;
        gbt = db_dy * g.ir;
        vdx = vdp * ((dbz_dy + g.cot_theta * bz) * g.ir * ib2 - gbt * bz * 2.0 * ib3);
        vdy = vdp * (-((dbz_dx + bz * g.ir) * ib2) + gbr * bz * 2.0 * ib3);
    } else {
        vdx = vdp * (dbz_dy * ib2 - 2.0 * bz * db_dy * ib3);
        vdy = vdp * (-(dbz_dx * ib2) + 2.0 * bz * db_dx * ib3);
    }
    double vdz = 0.0;
    if (pr->check_drift_2d) {
        const double dbx_dy = f[21], dby_dx = f[23];
        if (c->sph)
            vdz = vdp * ((dby_dx + by * g.ir - dbx_dy * g.ir) * ib2 -
                         (gbr * by - gbt * bx * g.ir) * 2.0 * ib3);
        else
            vdz = vdp * ((dby_dx - dbx_dy) * ib2 - 2.0 * (by * db_dx - bx * db_dy) * ib3);
    }
    double dx_dt, dy_dt, dz_dt, divv;
    if (c->sph) {
        dx_dt = vx + vdx + kap[K_DKXX_DX] +
                (2.0 * kap[K_KXX] + kap[K_DKXY_DY] + kap[K_KXY] * g.cot_theta) * g.ir;
        dy_dt = (vy + vdy + kap[K_DKXY_DX]) * g.ir +
                (kap[K_KXY] + kap[K_DKYY_DY] + kap[K_KYY] * g.cot_theta) * g.ir2;
        dz_dt = vdz * g.istheta * g.ir;
        divv = dvx_dx + (2.0 * vx + dvy_dy + vy * g.ctheta * g.istheta) * g.ir;
    } else {
        dx_dt = vx + vdx + kap[K_DKXX_DX] + kap[K_DKXY_DY];
        dy_dt = vy + vdy + kap[K_DKXY_DX] + kap[K_DKYY_DY];
        dz_dt = vdz;
        divv = dvx_dx + dvy_dy;
    }
    double dp_dt = -(s->p * divv / 3.0);
    const double dpp = dpp_terms(pr, s->p, f, kap, b, divv, &dp_dt);
    const double skpara = kap[K_SKPARA], skperp = kap[K_SKPERP];
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double a = 0.5 * dxm / skpara, m = a * a;
            if (c->sph) {
                a = 0.5 * dym * s->x / skpara; if (a * a < m) m = a * a;
                a = sk / dx_dt; if (a * a < m) m = a * a;
                a = sk * g.ir / dy_dt; if (a * a < m) m = a * a;
            } else {
                a = 0.5 * dym / skpara; if (a * a < m) m = a * a;
                a = sk / dx_dt; if (a * a < m) m = a * a;
                a = sk / dy_dt; if (a * a < m) m = a * a;
            }
            a = (double)0.1f * s->p / fabs(dp_dt); if (a < m) m = a;
            s->dt = m;
        } else {
            s->dt = c->dt_min;
        }
        if (s->dt < c->dt_min) s->dt = c->dt_min;
        if (s->dt > c->dt_max) s->dt = c->dt_max;
    }
    const double sdt = sqrt(s->dt);
    double r[4];
    push_noise(c, s, r);
    double dX, dY;
    if (c->sph) {
        double nx, ny;
        spherical_noise_2d(kap, &g, r[0], r[1], sdt, &nx, &ny);
        dX = dx_dt * s->dt + nx;
        dY = dy_dt * s->dt + ny;
    } else {
        const double skpp = kap[K_SKPARA_PERP];
        dX = dx_dt * s->dt + r[0] * skperp * sdt + r[2] * skpp * sdt * bx * ib;
        dY = dy_dt * s->dt + r[1] * skperp * sdt + r[2] * skpp * sdt * by * ib;
    }
    const double dZ = dz_dt * s->dt;
    s->x = s->x + dX;
    s->y = s->y + dY;
    s->z = s->z + dZ;
    s->t = s->t + s->dt;
    /* deltaz is local to push_particle_2d: the mover's deltaz stays 0, so an
     * undone push keeps its out-of-plane drift. */
    d[0] = dX; d[1] = dY; d[2] = 0.0; d[4] = 0.0; d[5] = 0.0;
    push_momentum(c, s, dp_dt, dpp, sdt, r[3], &d[3]);
}

/* push_particle_3d: particle_module.f90:4625-4907, Cartesian and spherical
 * (x = r, y = theta, z = phi), without the acceleration surfaces. */
static void push_3d(const mover_ctx *c, ptl_state *s, const double *f, const double *kap,
                    const cell_size *cs, int fixed_dt, double d[6])
{
    const orc_params *pr = c->pr;
    const double vx = f[0], vy = f[1], vz = f[2], bx = f[4], by = f[5], bz = f[6];
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    const double bxn = bx * ib, byn = by * ib, bzn = bz * ib;
    const double bxyn = sqrt(bxn * bxn + byn * byn);
    const double ibxyn = (bxyn < DBL_EPSILON) ? 0.0 : 1.0 / bxyn;
    const double dvx_dx = f[8], dvy_dy = f[12], dvz_dz = f[16];
    const double dxm = cs->dxm, dym = cs->dym, dzm = cs->dzm;
    sph_terms g = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (c->sph) g = spherical_terms(s);
    const double dbx_dy = f[21], dbx_dz = f[22], dby_dx = f[23], dby_dz = f[25];
    const double dbz_dx = f[26], dbz_dy = f[27];
    const double db_dx = f[29], db_dy = f[30], db_dz = f[31];
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor(pr, s->p);
    double vdx, vdy, vdz;
    if (c->sph) {
        const double gbr = db_dx, gbt = db_dy * g.ir, gbp = db_dz * g.ir * g.istheta;
        vdx = vdp * ((dbz_dy + bz * g.ctheta * g.istheta - dby_dz * g.istheta) * g.ir * ib2 -
                     (gbt * bz - gbp * by) * 2.0 * ib3);
        vdy = vdp * ((dbx_dz * g.istheta * g.ir - dbz_dx - bz * g.ir) * ib2 -
                     (gbp * bx - gbr * bz) * 2.0 * ib3);
        vdz = vdp * ((dby_dx + by * g.ir - dbx_dy * g.ir) * ib2 -
                     (gbr * by - gbt * bx) * 2.0 * ib3);
    } else {
        vdx = vdp * ((dbz_dy - dby_dz) * ib2 - 2.0 * (bz * db_dy - by * db_dz) * ib3);
        vdy = vdp * ((dbx_dz - dbz_dx) * ib2 - 2.0 * (bx * db_dz - bz * db_dx) * ib3);
        vdz = vdp * ((dby_dx - dbx_dy) * ib2 - 2.0 * (by * db_dx - bx * db_dy) * ib3);
    }
    double dx_dt, dy_dt, dz_dt, divv;
    if (c->sph) {
        dx_dt = vx + vdx + kap[K_DKXX_DX] +
                (2.0 * kap[K_KXX] + kap[K_DKXY_DY] + kap[K_KXY] * g.ctheta * g.istheta +
                 kap[K_DKXZ_DZ] * g.istheta) * g.ir;
        dy_dt = (vy + vdy + kap[K_DKXY_DX]) * g.ir +
                (kap[K_KXY] + kap[K_DKYY_DY] + kap[K_KYY] * g.ctheta * g.istheta +
                 kap[K_DKYZ_DZ] * g.istheta) * g.ir2;
        dz_dt = (vz + vdz + kap[K_DKXZ_DX]) * g.istheta * g.ir +
                (kap[K_KXZ] + kap[K_DKYZ_DY] + kap[K_DKZZ_DZ] * g.istheta) * g.istheta * g.ir2;
        divv = dvx_dx + (2.0 * vx + dvy_dy + vy * g.ctheta * g.istheta + dvz_dz * g.istheta) * g.ir;
    } else {
        dx_dt = vx + vdx + kap[K_DKXX_DX] + kap[K_DKXY_DY] + kap[K_DKXZ_DZ];
        dy_dt = vy + vdy + kap[K_DKXY_DX] + kap[K_DKYY_DY] + kap[K_DKYZ_DZ];
        dz_dt = vz + vdz + kap[K_DKXZ_DX] + kap[K_DKYZ_DY] + kap[K_DKZZ_DZ];
        divv = dvx_dx + dvy_dy + dvz_dz;
    }
    double dp_dt = -(s->p * divv / 3.0);
    const double dpp = dpp_terms(pr, s->p, f, kap, b, divv, &dp_dt);
    const double skpara = kap[K_SKPARA], skperp = kap[K_SKPERP];
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dy_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double a = 0.5 * dxm / skpara, m = a * a;
            /* include_3rd_dim keeps the 2D limits (:4141-4175) */
            const int z = !c->i3;
            if (c->sph) {
                a = 0.5 * dym * s->x / skpara; if (a * a < m) m = a * a;
                if (z) { a = 0.5 * dzm * s->x * sin(s->y) / skpara; if (a * a < m) m = a * a; }
                a = sk / dx_dt; if (a * a < m) m = a * a;
                a = sk * g.ir / dy_dt; if (a * a < m) m = a * a;
                if (z) { a = sk * g.ir * g.istheta / dz_dt; if (a * a < m) m = a * a; }
            } else {
                a = 0.5 * dym / skpara; if (a * a < m) m = a * a;
                if (z) { a = 0.5 * dzm / skpara; if (a * a < m) m = a * a; }
                a = sk / dx_dt; if (a * a < m) m = a * a;
                a = sk / dy_dt; if (a * a < m) m = a * a;
                if (z) { a = sk / dz_dt; if (a * a < m) m = a * a; }
            }
            a = (double)0.1f * s->p / fabs(dp_dt); if (a < m) m = a;
            s->dt = m;
        } else {
            s->dt = c->dt_min;
        }
        if (s->dt < c->dt_min) s->dt = c->dt_min;
        if (s->dt > c->dt_max) s->dt = c->dt_max;
    }
    const double sdt = sqrt(s->dt);
    double r[4];
    push_noise(c, s, r);
    double dX, dY, dZ;
    if (c->sph) {
        double q[6];
        spherical_noise_3d(kap, &g, 0, q);
        dX = dx_dt * s->dt + (q[0] * r[0] + q[1] * r[1] + q[2] * r[2]) * sdt;
        dY = dy_dt * s->dt + (q[3] * r[1] + q[4] * r[2]) * sdt;
        dZ = dz_dt * s->dt + q[5] * r[2] * sdt;
    } else {
        dX = dx_dt * s->dt +
            (bxn * skpara * r[0] - bxn * bzn * skperp * ibxyn * r[1] - byn * skperp * ibxyn * r[2]) * sdt;
        dY = dy_dt * s->dt +
            (byn * skpara * r[0] - byn * bzn * skperp * ibxyn * r[1] + bxn * skperp * ibxyn * r[2]) * sdt;
        dZ = dz_dt * s->dt + (bzn * skpara * r[0] + bxyn * skperp * r[1]) * sdt;
    }
    s->x = s->x + dX;
    s->y = s->y + dY;
    s->z = s->z + dZ;
    s->t = s->t + s->dt;
    d[0] = dX; d[1] = dY; d[2] = dZ; d[4] = 0.0; d[5] = 0.0;
    push_momentum(c, s, dp_dt, dpp, sdt, r[3], &d[3]);
}

/* ------------------------------------------------------------------------ */
/* Focused transport.                                                        */
/* ------------------------------------------------------------------------ */
/* calc_duu: particle_module.f90:3116-3155 without delta-B or correlation   */
/* length.                                                                   */
static void calc_duu(const orc_params *pr, const ptl_state *s, double b, const double *aux,
                     double div_bnorm, double divv, double bb_gradv, double bv_gradv,
                     double mu2, double *dmu_dt, double *duu, double *duu_du)
{
    double dm = s->v * div_bnorm + s->mu * divv - 3.0 * s->mu * bb_gradv - 2.0 * bv_gradv / s->v;
    dm = dm * (1.0 - mu2) * 0.5;
    const double h0 = (double)0.2f;
    const double dtmp = pow(fabs(s->mu), pr->gamma_turb - 1.0) + h0;
    double u = pr->duu0 * (1.0 - mu2) * dtmp;
    double ud;
    if (s->mu > 0.0)
        ud = pr->duu0 * (-(2.0 * s->mu * dtmp) + (1.0 - mu2) * pow(fabs(s->mu), pr->gamma_turb - 2.0));
    else if (s->mu < 0.0)
        ud = pr->duu0 * (-(2.0 * s->mu * dtmp) - (1.0 - mu2) * pow(fabs(s->mu), pr->gamma_turb - 2.0));
    else
        ud = 0.0;
    double norm = 1.0;
    if (pr->mag_dependency == 1) norm = norm * pow(b, 2.0 - pr->gamma_turb);
    if (pr->deltab_flag && aux) norm = norm * aux[0];
    if (pr->correlation_flag && aux) norm = norm * pow(aux[8], 1.0 - pr->gamma_turb);
    if (pr->momentum_dependency == 1) norm = norm * pow(s->p / pr->p0, pr->gamma_turb - 1.0);
    ud = ud * norm;
    u = u * norm;
    *dmu_dt = dm + ud;
    *duu = u;
    *duu_du = ud;
}

/* 1 / pcharge is single precision in the focused-transport pushes. */
static double vdrift_prefactor_ft(const orc_params *pr, double p)
{
    const float q = 1.0f / (float)pr->charge;
    const double t1 = pr->drift1 * pr->p0 / p;
    const double t2 = pr->drift2 * (pr->p0 * pr->p0) / (p * p);
    return (double)q / sqrt(t1 * t1 + t2 * t2);
}

/* The tail shared by push_particle_2d_ft and push_particle_3d_ft: the
 * momentum, speed and pitch-angle increments, the mu_max clamp, the
 * acceleration-region mask and the 0.25 p0 floor (:3920-3963,
 * :5280-5323).  r[2] drives momentum diffusion, r[3] pitch-angle. */
static void push_ft_tail(const mover_ctx *c, ptl_state *s, double dX, double dY, double dZ,
                         double dp_dt, double dpp, double dmu_dt, double duu, double sdt,
                         const double r[4], double d[6])
{
    double dP = dp_dt * s->dt + r[2] * sqrt(2.0 * dpp) * sdt;
    double dV = s->v * dP / s->p;
    double dMu = dmu_dt * s->dt + r[3] * sqrt(2.0 * duu) * sdt;
    s->x = s->x + dX;
    s->y = s->y + dY;
    s->z = s->z + dZ;
    s->mu = s->mu + dMu;
    s->t = s->t + s->dt;
    const double mu_max = (double)0.99f;
    if (s->mu > mu_max) {
        dMu = mu_max - (s->mu - dMu);
        s->mu = mu_max;
    } else if (s->mu < -mu_max) {
        dMu = -mu_max - (s->mu - dMu);
        s->mu = -mu_max;
    }
    if (c->pr->acc_region_flag == 1) {
        if (in_acc_region(c, s)) {
            s->p = s->p + dP;
            s->v = s->v + dV;
        } else {
            dP = 0.0;
            dV = 0.0;
        }
    } else {
        s->p = s->p + dP;
        s->v = s->v + dV;
    }
    const double pfloor = 0.25 * c->pr->p0;
    if (s->p < pfloor) {
        s->v = s->v - dV;
        dV = s->v * 0.25 * c->pr->p0 / s->p - s->v;
        s->v = s->v + dV;
        s->p = s->p - dP;
        dP = pfloor - s->p;
        s->p = pfloor;
    }
    d[0] = dX; d[1] = dY; d[2] = dZ; d[3] = dP; d[4] = dV; d[5] = dMu;
}

/* The adaptive time step of the focused-transport pushes (:3850-3905,
 * :5170-5230): the minimum of the cell-crossing, drift, momentum and
 * pitch-angle limits, dt_min when any first-order rate is exactly 0.  In
 * spherical coordinates the theta and phi limits carry r and r sin(theta). */
static void ft_time_step(const mover_ctx *c, ptl_state *s, const double *kap, int ndim,
                         const cell_size *cs, const sph_terms *g, double dx_dt, double dy_dt,
                         double dz_dt, double dp_dt, double dmu_dt, double duu)
{
    const int rates_nonzero = (dx_dt != 0.0) && (dy_dt != 0.0) && (ndim < 3 || dz_dt != 0.0) &&
                              (dp_dt != 0.0) && (dmu_dt != 0.0);
    if (rates_nonzero) {
        const double sk = (kap[K_SKPERP] > 0.0) ? kap[K_SKPERP] : kap[K_SKPARA];
        double a = 0.5 * cs->dxm / sk, m = a * a;
        if (c->sph) {
            a = 0.5 * cs->dym * s->x / sk; if (a * a < m) m = a * a;
            if (ndim == 3) { a = 0.5 * cs->dzm * s->x * sin(s->y) / sk; if (a * a < m) m = a * a; }
            a = sk / dx_dt; if (a * a < m) m = a * a;
            a = sk * g->ir / dy_dt; if (a * a < m) m = a * a;
            if (ndim == 3) { a = sk * g->ir * g->istheta / dz_dt; if (a * a < m) m = a * a; }
        } else {
            a = 0.5 * cs->dym / sk; if (a * a < m) m = a * a;
            if (ndim == 3) { a = 0.5 * cs->dzm / sk; if (a * a < m) m = a * a; }
            a = sk / dx_dt; if (a * a < m) m = a * a;
            a = sk / dy_dt; if (a * a < m) m = a * a;
            if (ndim == 3) { a = sk / dz_dt; if (a * a < m) m = a * a; }
        }
        a = (double)0.1f * s->p / fabs(dp_dt); if (a < m) m = a;
        a = (double)0.1f / fabs(dmu_dt); if (a < m) m = a;
        a = 2.0 * duu / (dmu_dt * dmu_dt); if (a < m) m = a;
        s->dt = m;
    } else {
        s->dt = c->dt_min;
    }
    if (s->dt < c->dt_min) s->dt = c->dt_min;
    if (s->dt > c->dt_max) s->dt = c->dt_max;
}

/* push_particle_2d_ft: particle_module.f90:3626-3964, Cartesian and
 * spherical. */
static void push_2d_ft(const mover_ctx *c, ptl_state *s, const double *f, const double *aux,
                       const double *kap, const cell_size *cs, int fixed_dt, double d[6])
{
    const orc_params *pr = c->pr;
    const double vx = f[0], vy = f[1], vz = f[2], bx = f[4], by = f[5], bz = f[6];
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    sph_terms g = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (c->sph) g = spherical_terms(s);
    const double dbx_dx = f[20], dbx_dy = f[21], dby_dx = f[23], dby_dy = f[24];
    const double dbz_dx = f[26], dbz_dy = f[27], db_dx = f[29], db_dy = f[30];
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor_ft(pr, s->p);
    const double mu2 = s->mu * s->mu;
    const double muf1 = 0.5 * (1.0 - mu2);
    const double muf2 = 0.5 * (3.0 * mu2 - 1.0);
    double kx, ky, kz, bdot_curvb, vdx, vdy, gbr = 0.0, gbt = 0.0;
    if (c->sph) {
        const double ir = g.ir, cot = g.cot_theta;
        gbr = db_dx;
        gbt = db_dy * ir;
        kx = bx * dbx_dx + by * dbx_dy * ir - (by * by + bz * bz) * ir;
        ky = bx * dby_dx + by * dby_dy * ir + (bx * by - cot * (bz * bz)) * ir;
        kz = bx * dbz_dx + by * dbz_dy * ir + (bx * bz + cot * by * bz) * ir;
        bdot_curvb = bx * (dbz_dy + cot * bz) * ir + by * (-dbz_dx - bz * ir) +
                     bz * (dby_dx + by * ir - dbx_dy * ir);
        vdx = vdp * (muf1 * (-(bz * gbt)) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                     muf1 * bx * bdot_curvb * ib3);
        vdy = vdp * (muf1 * (bz * gbr) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                     muf1 * by * bdot_curvb * ib3);
    } else {
        kx = bx * dbx_dx + by * dbx_dy;
        ky = bx * dby_dx + by * dby_dy;
        kz = bx * dbz_dx + by * dbz_dy;
        bdot_curvb = bx * dbz_dy - by * dbz_dx + bz * (dby_dx - dbx_dy);
        vdx = vdp * (muf1 * (-(bz * db_dy)) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                     muf1 * bx * bdot_curvb * ib3);
        vdy = vdp * (muf1 * (bz * db_dx) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                     muf1 * by * bdot_curvb * ib3);
    }
    double vdz = 0.0;
    if (pr->check_drift_2d) {
        if (c->sph)
            vdz = vdp * (muf1 * (bx * gbt - by * gbr) * ib2 + mu2 * (bx * ky - by * kx) * ib3 +
                         muf1 * bz * bdot_curvb * ib3);
        else
            vdz = vdp * (muf1 * (bx * db_dy - by * db_dx) * ib2 + mu2 * (bx * ky - by * kx) * ib3 +
                         muf1 * bz * bdot_curvb * ib3);
    }
    double vbx = s->v * s->mu * ib;
    const double vby = vbx * by;
    vbx = vbx * bx;
    const double dvx_dx = f[8], dvx_dy = f[9], dvy_dx = f[11], dvy_dy = f[12];
    const double dvz_dx = f[14], dvz_dy = f[15];
    double dx_dt, dy_dt, dz_dt, divv, bb_gradv, bv_gradv;
    if (c->sph) {
        const double ir = g.ir, cot = g.cot_theta;
        dx_dt = vx + vdx + vbx + kap[K_DKXX_DX] +
                (2.0 * kap[K_KXX] + kap[K_DKXY_DY] + kap[K_KXY] * cot) * ir;
        dy_dt = (vy + vdy + vby + kap[K_DKXY_DX]) * ir +
                (kap[K_KXY] + kap[K_DKYY_DY] + kap[K_KYY] * cot) * g.ir2;
        dz_dt = vdz * g.istheta * ir;
        divv = dvx_dx + (2.0 * vx + dvy_dy + vy * cot) * ir;
        bb_gradv = (bx * bx * dvx_dx + bx * by * dvx_dy * ir - bx * (by * vy + bz * vz) * ir +
                    by * bx * dvy_dx + by * by * dvy_dy * ir + by * (by * vx - cot * bz * vz) * ir +
                    bz * bx * dvz_dx + bz * by * dvz_dy * ir + (bz * bz) * (vx + cot * vy) * ir) * ib2;
        bv_gradv = (bx * vx * dvx_dx + bx * vy * dvx_dy * ir - bx * (vy * vy + vz * vz) * ir +
                    by * vx * dvy_dx + by * vy * dvy_dy * ir + by * (vy * vx - cot * vz * vz) * ir +
                    bz * vx * dvz_dx + bz * vy * dvz_dy * ir + bz * vz * (vx + cot * vy) * ir) * ib;
    } else {
        dx_dt = vx + vdx + vbx + kap[K_DKXX_DX] + kap[K_DKXY_DY];
        dy_dt = vy + vdy + vby + kap[K_DKXY_DX] + kap[K_DKYY_DY];
        dz_dt = vdz;
        divv = dvx_dx + dvy_dy;
        bb_gradv = (bx * (bx * dvx_dx + by * dvx_dy) +
                    by * (bx * dvy_dx + by * dvy_dy) +
                    bz * (bx * dvz_dx + by * dvz_dy)) * ib2;
        bv_gradv = (bx * (vx * dvx_dx + vy * dvx_dy) +
                    by * (vx * dvy_dx + vy * dvy_dy) +
                    bz * (vx * dvz_dx + vy * dvz_dy)) * ib;
    }
    const double acc_rate = -(muf1 * divv + muf2 * bb_gradv + s->mu * bv_gradv / s->v);
    double dp_dt = s->p * acc_rate;
    const double dpp = dpp_terms(pr, s->p, f, kap, b, divv, &dp_dt);
    const double div_bnorm = c->sph ? -((bx * db_dx + by * db_dy * g.ir) * ib2)
                                    : -((bx * db_dx + by * db_dy) * ib2);
    double dmu_dt, duu, duu_du;
    calc_duu(pr, s, b, aux, div_bnorm, divv, bb_gradv, bv_gradv, mu2, &dmu_dt, &duu, &duu_du);
    if (!fixed_dt) ft_time_step(c, s, kap, 2, cs, &g, dx_dt, dy_dt, dz_dt, dp_dt, dmu_dt, duu);
    const double sdt = sqrt(s->dt);
    double r[4];
    push_noise(c, s, r);
    double dX, dY;
    if (c->sph) {
        double nx, ny;
        spherical_noise_2d(kap, &g, r[0], r[1], sdt, &nx, &ny);
        dX = dx_dt * s->dt + nx;
        dY = dy_dt * s->dt + ny;
    } else {
        const double bxn = bx * ib, byn = by * ib, bzn = bz * ib;
        const double ibxyn = 1.0 / sqrt(bxn * bxn + byn * byn);
        const double skperp = kap[K_SKPERP];
        dX = dx_dt * s->dt + skperp * ibxyn * sdt * (-(bxn * bzn * r[0]) - by * r[1]);
        dY = dy_dt * s->dt + skperp * ibxyn * sdt * (-(byn * bzn * r[0]) + bx * r[1]);
    }
    const double dZ = dz_dt * s->dt;
    push_ft_tail(c, s, dX, dY, dZ, dp_dt, dpp, dmu_dt, duu, sdt, r, d);
    d[2] = 0.0;   /* deltaz is local to push_particle_2d_ft, as in push_2d */
}

/* push_particle_3d_ft: particle_module.f90:4930-5324, Cartesian and
 * spherical.  The spherical position noise draws a third number (ran3);
 * it comes from the push's extra Philox block. */
static void push_3d_ft(const mover_ctx *c, ptl_state *s, const double *f, const double *aux,
                       const double *kap, const cell_size *cs, int fixed_dt, double d[6])
{
    const orc_params *pr = c->pr;
    const double vx = f[0], vy = f[1], vz = f[2], bx = f[4], by = f[5], bz = f[6];
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double ib = (b < DBL_EPSILON) ? 0.0 : 1.0 / b;
    const double bxn = bx * ib, byn = by * ib, bzn = bz * ib;
    const double bxyn = sqrt(bxn * bxn + byn * byn);
    const double ibxyn = (bxyn < DBL_EPSILON) ? 0.0 : 1.0 / bxyn;
    sph_terms g = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (c->sph) g = spherical_terms(s);
    const double dbx_dx = f[20], dbx_dy = f[21], dbx_dz = f[22];
    const double dby_dx = f[23], dby_dy = f[24], dby_dz = f[25];
    const double dbz_dx = f[26], dbz_dy = f[27], dbz_dz = f[28];
    const double db_dx = f[29], db_dy = f[30], db_dz = f[31];
    const double ib2 = ib * ib;
    const double ib3 = ib * ib2;
    const double vdp = vdrift_prefactor_ft(pr, s->p);
    const double mu2 = s->mu * s->mu;
    const double muf1 = 0.5 * (1.0 - mu2);
    const double muf2 = 0.5 * (3.0 * mu2 - 1.0);
    double kx, ky, kz, bdot_curvb, vdx, vdy, vdz;
    if (c->sph) {
        const double ir = g.ir, ist = g.istheta, cot = g.cot_theta;
        const double gbr = db_dx, gbt = db_dy * ir, gbp = db_dz * ir * ist;
        kx = bx * dbx_dx + ir * (by * dbx_dy + bz * dbx_dz * ist - (by * by + bz * bz));
        ky = bx * dby_dx + ir * (by * dby_dy + bz * dby_dz * ist + (bx * by - cot * (bz * bz)));
        kz = bx * dbz_dx + ir * (by * dbz_dy + bz * dbz_dz * ist + (bx * bz + cot * by * bz));
        bdot_curvb = bx * (dbz_dy + cot * bz - dby_dz * ist) * ir +
                     by * (dbx_dz * ist * ir - dbz_dx - bz * ir) +
                     bz * (dby_dx + by * ir - dbx_dy * ir);
        vdx = vdp * (muf1 * (by * gbp - bz * gbt) * ib2 + mu2 * (by * kz - bz * ky) * ib3 +
                     muf1 * bx * bdot_curvb * ib3);
        vdy = vdp * (muf1 * (bz * gbr - bx * gbp) * ib2 + mu2 * (bz * kx - bx * kz) * ib3 +
                     muf1 * by * bdot_curvb * ib3);
        vdz = vdp * (muf1 * (bx * gbt - by * gbr) * ib2 + mu2 * (bx * ky - by * kx) * ib3 +
                     muf1 * bz * bdot_curvb * ib3);
    } else {
        kx = bx * dbx_dx + by * dbx_dy + bz * dbx_dz;
        ky = bx * dby_dx + by * dby_dy + bz * dby_dz;
        kz = bx * dbz_dx + by * dbz_dy + bz * dbz_dz;
        bdot_curvb = bx * (dbz_dy - dby_dz) + by * (dbx_dz - dbz_dx) + bz * (dby_dx - dbx_dy);
        vdx = vdp * (muf1 * (by * db_dz - bz * db_dy) * ib2 +
                     mu2 * (by * kz - bz * ky) * ib3 + muf1 * bx * bdot_curvb * ib3);
        vdy = vdp * (muf1 * (bz * db_dx - bx * db_dz) * ib2 +
                     mu2 * (bz * kx - bx * kz) * ib3 + muf1 * by * bdot_curvb * ib3);
        vdz = vdp * (muf1 * (bx * db_dy - by * db_dx) * ib2 +
                     mu2 * (bx * ky - by * kx) * ib3 + muf1 * bz * bdot_curvb * ib3);
    }
    double vbx = s->v * s->mu * ib;
    const double vby = vbx * by;
    const double vbz = vbx * bz;
    vbx = vbx * bx;
    const double dvx_dx = f[8], dvx_dy = f[9], dvx_dz = f[10];
    const double dvy_dx = f[11], dvy_dy = f[12], dvy_dz = f[13];
    const double dvz_dx = f[14], dvz_dy = f[15], dvz_dz = f[16];
    double dx_dt, dy_dt, dz_dt, divv, bb_gradv, bv_gradv;
    if (c->sph) {
        const double ir = g.ir, ist = g.istheta, cot = g.cot_theta;
        if (c->i3) {
            /* push_particle_2d_include_3rd_ft (:4417-4425) */
            dx_dt = vx + vbx + vdx + kap[K_DKXX_DX] +
                    (2.0 * kap[K_KXX] + kap[K_DKXY_DY] + kap[K_KXY] * cot) * ir;
        } else {
            dx_dt = vx + vbx + vdx + kap[K_DKXX_DX] +
                    (2.0 * kap[K_KXX] + kap[K_DKXY_DY] + kap[K_KXY] * g.ctheta * ist +
                     kap[K_DKXZ_DZ] * ist) * ir;
        }
        if (c->i3)
            dy_dt = (vy + vby + vdy + kap[K_DKXY_DX]) * ir +
                    (kap[K_KXY] + kap[K_DKYY_DY] + kap[K_KYY] * cot) * g.ir2;
        else
            dy_dt = (vy + vby + vdy + kap[K_DKXY_DX]) * ir +
                    (kap[K_KXY] + kap[K_DKYY_DY] + kap[K_KYY] * g.ctheta * ist +
                     kap[K_DKYZ_DZ] * ist) * g.ir2;
        dz_dt = (vz + vbz + vdz + kap[K_DKXZ_DX]) * ist * ir +
                (kap[K_KXZ] + kap[K_DKYZ_DY] + kap[K_DKZZ_DZ] * ist) * ist * g.ir2;
        divv = dvx_dx + (2.0 * vx + dvy_dy + vy * cot + dvz_dz * ist) * ir;
        const double dtmp = ist * ir;
        bb_gradv = (bx * bx * dvx_dx + bx * by * dvx_dy * ir + bx * bz * dvx_dz * dtmp -
                    bx * (by * vy + bz * vz) * ir +
                    by * bx * dvy_dx + by * by * dvy_dy * ir + by * bz * dvy_dz * dtmp +
                    by * (by * vx - cot * bz * vz) * ir +
                    bz * bx * dvz_dx + bz * by * dvz_dy * ir + bz * bz * dvz_dz * dtmp +
                    (bz * bz) * (vx + cot * vy) * ir) * ib2;
        bv_gradv = (bx * vx * dvx_dx + bx * vy * dvx_dy * ir + bx * vz * dvx_dz * dtmp -
                    bx * (vy * vy + vz * vz) * ir +
                    by * vx * dvy_dx + by * vy * dvy_dy * ir + by * vz * dvy_dz * dtmp +
                    by * (vy * vx - cot * vz * vz) * ir +
                    bz * vx * dvz_dx + bz * vy * dvz_dy * ir + bz * vz * dvz_dz * dtmp +
                    bz * vz * (vx + cot * vy) * ir) * ib;
    } else {
        dx_dt = vx + vbx + vdx + kap[K_DKXX_DX] + kap[K_DKXY_DY] + kap[K_DKXZ_DZ];
        dy_dt = vy + vby + vdy + kap[K_DKXY_DX] + kap[K_DKYY_DY] + kap[K_DKYZ_DZ];
        dz_dt = vz + vbz + vdz + kap[K_DKXZ_DX] + kap[K_DKYZ_DY] + kap[K_DKZZ_DZ];
        divv = dvx_dx + dvy_dy + dvz_dz;
        bb_gradv = (bx * (bx * dvx_dx + by * dvx_dy + bz * dvx_dz) +
                    by * (bx * dvy_dx + by * dvy_dy + bz * dvy_dz) +
                    bz * (bx * dvz_dx + by * dvz_dy + bz * dvz_dz)) * ib2;
        bv_gradv = (bx * (vx * dvx_dx + vy * dvx_dy + vz * dvx_dz) +
                    by * (vx * dvy_dx + vy * dvy_dy + vz * dvy_dz) +
                    bz * (vx * dvz_dx + vy * dvz_dy + vz * dvz_dz)) * ib;
    }
    const double acc_rate = -(muf1 * divv + muf2 * bb_gradv + s->mu * bv_gradv / s->v);
    double dp_dt = s->p * acc_rate;
    const double dpp = dpp_terms(pr, s->p, f, kap, b, divv, &dp_dt);
    const double div_bnorm =
        c->sph ? -((bx * db_dx + by * db_dy * g.ir + bz * db_dz * g.ir * g.istheta) * ib2)
               : -((bx * db_dx + by * db_dy + bz * db_dz) * ib2);
    double dmu_dt, duu, duu_du;
    calc_duu(pr, s, b, aux, div_bnorm, divv, bb_gradv, bv_gradv, mu2, &dmu_dt, &duu, &duu_du);
    /* include_3rd_dim keeps the 2D limits (:4481-4532) */
    if (!fixed_dt)
        ft_time_step(c, s, kap, c->i3 ? 2 : 3, cs, &g, dx_dt, dy_dt, dz_dt, dp_dt, dmu_dt, duu);
    const double sdt = sqrt(s->dt);
    double r[6];
    push_noise_n(c, s, r, c->sph);
    double dX, dY, dZ;
    if (c->sph) {
        double q[6];
        /* the include_3rd_dim variant has no radicand guards (:4544-4560) */
        spherical_noise_3d(kap, &g, !c->i3, q);
        dX = dx_dt * s->dt + (q[0] * r[0] + q[1] * r[1] + q[2] * r[4]) * sdt;
        dY = dy_dt * s->dt + (q[3] * r[1] + q[4] * r[4]) * sdt;
        dZ = dz_dt * s->dt + q[5] * r[4] * sdt;
    } else {
        const double skperp = kap[K_SKPERP];
        dX = dx_dt * s->dt +
            (-(bxn * bzn * skperp * ibxyn * r[0]) - byn * skperp * ibxyn * r[1]) * sdt;
        dY = dy_dt * s->dt +
            (-(byn * bzn * skperp * ibxyn * r[0]) + bxn * skperp * ibxyn * r[1]) * sdt;
        dZ = dz_dt * s->dt + bxyn * skperp * r[0] * sdt;
    }
    push_ft_tail(c, s, dX, dY, dZ, dp_dt, dpp, dmu_dt, duu, sdt, r, d);
}

/* push_particle_1d: particle_module.f90:2993-3110, Cartesian or spherical
 * (x = r).  r[0] drives x, r[3] momentum. */
static void push_1d(const mover_ctx *c, ptl_state *s, const double *f, const double *kap,
                    const cell_size *cs, int fixed_dt, double d[6])
{
    const orc_params *pr = c->pr;
    const double vx = f[0], bx = f[4], by = f[5], bz = f[6];
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double dvx_dx = f[8];
    double dx_dt, divv;
    if (c->sph) {
        dx_dt = vx + kap[K_DKXX_DX] + 2.0 * kap[K_KXX] / s->x;
        divv = dvx_dx + 2.0 * vx / s->x;
    } else {
        dx_dt = vx + kap[K_DKXX_DX];
        divv = dvx_dx;
    }
    double dp_dt = -(s->p * divv / 3.0);
    const double dpp = dpp_terms(pr, s->p, f, kap, b, divv, &dp_dt);
    const double skpara = kap[K_SKPARA], skperp = kap[K_SKPERP];
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dp_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double a = 0.5 * cs->dxm / skpara, m = a * a;
            a = sk / dx_dt; if (a * a < m) m = a * a;
            a = (double)0.1f * s->p / fabs(dp_dt); if (a < m) m = a;
            s->dt = m;
        } else {
            s->dt = c->dt_min;
        }
        if (s->dt < c->dt_min) s->dt = c->dt_min;
        if (s->dt > c->dt_max) s->dt = c->dt_max;
    }
    const double sdt = sqrt(s->dt);
    double r[4];
    push_noise(c, s, r);
    const double dX = dx_dt * s->dt + r[0] * skpara * sdt;
    s->x = s->x + dX;
    s->t = s->t + s->dt;
    d[0] = dX; d[1] = 0.0; d[2] = 0.0; d[4] = 0.0; d[5] = 0.0;
    push_momentum(c, s, dp_dt, dpp, sdt, r[3], &d[3]);
}

/* push_particle_1d_ft: particle_module.f90:3174-3357.  The reference
 * computes the x rate into dv_dt and then reads dx_dt, which it never
 * sets; the rate it computed is used here.  r[0] drives x, r[2] momentum,
 * r[3] pitch angle. */
static void push_1d_ft(const mover_ctx *c, ptl_state *s, const double *f, const double *aux,
                       const double *kap, const cell_size *cs, int fixed_dt, double d[6])
{
    const orc_params *pr = c->pr;
    const double vx = f[0], vy = f[1], vz = f[2], bx = f[4], by = f[5], bz = f[6];
    const double b = sqrt(bx * bx + by * by + bz * bz);
    const double dvx_dx = f[8], dvy_dx = f[11], dvz_dx = f[14];
    double dx_dt, divv, bb_gradv, bv_gradv;
    if (c->sph) {
        const double ir = 1.0 / s->x;
        dx_dt = vx + s->v * s->mu + kap[K_DKXX_DX] + 2.0 * kap[K_KXX] * ir;
        const double cot = 1.0 / tan(s->y);
        divv = dvx_dx + 2.0 * vx * ir;
        bb_gradv = (bx * bx * dvx_dx - bx * (by * vy + bz * vz) * ir + by * bx * dvy_dx +
                    by * (by * vx - cot * bz * vz) * ir + bz * bx * dvz_dx +
                    (bz * bz) * (vx + cot * vy) * ir) / (b * b);
        bv_gradv = (bx * vx * dvx_dx - bx * (vy * vy + vz * vz) * ir + by * vx * dvy_dx +
                    by * (vy * vx - cot * vz * vz) * ir + bz * vx * dvz_dx +
                    bz * vz * (vx + cot * vy) * ir) / (b * b);
    } else {
        dx_dt = vx + s->v * s->mu + kap[K_DKXX_DX];
        divv = dvx_dx;
        bb_gradv = (bx * bx * dvx_dx + by * bx * dvy_dx + bz * bx * dvz_dx) / (b * b);
        bv_gradv = (bx * vx * dvx_dx + by * vx * dvy_dx + bz * vx * dvz_dx) / b;
    }
    const double mu2 = s->mu * s->mu;
    const double acc_rate = -(0.5 * (1.0 - mu2) * divv + 0.5 * (3.0 * mu2 - 1.0) * bb_gradv +
                              s->mu * bv_gradv / s->v);
    double dp_dt = s->p * acc_rate;
    const double dpp = dpp_terms(pr, s->p, f, kap, b, divv, &dp_dt);
    const double div_bnorm = -(bx * f[29] / (b * b));
    double dmu_dt, duu, duu_du;
    calc_duu(pr, s, b, aux, div_bnorm, divv, bb_gradv, bv_gradv, mu2, &dmu_dt, &duu, &duu_du);
    const double skpara = kap[K_SKPARA], skperp = kap[K_SKPERP];
    if (!fixed_dt) {
        if (dx_dt != 0.0 && dp_dt != 0.0 && dmu_dt != 0.0) {
            const double sk = (skperp > 0.0) ? skperp : skpara;
            double a = 0.5 * cs->dxm / sk, m = a * a;
            a = sk / dx_dt; if (a * a < m) m = a * a;
            a = (double)0.1f * s->p / fabs(dp_dt); if (a < m) m = a;
            a = (double)0.1f / fabs(dmu_dt); if (a < m) m = a;
            a = 2.0 * duu / (dmu_dt * dmu_dt); if (a < m) m = a;
            s->dt = m;
        } else {
            s->dt = c->dt_min;
        }
        if (s->dt < c->dt_min) s->dt = c->dt_min;
        if (s->dt > c->dt_max) s->dt = c->dt_max;
    }
    const double sdt = sqrt(s->dt);
    double r[4];
    push_noise(c, s, r);
    const double dX = dx_dt * s->dt + r[0] * skpara * sdt;
    push_ft_tail(c, s, dX, 0.0, 0.0, dp_dt, dpp, dmu_dt, duu, sdt, r, d);
}

/* particle_boundary_condition on a single rank: particle_module.f90:1984-2129.
 * A periodic direction has itself as neighbour and wraps by the box passed
 * in; an open direction escapes with count_flag -1..-6 and adds to leak. */
/* After particle_boundary_condition's one-period wrap (particle_module.f90
 * :1984-2129): a push longer than a period leaves the particle outside, where
 * the reference indexes outside its arrays (undefined).  The engine wraps by
 * whole periods more; inside the box this is the identity. */
static double wrap_rest(double x, double lo, double hi)
{
    const double per = hi - lo;
    if (x < lo) x += per * ceil((lo - x) / per);
    else if (x > hi) x -= per * ceil((x - hi) / per);
    return x;
}

static void boundary(const mover_ctx *c, ptl_state *s, double xlo, double xhi, double ylo,
                     double yhi, double zlo, double zhi, thread_acc *acc)
{
    const orc_params *pr = c->pr;
    if (s->x < xlo && s->flag == 1) {
        if (pr->pbcx) { orc_fixed_add(&acc->leak_hi, &acc->leak_lo, s->weight); s->flag = -1; }
        else s->x = wrap_rest(s->x - xlo + xhi, xlo, xhi);
    } else if (s->x > xhi && s->flag == 1) {
        if (pr->pbcx) { orc_fixed_add(&acc->leak_hi, &acc->leak_lo, s->weight); s->flag = -2; }
        else s->x = wrap_rest(s->x - xhi + xlo, xlo, xhi);
    }
    if (c->ndim > 1) {
        if (s->y < ylo && s->flag == 1) {
            if (pr->pbcy) { orc_fixed_add(&acc->leak_hi, &acc->leak_lo, s->weight); s->flag = -3; }
            else s->y = wrap_rest(s->y - ylo + yhi, ylo, yhi);
        } else if (s->y > yhi && s->flag == 1) {
            if (pr->pbcy) { orc_fixed_add(&acc->leak_hi, &acc->leak_lo, s->weight); s->flag = -4; }
            else s->y = wrap_rest(s->y - yhi + ylo, ylo, yhi);
        }
    }
    /* z too for include_3rd_dim runs (:2084) */
    if (c->ndim == 3 || c->i3) {
        if (s->z < zlo && s->flag == 1) {
            if (pr->pbcz) { orc_fixed_add(&acc->leak_hi, &acc->leak_lo, s->weight); s->flag = -5; }
            else s->z = wrap_rest(s->z - zlo + zhi, zlo, zhi);
        } else if (s->z > zhi && s->flag == 1) {
            if (pr->pbcz) { orc_fixed_add(&acc->leak_hi, &acc->leak_lo, s->weight); s->flag = -6; }
            else s->z = wrap_rest(s->z - zhi + zlo, zlo, zhi);
        }
    }
}

static void check_negp_or_boundary(const mover_ctx *c, ptl_state *s, thread_acc *acc)
{
    if (s->p < 0.0) {
        s->flag = 0;
        orc_fixed_add(&acc->negp_hi, &acc->negp_lo, s->weight);
    } else {
        boundary(c, s, c->xmin1, c->xmax1, c->ymin1, c->ymax1, c->zmin1, c->zmax1, acc);
    }
}

/* One push at the particle's current state: interpolation parameters,
 * interp_fields, kappa, push (the body at particle_module.f90:1615-1703). */
static void do_push(const mover_ctx *c, ptl_state *s, int fixed_dt, double d[6])
{
    const double rt = (s->t - c->t0) / c->dtf;
    int32_t pos[3];
    double w[8], f[32], kap[22], aux[16];
    const double *ap = NULL;
    cell_size cs = {c->dx, c->dy, c->dz};
    if (c->sph || c->nonuni) {
        orc_grid_interp_paramters(c->pr, NULL, s->x, s->y, s->z, pos, w);
        if (c->nonuni) {
            /* the pushes search the cell again (:3404-3407, :4693-4699) */
            const double *X = g_grid.pos[0], *Y = g_grid.pos[1], *Z = g_grid.pos[2];
            const int ix = grid_count(0, s->x) - 2;
            cs.dxm = X[ix + 2] - X[ix + 1];
            if (c->ndim > 1) {
                const int iy = grid_count(1, s->y) - 2;
                cs.dym = Y[iy + 2] - Y[iy + 1];
            }
            if (c->ndim == 3) {
                const int iz = grid_count(2, s->z) - 2;
                cs.dzm = Z[iz + 2] - Z[iz + 1];
            }
        }
    } else {
        orc_get_interp_paramters(c->ndim, (s->x - c->xmin) / c->dx, (s->y - c->ymin) / c->dy,
                                 (s->z - c->zmin) / c->dz, pos, w);
    }
    orc_interp_fields(c->f1, c->f2, c->time_interp, c->ndim, c->nxg, c->nyg, pos, w, rt, f);
    if (c->ndim == 3 && g_surf.on) {
        s->h1 = surface_height(0, pos, w, rt, c->time_interp);
        s->h2 = g_surf.has2 ? surface_height(1, pos, w, rt, c->time_interp) : 0.0;
    }
    if (c->aux1 && (c->pr->deltab_flag || c->pr->correlation_flag)) {
        orc_interp_aux(c->aux1, c->aux2, c->time_interp, c->ndim, c->nxg, c->nyg, pos, w, rt, aux);
        ap = aux;
    }
    orc_calc_spatial_diffusion_coefficients(c->pr, s->p, s->mu, f, ap, kap);
    if (c->pr->focused_transport) {
        if (c->ndim == 1) push_1d_ft(c, s, f, ap, kap, &cs, fixed_dt, d);
        else if (c->ndim == 2 && !c->i3) push_2d_ft(c, s, f, ap, kap, &cs, fixed_dt, d);
        else push_3d_ft(c, s, f, ap, kap, &cs, fixed_dt, d);
    } else {
        if (c->ndim == 1) push_1d(c, s, f, kap, &cs, fixed_dt, d);
        else if (c->ndim == 2 && !c->i3) push_2d(c, s, f, kap, &cs, fixed_dt, d);
        else push_3d(c, s, f, kap, &cs, fixed_dt, d);
    }
}

/* The per-particle body of particle_mover_one_cycle: :1560-1830. */
static void move_one(const mover_ctx *c, ptl_state *s, int nsteps_interval,
                     int num_fine_steps, thread_acc *acc)
{
    const double t0 = c->t0, dtf = c->dtf;
    const double dt_fine = dtf / num_fine_steps;
    double dl[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   /* deltax..deltamu */
    const double step = ceil((s->t - t0) / dt_fine);
    double dt_target = (step <= 0.0) ? dt_fine : step * dt_fine;
    if (dt_target > dtf) dt_target = dtf;

    if (s->p < 0.0 && s->flag == 1) {
        s->flag = 0;
        orc_fixed_add(&acc->negp_hi, &acc->negp_lo, s->weight);
    } else {
        boundary(c, s, c->xmin1, c->xmax1, c->ymin1, c->ymax1, c->zmin1, c->zmax1, acc);
    }
    if (s->flag != 1) return;

    const double limit = dtf + dt_fine * (double)0.1f;
    while (dt_target < limit) {
        if (s->flag != 1) break;
        while ((s->t - t0) < dt_target && s->flag == 1) {
            check_negp_or_boundary(c, s, acc);
            if (s->flag != 1) break;
            do_push(c, s, 0, dl);
            acc->steps += 1;
            s->nsteps_pushed = (s->nsteps_pushed + 1) % nsteps_interval;
            trk_after_push(s);
        }
        if ((s->t - t0) > dt_target && s->flag == 1) {
            s->x = s->x - dl[0];
            s->y = s->y - dl[1];
            s->z = s->z - dl[2];
            s->p = s->p - dl[3];
            s->v = s->v - dl[4];
            s->mu = s->mu - dl[5];
            s->t = s->t - s->dt;
            const double dt_old = s->dt;
            s->dt = t0 + dt_target - s->t;
            if (s->dt > 0.0) {
                if (s->tag_splitted < 0 && s->nsteps_pushed == 0) {
                    /* back one step if necessary (:1716-1722) */
                    s->nsteps_tracked = s->nsteps_tracked - 1;
                    s->nsteps_pushed = nsteps_interval - 2;
                } else {
                    s->nsteps_pushed = s->nsteps_pushed - 1;
                }
                do_push(c, s, 1, dl);
                acc->steps += 1;
                s->nsteps_pushed = (s->nsteps_pushed + 1) % nsteps_interval;
                trk_after_push(s);
            }
            s->dt = dt_old;
            check_negp_or_boundary(c, s, acc);
        }
        dt_target = dt_target + dt_fine;
    }
}

static void load_state(const orc_particles *P, int64_t i, ptl_state *s)
{
    s->x = P->x[i]; s->y = P->y[i]; s->z = P->z[i]; s->p = P->p[i];
    s->v = P->v[i]; s->mu = P->mu[i];
    s->t = P->t[i]; s->dt = P->dt[i]; s->weight = P->weight[i];
    s->flag = P->count_flag[i];
    s->nsteps_pushed = P->nsteps_pushed[i];
    s->split_times = P->split_times[i];
    s->origin = P->origin[i];
    s->nsteps_tracked = P->nsteps_tracked[i];
    s->tag_injected = P->tag_injected[i];
    s->tag_splitted = P->tag_splitted[i];
    s->rng_ctr = P->rng_ctr[i];
}

static void store_state(orc_particles *P, int64_t i, const ptl_state *s)
{
    P->x[i] = s->x; P->y[i] = s->y; P->z[i] = s->z; P->p[i] = s->p;
    P->v[i] = s->v; P->mu[i] = s->mu;
    P->t[i] = s->t; P->dt[i] = s->dt;
    P->count_flag[i] = (int8_t)s->flag;
    P->nsteps_pushed[i] = s->nsteps_pushed;
    P->nsteps_tracked[i] = s->nsteps_tracked;
    P->rng_ctr[i] = s->rng_ctr;
}

static void swap_particles(orc_particles *P, int64_t a, int64_t b)
{
#define SWP(arr, T) do { T t_ = P->arr[a]; P->arr[a] = P->arr[b]; P->arr[b] = t_; } while (0)
    SWP(x, double); SWP(y, double); SWP(z, double); SWP(p, double); SWP(v, double);
    SWP(mu, double); SWP(weight, double); SWP(t, double); SWP(dt, double);
    SWP(split_times, int8_t); SWP(count_flag, int8_t); SWP(origin, int32_t);
    SWP(nsteps_tracked, int32_t); SWP(nsteps_pushed, int32_t);
    SWP(tag_injected, int32_t); SWP(tag_splitted, int32_t); SWP(rng_ctr, uint32_t);
#undef SWP
}

/* Escaped-particle distribution (calc_escaped_distributions,
 * diagnostics.f90:950-957), filled by remove_particles when enabled. */
static struct {
    int npp;
    double pmin, pmax, pmin_log, dp_log;
    uint64_t *counts, *whi, *wlo;
} g_esc;

void orc_set_escaped_histogram(int npp, double pmin, double pmax, uint64_t *counts,
                               uint64_t *whi, uint64_t *wlo)
{
    g_esc.npp = npp;
    g_esc.pmin = pmin;
    g_esc.pmax = pmax;
    g_esc.pmin_log = npp > 0 ? log10(pmin) : 0.0;
    g_esc.dp_log = npp > 0 ? (log10(pmax) - g_esc.pmin_log) / npp : 0.0;
    g_esc.counts = counts;
    g_esc.whi = whi;
    g_esc.wlo = wlo;
}

static void escaped_add(const orc_particles *P, int64_t i)
{
    if (!g_esc.counts || P->count_flag[i] >= 0 || P->count_flag[i] < -6) return;
    const double p = P->p[i], mu = P->mu[i];
    if (!(p > g_esc.pmin && p <= g_esc.pmax && mu >= -1.0 && mu <= 1.0)) return;
    const int ip = (int)floor((log10(p) - g_esc.pmin_log) / g_esc.dp_log);
    if (ip < 0 || ip >= g_esc.npp) return;
    const int k = (-P->count_flag[i] - 1) * g_esc.npp + ip;
    g_esc.counts[k] += 1;
    orc_fixed_add(&g_esc.whi[k], &g_esc.wlo[k], P->weight[i]);
}

static struct {
    orc_particles *P;
    int64_t cap, *n;
} g_estore;

void orc_set_escaped_store(orc_particles *store, int64_t cap, int64_t *n)
{
    g_estore.P = store;
    g_estore.cap = cap;
    g_estore.n = n;
}

static void copy_one(const orc_particles *S, int64_t i, orc_particles *D, int64_t j)
{
    D->x[j] = S->x[i]; D->y[j] = S->y[i]; D->z[j] = S->z[i]; D->p[j] = S->p[i];
    D->v[j] = S->v[i]; D->mu[j] = S->mu[i]; D->weight[j] = S->weight[i];
    D->t[j] = S->t[i]; D->dt[j] = S->dt[i];
    D->split_times[j] = S->split_times[i]; D->count_flag[j] = S->count_flag[i];
    D->origin[j] = S->origin[i]; D->nsteps_tracked[j] = S->nsteps_tracked[i];
    D->nsteps_pushed[j] = S->nsteps_pushed[i]; D->tag_injected[j] = S->tag_injected[i];
    D->tag_splitted[j] = S->tag_splitted[i]; D->rng_ctr[j] = S->rng_ctr[i];
}

/* remove_particles: particle_module.f90:5365-5403 (same swap order); with
 * an escaped store set, escaped particles are copied to it first
 * (escaped_ptls, :5386-5389). */
int64_t orc_remove_particles(orc_particles *P, int64_t n, orc_counters *cnt)
{
    if (n <= 0) return n;
    int64_t nremoved = 0, i = 0;   /* i is 0-based; Fortran i = i0 + 1 */
    while (i < n) {
        if ((n - (i + 1)) == (nremoved - 1)) break;
        if (P->count_flag[i] == 1) {
            i += 1;
        } else {
            if (P->count_flag[i] < 0) {
                cnt->nptl_escaped += 1;
                escaped_add(P, i);
                if (g_estore.P && *g_estore.n < g_estore.cap) {
                    copy_one(P, i, g_estore.P, *g_estore.n);
                    *g_estore.n += 1;
                }
            }
            swap_particles(P, n - nremoved - 1, i);
            nremoved += 1;
        }
    }
    return n - nremoved;
}

static void setup_ctx(mover_ctx *c, const orc_params *pr, const orc_mhd_config *cfg,
                      const float *f1, const float *f2, int time_interp, double t0, double dtf)
{
    memset(c, 0, sizeof(*c));
    c->pr = pr; c->f1 = f1; c->f2 = f2; c->time_interp = time_interp;
    c->ndim = pr->ndim;
    c->nxg = cfg->nx + 4;
    c->nyg = (pr->ndim == 1) ? 1 : cfg->ny + 4;   /* 1D arrays are (-1:nx+2, 1, 1) */
    c->dx = cfg->dx; c->dy = cfg->dy; c->dz = cfg->dz;
    /* set_field_configuration on one rank: simulation_setup.f90:171-253. */
    c->xmin = cfg->xmin;
    const double xmax = c->xmin + (double)cfg->nx * cfg->dx;
    c->ymin = cfg->ymin;
    const double ymax = c->ymin + (double)cfg->ny * cfg->dy;
    double zmax;
    if (pr->ndim == 3) {
        c->zmin = cfg->zmin;
        zmax = c->zmin + (double)cfg->nz * cfg->dz;
    } else {
        c->zmin = cfg->zmin;
        zmax = cfg->zmax;
    }
    c->xmin1 = c->xmin - c->dx * 0.5; c->xmax1 = xmax + c->dx * 0.5;
    c->ymin1 = c->ymin - c->dy * 0.5; c->ymax1 = ymax + c->dy * 0.5;
    c->zmin1 = c->zmin - c->dz * 0.5; c->zmax1 = zmax + c->dz * 0.5;
    c->sph = pr->spherical_coord != 0;
    c->i3 = pr->ndim == 2 && pr->include_3rd_dim != 0;
    c->nonuni = pr->nonuniform_grid != 0;
    if (c->nonuni) {
        /* :1535-1546: the half cells beyond the box are those of the first
         * and last cells; xpos_local(i) is X[i + 1].  The z extension only
         * matters in 3D. */
        const double *X = g_grid.pos[0], *Y = g_grid.pos[1], *Z = g_grid.pos[2];
        const int nx = cfg->nx, ny = cfg->ny, nz = cfg->nz;
        c->xmin1 = c->xmin - (X[3] - X[2]) * 0.5;
        c->xmax1 = xmax + (X[nx + 2] - X[nx + 1]) * 0.5;
        if (pr->ndim > 1) {   /* 1D runs keep no y positions */
            c->ymin1 = c->ymin - (Y[3] - Y[2]) * 0.5;
            c->ymax1 = ymax + (Y[ny + 2] - Y[ny + 1]) * 0.5;
        }
        if (pr->ndim == 3) {
            c->zmin1 = c->zmin - (Z[3] - Z[2]) * 0.5;
            c->zmax1 = zmax + (Z[nz + 2] - Z[nz + 1]) * 0.5;
        }
    }
    c->cfg_xmin = cfg->xmin; c->cfg_ymin = cfg->ymin; c->cfg_zmin = cfg->zmin;
    c->cfg_lx = cfg->lx; c->cfg_ly = cfg->ly; c->cfg_lz = cfg->lz;
    /* set_dt_min_max: particle_module.f90:5519-5524. */
    c->dt_min = pr->dt_min_rel * dtf;
    c->dt_max = pr->dt_max_rel * dtf;
    c->t0 = t0; c->dtf = dtf;
    c->key[0] = (uint32_t)pr->seed;
    c->key[1] = (uint32_t)(pr->seed >> 32);
}

/* particle_mover on a single rank: particle_module.f90:1846-1974.  One
 * mover cycle, remove_particles, then the boundary pass on the exact box
 * and a second remove_particles.  Returns the new particle count. */
int64_t orc_particle_mover(const orc_params *pr, const orc_mhd_config *cfg,
                           const float *f1, const float *f2, const float *aux1,
                           const float *aux2, int time_interp,
                           orc_particles *P, int64_t n, double t0, double dtf,
                           int nsteps_interval, int num_fine_steps, int nthreads,
                           orc_counters *cnt)
{
    mover_ctx c;
    setup_ctx(&c, pr, cfg, f1, f2, time_interp, t0, dtf);
    c.aux1 = aux1;
    c.aux2 = aux2 ? aux2 : aux1;
    for (int64_t i = 0; i < n; ++i) P->nsteps_tracked[i] = 1;
    uint64_t lh = 0, ll = 0, nh = 0, nl = 0, steps = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
    {
        thread_acc acc = {0, 0, 0, 0, 0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t i = 0; i < n; ++i) {
            ptl_state s;
            load_state(P, i, &s);
            move_one(&c, &s, nsteps_interval, num_fine_steps, &acc);
            store_state(P, i, &s);
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            uint64_t o = ll; ll += acc.leak_lo; lh += acc.leak_hi + (ll < o);
            o = nl; nl += acc.negp_lo; nh += acc.negp_hi + (nl < o);
            steps += acc.steps;
        }
    }
    (void)nthreads;
    {
        uint64_t o = cnt->leak_lo; cnt->leak_lo += ll; cnt->leak_hi += lh + (cnt->leak_lo < o);
        o = cnt->leak_negp_lo; cnt->leak_negp_lo += nl; cnt->leak_negp_hi += nh + (cnt->leak_negp_lo < o);
        cnt->steps += steps;
    }
    n = orc_remove_particles(P, n, cnt);
    /* Final pass on the exact box (:1959-1973). */
    thread_acc acc = {0, 0, 0, 0, 0};
    const double xmax = c.xmin + (double)cfg->nx * cfg->dx;
    const double ymax = c.ymin + (double)cfg->ny * cfg->dy;
    const double zmax = (pr->ndim == 3) ? c.zmin + (double)cfg->nz * cfg->dz : cfg->zmax;
    for (int64_t i = 0; i < n; ++i) {
        ptl_state s;
        load_state(P, i, &s);
        if (s.p < 0.0 && s.flag != 1) {
            s.flag = 0;
            orc_fixed_add(&acc.negp_hi, &acc.negp_lo, s.weight);
        } else {
            boundary(&c, &s, c.xmin, xmax, c.ymin, ymax, c.zmin, zmax, &acc);
        }
        store_state(P, i, &s);
    }
    {
        uint64_t o = cnt->leak_lo; cnt->leak_lo += acc.leak_lo; cnt->leak_hi += acc.leak_hi + (cnt->leak_lo < o);
        o = cnt->leak_negp_lo; cnt->leak_negp_lo += acc.negp_lo; cnt->leak_negp_hi += acc.negp_hi + (cnt->leak_negp_lo < o);
    }
    return orc_remove_particles(P, n, cnt);
}

/* split_particle: particle_module.f90:5430-5480.  The
 * threshold uses split_ratio**split_times by repeated multiplication, the
 * new weight is 0.5**(1+split_times) (exact in single precision). */
int64_t orc_split_particle(const orc_params *pr, orc_particles *P, int64_t n,
                           int64_t nptl_max, double split_ratio, double pmin_split,
                           orc_counters *cnt)
{
    const int64_t nptl = n;
    for (int64_t i = 0; i < nptl; ++i) {
        const int k = P->split_times[i];
        double rk = 1.0;
        for (int j = 0; j < k; ++j) rk = rk * split_ratio;
        const double p_threshold = pmin_split * pr->p0 * rk;
        if (P->p[i] > p_threshold && P->p[i] <= pr->pmax) {
            if (n + 1 > nptl_max) return n;
            cnt->nptl_split += 1;
            P->weight[i] = ldexp(1.0, -(k + 1));
            P->split_times[i] = (int8_t)(k + 1);
            const int64_t c = n;
            n += 1;
            P->x[c] = P->x[i]; P->y[c] = P->y[i]; P->z[c] = P->z[i]; P->p[c] = P->p[i];
            P->v[c] = P->v[i]; P->mu[c] = P->mu[i]; P->weight[c] = P->weight[i];
            P->t[c] = P->t[i]; P->dt[c] = P->dt[i];
            P->split_times[c] = P->split_times[i]; P->count_flag[c] = P->count_flag[i];
            P->origin[c] = P->origin[i]; P->nsteps_tracked[c] = P->nsteps_tracked[i];
            P->nsteps_pushed[c] = P->nsteps_pushed[i];
            P->tag_injected[c] = P->tag_injected[i];
            P->rng_ctr[c] = P->rng_ctr[i];
            if (g_trk.tags && P->tag_splitted[i] < 0) {
                /* tracked parent (:5452-5474) */
                const int32_t tg = P->tag_splitted[i];
                int lo, hi;
                P->tag_splitted[c] = (int32_t)((uint32_t)tg - (1u << k));
                if (trk_selected(P->origin[c], P->tag_injected[c], k + 1, P->tag_splitted[c],
                                 &lo, &hi)) {
                    if (P->nsteps_pushed[i] == 0) {
                        P->nsteps_tracked[c] += 1;
                        trk_write(P->nsteps_tracked[c], lo, hi, P, c, NULL);
                    }
                } else {
                    P->tag_splitted[c] = -P->tag_splitted[c];
                }
                if (trk_selected(P->origin[i], P->tag_injected[i], k + 1, tg, &lo, &hi)) {
                    if (P->nsteps_pushed[i] == 0) {
                        P->nsteps_tracked[i] += 1;
                        trk_write(P->nsteps_tracked[i], lo, hi, P, i, NULL);
                    }
                } else {
                    P->tag_splitted[i] = -tg;   /* stop tracking */
                }
            } else {
                P->tag_splitted[c] = (int32_t)((uint32_t)P->tag_splitted[i] + (1u << k));
            }
        }
    }
    return n;
}

/* Bin edges: init_particle_distributions, diagnostics.f90:194-204. */
void orc_pbins_edges(const orc_params *pr, double *edges)
{
    const double lo = log10(pr->pmin), hi = log10(pr->pmax);
    const double d = (hi - lo) / pr->npp_global;
    for (int i = 0; i <= pr->npp_global; ++i) edges[i] = pow(10.0, lo + i * d);
}

/* Global f(p): calc_particle_distributions, diagnostics.f90:738-780 (Parker,
 * one mu bin).  Counts and exact fixed-point weight sums per bin. */
void orc_calc_particle_distributions(const orc_params *pr, const orc_particles *P,
                                     int64_t n, uint64_t *counts, uint64_t *whi,
                                     uint64_t *wlo, double *fglobal)
{
    const int npp = pr->npp_global;
    const double pmin_log = log10(pr->pmin), pmax_log = log10(pr->pmax);
    const double dp_log = (pmax_log - pmin_log) / npp;
    for (int b = 0; b < npp; ++b) { counts[b] = 0; whi[b] = 0; wlo[b] = 0; }
    for (int64_t i = 0; i < n; ++i) {
        const double p = P->p[i], mu = P->mu[i];
        if (p > pr->pmin && p <= pr->pmax && mu >= -1.0 && mu <= 1.0) {
            int ip = (int)floor((log10(p) - pmin_log) / dp_log);
            if (ip < 0 || ip >= npp) continue;   /* unreachable for p in range */
            counts[ip] += 1;
            orc_fixed_add(&whi[ip], &wlo[ip], P->weight[i]);
        }
    }
    for (int b = 0; b < npp; ++b) fglobal[b] = orc_fixed_to_double(whi[b], wlo[b]);
}

/* ------------------------------------------------------------------------ */
/* Injection.  Draw order follows the reference; the draws come from a     */
/* Philox stream keyed (seed_lo, seed_hi + 1) with counter (tag, call,      */
/* 0x494E4A43, 0), two uniforms per call.                                   */
/* ------------------------------------------------------------------------ */
typedef struct inj_stream {
    uint32_t key[2], tag, call;
    double buf[2];
    int avail;
} inj_stream;

static double inj_u01(inj_stream *s)
{
    if (s->avail == 0) {
        uint32_t ctr[4] = {s->tag, s->call, 0x494E4A43u, 0u}, w[4];
        orc_philox4x32_10(ctr, s->key, w);
        s->call += 1;
        s->buf[0] = orc_u01(w[0], w[1]);
        s->buf[1] = orc_u01(w[2], w[3]);
        s->avail = 2;
    }
    double u = s->buf[2 - s->avail];
    s->avail -= 1;
    return u;
}

static void inj_stream_init(inj_stream *s, const orc_params *pr, uint32_t tag)
{
    s->key[0] = (uint32_t)pr->seed;
    s->key[1] = (uint32_t)(pr->seed >> 32) + 1u;
    s->tag = tag; s->call = 0; s->avail = 0;
}

static void set_new_particle(orc_particles *P, int64_t c, double x, double y, double z, double p,
                             double v, double mu, double t, double dt, int32_t tag)
{
    P->x[c] = x; P->y[c] = y; P->z[c] = z; P->p[c] = p; P->v[c] = v; P->mu[c] = mu;
    P->weight[c] = 1.0; P->t[c] = t; P->dt[c] = dt;
    P->split_times[c] = 0; P->count_flag[c] = 1; P->origin[c] = 0;
    P->nsteps_tracked[c] = 0; P->nsteps_pushed[c] = 0;
    P->tag_injected[c] = tag; P->tag_splitted[c] = 1; P->rng_ctr[c] = 0;
}

/* inject_one_particle momentum draw: particle_module.f90:398-418. */
static double draw_p_one(const orc_params *pr, inj_stream *s, int dist_flag, double power_index)
{
    if (dist_flag == 0) {
        double ftest = 1.0, fxp = 0.5, ptmp = 0.0;
        while (ftest > fxp) {
            ptmp = (inj_u01(s) * (pr->pmax - pr->pmin) + pr->pmin) / pr->p0;
            fxp = ptmp * ptmp * exp(-(ptmp * ptmp));
            ftest = inj_u01(s) * (double)0.37f;
        }
        return ptmp * pr->p0;
    } else if (dist_flag == 2) {
        const double r01 = inj_u01(s);
        if ((int)power_index == 1) return pow(pr->pmax / pr->p0, r01) * pr->p0;
        const double norm = pow(pr->pmax, -power_index + 1.0) - pow(pr->p0, -power_index + 1.0);
        return pow(r01 * norm + pow(pr->p0, -power_index + 1.0), 1.0 / (-power_index + 1.0));
    }
    return pr->p0;
}

/* inject_particles_spatial_uniform + inject_one_particle, single rank:
 * particle_module.f90:385-530.  Returns the new particle count; at most
 * nptl_max - n particles are added. */
int64_t orc_inject_spatial_uniform(const orc_params *pr, orc_particles *P, int64_t n,
                                   int64_t nptl_max, int64_t nptl, double dt,
                                   int dist_flag, double particle_v0, double t_frame,
                                   double dt_mhd, const double box[6],
                                   double power_index, orc_counters *cnt)
{
    for (int64_t i = 0; i < nptl && n < nptl_max; ++i) {
        const int32_t tag = (int32_t)cnt->tag_max;
        cnt->tag_max += 1;
        inj_stream s;
        inj_stream_init(&s, pr, (uint32_t)tag);
        const double x = inj_u01(&s) * (box[3] - box[0]) + box[0];
        const double y = inj_u01(&s) * (box[4] - box[1]) + box[1];
        const double z = inj_u01(&s) * (box[5] - box[2]) + box[2];
        const double mu = (double)0.99f * (2.0 * inj_u01(&s) - 1.0);
        const double p = draw_p_one(pr, &s, dist_flag, power_index);
        const double v = particle_v0 * p / pr->p0;
        const double t = t_frame + inj_u01(&s) * dt_mhd;
        set_new_particle(P, n, x, y, z, p, v, mu, t, dt, tag);
        trk_injected(P, n);
        n += 1;
    }
    return n;
}


/* ------------------------------------------------------------------------ */
/* Injection where a field quantity is large: inject_particles_at_large_jz  */
/* (particle_module.f90:785-903), _absj (:922-1056), _divv (:1205-1337),    */
/* _rho (:1356-1468), and the cell counts get_ncells_large_*                 */
/* (mhd_data_parallel.f90:2211-2498) on one rank, uniform grid.             */
/* ------------------------------------------------------------------------ */
static double large_quantity(int quantity, int ndim, int sph, double x, double y,
                             const double f[32])
{
    if (sph) {
        /* the spherical forms of :866-890, :1030-1043, :1306-1316 */
        if (quantity == 0) return fabs(f[23] + (f[5] - f[21]) / x);
        if (quantity == 1) {
            const double ctheta = cos(y), stheta = sin(y), r = x;
            const double t1 = (ctheta * f[6] + stheta * f[27] - f[25]) / (r * stheta);
            const double t2 = (f[22] / stheta - f[6] - r * f[26]) / r;
            const double t3 = (f[5] + r * f[23] - f[21]) / r;
            return sqrt(t1 * t1 + t2 * t2 + t3 * t3);
        }
        if (quantity == 2) {
            double d = f[8] + 2.0 * f[0] / x;
            if (ndim > 1) {
                const double ctheta = cos(y), istheta = 1.0 / sin(y);
                d = d + (f[12] + f[1] * ctheta * istheta) / x;
                if (ndim > 2) d = d + f[2] * istheta / x;   /* vz, as the reference */
            }
            return -d;
        }
        return f[3];
    }
    if (quantity == 0) return fabs(f[23] - f[21]);
    if (quantity == 1) {
        const double a = f[25] - f[27], b = f[26] - f[22], c = f[21] - f[23];
        return sqrt(a * a + b * b + c * c);
    }
    if (quantity == 2) {
        double d = f[8];
        d = d + f[12];
        if (ndim > 2) d = d + f[16];
        return -d;
    }
    return f[3];
}

/* xpos_local(i) for the count loops: the grid's node i + 1 (i 1-based
 * interior index), or mhd_config's uniform positions. */
static double node_position(const orc_params *pr, const orc_mhd_config *cfg, int axis, int i)
{
    if ((pr->spherical_coord || pr->nonuniform_grid) && g_grid.pos[axis])
        return g_grid.pos[axis][i + 1];
    const double d = axis == 0 ? cfg->dx : axis == 1 ? cfg->dy : cfg->dz;
    const double o = axis == 0 ? cfg->xmin : axis == 1 ? cfg->ymin : cfg->zmin;
    return d * (double)(i - 1) + o;
}

int64_t orc_count_cells_large(const orc_params *pr, const orc_mhd_config *cfg, const float *full,
                              const float *aux, int quantity, double qmin, const double box[6])
{
    const int ndim = pr->ndim;
    const int nx = cfg->nx, ny = cfg->ny, nz = (ndim == 3) ? cfg->nz : 1;
    const size_t nxg = (size_t)nx + 4, nyg = (size_t)ny + 4;
    int64_t count = 0;
    const int sph = pr->spherical_coord != 0;
    for (int iz = 1; iz <= nz; ++iz) {
        const double zp = node_position(pr, cfg, 2, iz);
        const int inz = (ndim > 2) ? (zp > box[2] && zp < box[5]) : 1;
        for (int iy = 1; iy <= ny; ++iy) {
            const double yp = node_position(pr, cfg, 1, iy);
            const int iny = (ndim > 1) ? (yp > box[1] && yp < box[4]) : 1;
            for (int ix = 1; ix <= nx; ++ix) {
                const double xp = node_position(pr, cfg, 0, ix);
                if (!(inz && iny && xp > box[0] && xp < box[3])) continue;
                const size_t cz = (ndim == 3) ? (size_t)iz + 1 : 0;
                const float *r = full + 32 * ((size_t)ix + 1 + nxg * ((size_t)iy + 1 + nyg * cz));
                double q;
                if (sph && quantity == 0) {
                    /* get_ncells_large_jz (:2226-2234): (by - dbx_dy) in single */
                    const float t = r[5] - r[21];
                    q = fabs((double)r[23] + (double)t / xp);
                } else if (sph && quantity == 1) {
                    /* get_ncells_large_absj (:2285-2303) */
                    const double stheta = sin(yp), ctheta = cos(yp);
                    const double t1 = (ctheta * (double)r[6] + stheta * (double)r[27] -
                                       (double)r[25]) / (xp * stheta);
                    const double t2 = ((double)r[22] / stheta - (double)r[6] -
                                       xp * (double)r[26]) / xp;
                    const double t3 = ((double)r[5] - xp * (double)r[23] - (double)r[21]) / xp;
                    q = sqrt(t1 * t1 + t2 * t2 + t3 * t3);
                } else if (sph && quantity == 2) {
                    /* get_ncells_large_divv (:2404-2420).  ctheta and
                     * istheta are re-allocated over all ny + 4 nodes, so row
                     * iy reads node iy - 2; the dvz/dz term is added from
                     * ndim > 1; 2.0 * vx is single precision. */
                    const double yq = g_grid.pos[1] ? g_grid.pos[1][iy - 1] : 0.0;
                    const double ctheta = cos(yq), istheta = 1.0 / sin(yq);
                    const float vx2 = 2.0f * r[0];
                    double d = (double)r[8] + (double)vx2 / xp;
                    if (ndim > 1) {
                        d = d + ((double)r[12] + (double)r[1] * ctheta * istheta) / xp;
                        d = d + (double)r[16] * istheta / xp;
                    }
                    q = -d;
                } else if (quantity == 0) {
                    q = (double)fabsf(r[23] - r[21]);
                } else if (quantity == 1) {
                    const float t1 = r[25] - r[27], t2 = r[26] - r[22], t3 = r[21] - r[23];
                    q = (double)sqrtf(t1 * t1 + t2 * t2 + t3 * t3);
                } else if (quantity == 2) {
                    /* divv = farray1(nfields+1, :, :, :) re-allocates divv
                     * over the ghost-padded extent with lower bound 1:
                     * node (ix, iy, iz) reads the node two lower per axis. */
                    const size_t sz = (ndim == 3) ? (size_t)iz - 1 : 0;
                    const float *u = full + 32 * ((size_t)ix - 1 + nxg * ((size_t)iy - 1 + nyg * sz));
                    double d = (double)u[8];
                    d = d + (double)u[12];
                    if (ndim > 2) d = d + (double)u[16];
                    q = -d;
                } else if (quantity == 4) {
                    q = (double)aux[16 * ((size_t)ix + 1 + nxg * ((size_t)iy + 1 + nyg * cz))];
                } else {
                    q = (double)r[3];
                }
                if (q > qmin) count += 1;
            }
        }
    }
    return count;
}

int64_t orc_inject_at_large(const orc_params *pr, const orc_mhd_config *cfg, const float *full,
                            const float *aux, orc_particles *P, int64_t n, int64_t nptl_max,
                            int64_t nptl,
                            double dt, int dist_flag, double particle_v0, double t_frame,
                            double dt_mhd, int quantity, double qmin, const double box[6],
                            double power_index, orc_counters *cnt)
{
    const int ndim = pr->ndim;
    const double dom[6] = {cfg->xmin, cfg->ymin, cfg->zmin, cfg->xmin + (double)cfg->nx * cfg->dx,
                           cfg->ymin + (double)cfg->ny * cfg->dy,
                           (ndim == 3) ? cfg->zmin + (double)cfg->nz * cfg->dz : cfg->zmax};
    const int nxg = cfg->nx + 4, nyg = cfg->ny + 4;
    for (int64_t i = 0; i < nptl && n < nptl_max; ++i) {
        const int32_t tag = (int32_t)cnt->tag_max;
        cnt->tag_max += 1;
        inj_stream s;
        inj_stream_init(&s, pr, (uint32_t)tag);
        const int rho = (quantity == 3);
        double q = rho ? 0.0 : -2.0;
        double x = box[0], y = box[1], z = box[2];
        int64_t tries = 0;
        while (q < qmin && ++tries <= ((int64_t)1 << 22)) {   /* the engine's rejection bound */
            x = inj_u01(&s) * (dom[3] - dom[0]) + dom[0];
            y = inj_u01(&s) * (dom[4] - dom[1]) + dom[1];
            z = inj_u01(&s) * (dom[5] - dom[2]) + dom[2];
            if (x >= box[0] && x <= box[3] && y >= box[1] && y <= box[4] && z >= box[2] &&
                z <= box[5]) {
                int32_t pos[3];
                double w[8], f[32];
                orc_grid_interp_paramters(pr, cfg, x, y, z, pos, w);
                if (quantity == 4) {
                    double a16[16];
                    orc_interp_aux(aux, aux, 0, ndim, nxg, nyg, pos, w, 0.0, a16);
                    q = a16[0];
                } else {
                    orc_interp_fields(full, full, 0, ndim, nxg, nyg, pos, w, 0.0, f);
                    q = large_quantity(quantity, ndim, pr->spherical_coord != 0, x, y, f);
                }
            } else {
                q = rho ? 0.0 : -3.0;
            }
        }
        const double mu = (double)0.99f * (2.0 * inj_u01(&s) - 1.0);
        const double p = draw_p_one(pr, &s, dist_flag, power_index);
        const double v = particle_v0 * p / pr->p0;
        const double t = t_frame + inj_u01(&s) * dt_mhd;
        set_new_particle(P, n, x, y, z, p, v, mu, t, dt, tag);
        trk_injected(P, n);
        n += 1;
    }
    return n;
}

/* Injection on the plane x = xpos at the frame start, following the draw
 * order of inject_particles_at_shock (particle_module.f90:542-633) with the
 * shock locator replaced by the given x. */
/* locate_shock_xpos (mhd_data_parallel.f90:1988-2006) on a 32-variable
 * frame: per row (y fastest over nyg * nzg) maxloc of |dvx/dx| along x,
 * 1-based, first occurrence. */
void orc_locate_shock_xpos(const float *full, int nxg, int nyg, int nzg, int32_t *S)
{
    for (int r = 0; r < nyg * nzg; ++r) {
        float best = -1.0f;
        int at = 0;
        for (int ix = 0; ix < nxg; ++ix) {
            const float v = fabsf(full[8 + 32 * ((size_t)ix + (size_t)nxg * (size_t)r)]);
            if (v > best) { best = v; at = ix; }
        }
        S[r] = at + 1;
    }
}

/* The x of inject_particles_at_shock (particle_module.f90:568-588) with
 * interp_shock_location (mhd_data_parallel.f90:2017-2046) as described:
 * linear between the rows either side of y (and z), x = xmin + (index - 3) dx. */
static double shock_x(const orc_params *pr, const orc_mhd_config *cfg, const int32_t *S, int nyg,
                      int nzg, double y, double z)
{
    double sx;
    if (pr->ndim == 1) {
        sx = (double)S[0];
    } else {
        const double dpy = (y - cfg->ymin) / cfg->dy;
        const int jy = (int)floor(dpy);
        const double ry = dpy - (double)jy;
        int r0 = jy + 2, r1 = jy + 3;
        r0 = r0 < 0 ? 0 : (r0 > nyg - 1 ? nyg - 1 : r0);
        r1 = r1 < 0 ? 0 : (r1 > nyg - 1 ? nyg - 1 : r1);
        if (pr->ndim == 2) {
            sx = (1.0 - ry) * (double)S[r0] + ry * (double)S[r1];
        } else {
            const double dpz = (z - cfg->zmin) / cfg->dz;
            const int jz = (int)floor(dpz);
            const double rz = dpz - (double)jz;
            int k0 = jz + 2, k1 = jz + 3;
            k0 = k0 < 0 ? 0 : (k0 > nzg - 1 ? nzg - 1 : k0);
            k1 = k1 < 0 ? 0 : (k1 > nzg - 1 ? nzg - 1 : k1);
            sx = (1.0 - ry) * (1.0 - rz) * (double)S[r0 + nyg * k0] +
                 ry * (1.0 - rz) * (double)S[r1 + nyg * k0] +
                 (1.0 - ry) * rz * (double)S[r0 + nyg * k1] + ry * rz * (double)S[r1 + nyg * k1];
        }
    }
    return cfg->xmin + (sx - 3.0) * cfg->dx;
}

static int64_t inject_plane(const orc_params *pr, const orc_mhd_config *cfg, orc_particles *P,
                            int64_t n, int64_t nptl_max, int64_t nptl, double xpos,
                            const int32_t *S, int nyg, int nzg, double dt, int dist_flag,
                            double particle_v0, double t_frame, double power_index,
                            orc_counters *cnt);

int64_t orc_inject_at_shock(const orc_params *pr, const orc_mhd_config *cfg, const int32_t *S,
                            int nyg, int nzg, orc_particles *P, int64_t n, int64_t nptl_max,
                            int64_t nptl, double dt, int dist_flag, double particle_v0,
                            double t_frame, double power_index, orc_counters *cnt)
{
    return inject_plane(pr, cfg, P, n, nptl_max, nptl, 0.0, S, nyg, nzg, dt, dist_flag,
                        particle_v0, t_frame, power_index, cnt);
}

int64_t orc_inject_at_x(const orc_params *pr, const orc_mhd_config *cfg,
                        orc_particles *P, int64_t n, int64_t nptl_max,
                        int64_t nptl, double xpos, double dt, int dist_flag,
                        double particle_v0, double t_frame, double power_index,
                        orc_counters *cnt)
{
    return inject_plane(pr, cfg, P, n, nptl_max, nptl, xpos, NULL, 0, 0, dt, dist_flag,
                        particle_v0, t_frame, power_index, cnt);
}

/* The shared body: a plane at xpos, or the shock when S is given. */
static int64_t inject_plane(const orc_params *pr, const orc_mhd_config *cfg, orc_particles *P,
                            int64_t n, int64_t nptl_max, int64_t nptl, double xpos,
                            const int32_t *S, int nyg, int nzg, double dt, int dist_flag,
                            double particle_v0, double t_frame, double power_index,
                            orc_counters *cnt)
{
    const double ymin = cfg->ymin, ymax = cfg->ymin + (double)cfg->ny * cfg->dy;
    double zmin = cfg->zmin, zmax = cfg->zmax;
    if (pr->ndim == 3) zmax = cfg->zmin + (double)cfg->nz * cfg->dz;
    for (int64_t i = 0; i < nptl && n < nptl_max; ++i) {
        const int32_t tag = (int32_t)cnt->tag_max;
        cnt->tag_max += 1;
        inj_stream s;
        inj_stream_init(&s, pr, (uint32_t)tag);
        const double y = inj_u01(&s) * (ymax - ymin) + ymin;
        const double z = inj_u01(&s) * (zmax - zmin) + zmin;
        double p = pr->p0;
        if (dist_flag == 0) {
            double ftest = 1.0, fxp = 0.5, ptmp = 0.0;
            while (ftest > fxp) {
                ptmp = (inj_u01(&s) * (pr->pmax - pr->pmin) + pr->pmin) / pr->p0;
                fxp = ptmp * ptmp * exp((double)(-0.5f) * (ptmp * ptmp));
                ftest = inj_u01(&s) * (double)0.75f;
            }
            p = ptmp * pr->p0;
        } else if (dist_flag == 2) {
            p = draw_p_one(pr, &s, 2, power_index);
        }
        const double v = particle_v0 * p / pr->p0;
        const double mu = (double)0.99f * (2.0 * inj_u01(&s) - 1.0);
        const double x = S ? shock_x(pr, cfg, S, nyg, nzg, y, z) : xpos;
        set_new_particle(P, n, x, y, z, p, v, mu, t_frame, dt, tag);
        trk_injected(P, n);
        n += 1;
    }
    return n;
}

/* quick_check sums for one rank: diagnostics.f90:116-170.  out = {sum of
 * weights, pdt_min, pdt_max, sum of dt}. */
void orc_quick_check(const orc_particles *P, int64_t n, double out[4])
{
    double w = 0.0, mn = 1.0, mx = 0.0, s = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        w = w + P->weight[i];
        if (P->dt[i] < mn) mn = P->dt[i];
        if (P->dt[i] > mx) mx = P->dt[i];
        s = s + P->dt[i];
    }
    out[0] = w; out[1] = mn; out[2] = mx; out[3] = s;
}

/* One local distribution of calc_particle_distributions
 * (diagnostics.f90:782-878) on one rank, uniform grid: flocal(imu, ip, ix,
 * iy, iz), imu fastest; 0 < ip < npbins as in the reference. */
/* One parameter set of the local distributions (init_local_particle_
 * distributions, diagnostics.f90:262-290, on one rank). */
typedef struct {
    int ndim, spherical, nonuniform, nrx, nry, nrz, npb, nmu, rx, ry, rz;
    double xmin, ymin, zmin, dxd, dyd, dzd, pmin_log, dp_log, dmu;
} local_set;

static local_set local_set_of(const orc_mhd_config *cfg, int ndim, int spherical, int nonuniform,
                              double pmin, double pmax, int npbins, int nmu, int rx, int ry,
                              int rz)
{
    local_set s;
    const int nz = ndim == 3 ? cfg->nz : 1;
    s.ndim = ndim; s.spherical = spherical; s.nonuniform = nonuniform;
    s.nrx = (cfg->nx + rx - 1) / rx; s.nry = (cfg->ny + ry - 1) / ry; s.nrz = (nz + rz - 1) / rz;
    s.dxd = cfg->lx / s.nrx; s.dyd = cfg->ly / s.nry; s.dzd = cfg->lz / s.nrz;
    s.xmin = cfg->xmin; s.ymin = cfg->ymin; s.zmin = cfg->zmin;
    s.pmin_log = log10(pmin);
    s.dp_log = (log10(pmax) - s.pmin_log) / npbins;
    s.dmu = (double)(2.0f / (float)nmu);   /* single precision, :273 */
    s.npb = npbins; s.nmu = nmu; s.rx = rx; s.ry = ry; s.rz = rz;
    return s;
}

/* The bins of particle i (:785-800) and its weight (w / r^2 [/ sin(theta)]
 * in spherical coordinates, :765-772). */
static void local_bin(const local_set *s, const orc_particles *P, int64_t i, int *ix, int *iy,
                      int *iz, int *ip, int *imu, double *w)
{
    if (s->nonuniform) {
        *ix = (orc_binary_search(g_grid.pos[0], g_grid.n[0], P->x[i]) - 1) / s->rx + 1;
        *iy = (s->ndim > 1) ? (orc_binary_search(g_grid.pos[1], g_grid.n[1], P->y[i]) - 1) / s->ry + 1
                            : (int)floor((P->y[i] - s->ymin) / s->dyd) + 1;
        *iz = (s->ndim == 3) ? (orc_binary_search(g_grid.pos[2], g_grid.n[2], P->z[i]) - 1) / s->rz + 1
                             : (int)floor((P->z[i] - s->zmin) / s->dzd) + 1;
    } else {
        *ix = (int)floor((P->x[i] - s->xmin) / s->dxd) + 1;
        *iy = (int)floor((P->y[i] - s->ymin) / s->dyd) + 1;
        *iz = (int)floor((P->z[i] - s->zmin) / s->dzd) + 1;
    }
    *ip = (int)floor((log10(P->p[i]) - s->pmin_log) / s->dp_log) + 1;
    *imu = (int)floor((P->mu[i] + 1.0) / s->dmu) + 1;
    double ww = P->weight[i];
    if (s->spherical) {
        ww = ww / (P->x[i] * P->x[i]);
        if (s->ndim >= 2) ww = ww / sin(P->y[i]);
    }
    *w = ww;
}

/* Local escaped distributions (calc_escaped_distributions,
 * diagnostics.f90:958-1230) over escaped particles: the x faces into
 * fx(nmu, npbins, nry, nrz, 2), y into fy(nmu, npbins, nrx, nrz, 2) (ndim >
 * 1), z into fz(nmu, npbins, nrx, nry, 2) (ndim 3); each array as counts and
 * fixed-point (whi, wlo), zeroed here; NULL skips a face. */
void orc_calc_local_escaped_distribution(const orc_mhd_config *cfg, int ndim, int spherical,
                                         int nonuniform, double pmin, double pmax, int npbins,
                                         int nmu, int rx, int ry, int rz,
                                         const orc_particles *P, int64_t n,
                                         uint64_t *cx, uint64_t *hx, uint64_t *lx,
                                         uint64_t *cy, uint64_t *hy, uint64_t *ly,
                                         uint64_t *cz, uint64_t *hz, uint64_t *lz)
{
    const local_set s = local_set_of(cfg, ndim, spherical, nonuniform, pmin, pmax, npbins, nmu,
                                     rx, ry, rz);
    const size_t mp = (size_t)nmu * npbins;
    const size_t sz[3] = {mp * s.nry * s.nrz * 2, mp * s.nrx * s.nrz * 2, mp * s.nrx * s.nry * 2};
    uint64_t *C3[3] = {cx, cy, cz}, *H3[3] = {hx, hy, hz}, *L3[3] = {lx, ly, lz};
    for (int f = 0; f < 3; ++f)
        if (C3[f])
            for (size_t b = 0; b < sz[f]; ++b) { C3[f][b] = 0; H3[f][b] = 0; L3[f][b] = 0; }
    for (int64_t i = 0; i < n; ++i) {
        int ix, iy, iz, ip, imu;
        double w;
        local_bin(&s, P, i, &ix, &iy, &iz, &ip, &imu, &w);
        const int condx = ix >= 1 && ix <= s.nrx, condy = iy >= 1 && iy <= s.nry;
        const int condz = iz >= 1 && iz <= s.nrz;
        if (!(ip > 0 && ip < npbins && imu >= 1 && imu <= nmu)) continue;
        const int flag = P->count_flag[i];
        const size_t e0 = (size_t)(imu - 1) + (size_t)nmu * (size_t)(ip - 1);
        int f = -1;
        size_t e = 0;
        if ((flag == -1 || flag == -2) && condy && condz) {
            f = 0; e = e0 + mp * ((size_t)(iy - 1) + (size_t)s.nry * ((size_t)(iz - 1) + (size_t)s.nrz * (size_t)(-flag - 1)));
        } else if ((flag == -3 || flag == -4) && ndim > 1 && condx && condz) {
            f = 1; e = e0 + mp * ((size_t)(ix - 1) + (size_t)s.nrx * ((size_t)(iz - 1) + (size_t)s.nrz * (size_t)(-flag - 3)));
        } else if ((flag == -5 || flag == -6) && ndim > 2 && condx && condy) {
            f = 2; e = e0 + mp * ((size_t)(ix - 1) + (size_t)s.nrx * ((size_t)(iy - 1) + (size_t)s.nry * (size_t)(-flag - 5)));
        }
        if (f < 0 || !C3[f]) continue;
        C3[f][e] += 1;
        orc_fixed_add(&H3[f][e], &L3[f][e], w);
    }
}

/* The global distribution with pitch-angle bins (calc_particle_distributions
 * :773-779) or, by_face, the escaped one (calc_escaped_distributions
 * :949-957, column |count_flag|): the particle's own weight; the bins
 * p == pmax and mu == 1 would take (past the last) are dropped. */
void orc_calc_distribution_mu(const orc_params *pr, const orc_particles *P, int64_t n, int nmu,
                              int by_face, int nfaces, uint64_t *counts, uint64_t *whi,
                              uint64_t *wlo)
{
    const int npp = pr->npp_global;
    const double pmin_log = log10(pr->pmin);
    const double dp_log = (log10(pr->pmax) - pmin_log) / npp;
    const double dmu = (double)(2.0f / (float)nmu);   /* :206 */
    const size_t nb = (size_t)nmu * npp * (by_face ? nfaces : 1);
    for (size_t b = 0; b < nb; ++b) { counts[b] = 0; whi[b] = 0; wlo[b] = 0; }
    for (int64_t i = 0; i < n; ++i) {
        const double p = P->p[i], mu = P->mu[i];
        if (!(p > pr->pmin && p <= pr->pmax && mu >= -1.0 && mu <= 1.0)) continue;
        const int ip = (int)floor((log10(p) - pmin_log) / dp_log) + 1;
        const int imu = (int)floor((mu + 1.0) / dmu) + 1;
        if (ip < 1 || ip > npp || imu < 1 || imu > nmu) continue;
        int face = 0;
        if (by_face) {
            const int flag = P->count_flag[i];
            if (flag >= 0 || -flag > nfaces) continue;
            face = -flag - 1;
        }
        const size_t e = (size_t)(imu - 1) + (size_t)nmu * ((size_t)(ip - 1) + (size_t)npp * face);
        counts[e] += 1;
        orc_fixed_add(&whi[e], &wlo[e], P->weight[i]);
    }
}

void orc_calc_local_distribution(const orc_mhd_config *cfg, int ndim, int spherical,
                                 int nonuniform, double pmin, double pmax,
                                 int npbins, int nmu, int rx, int ry, int rz,
                                 const orc_particles *P, int64_t n, uint64_t *counts,
                                 uint64_t *whi, uint64_t *wlo, double *flocal)
{
    /* spherical: the local weight is w / r^2 (/ sin(theta) from 2D on),
     * diagnostics.f90:765-772; nonuniform: the spatial bin is
     * (binarySearch_R(xpos_local, x) - 1) / rx + 1 (:785-793), which counts
     * from the first ghost node. */
    const int nz = ndim == 3 ? cfg->nz : 1;
    const int nrx = (cfg->nx + rx - 1) / rx, nry = (cfg->ny + ry - 1) / ry, nrz = (nz + rz - 1) / rz;
    const double dxd = cfg->lx / nrx, dyd = cfg->ly / nry, dzd = cfg->lz / nrz;
    const double pmin_log = log10(pmin);
    const double dp_log = (log10(pmax) - pmin_log) / npbins;
    const double dmu = (double)(2.0f / (float)nmu);   /* single precision, :273 */
    const size_t nb = (size_t)nmu * npbins * nrx * nry * nrz;
    for (size_t b = 0; b < nb; ++b) { counts[b] = 0; whi[b] = 0; wlo[b] = 0; }
    for (int64_t i = 0; i < n; ++i) {
        int ix, iy, iz;
        if (nonuniform) {
            ix = (orc_binary_search(g_grid.pos[0], g_grid.n[0], P->x[i]) - 1) / rx + 1;
            iy = (ndim > 1) ? (orc_binary_search(g_grid.pos[1], g_grid.n[1], P->y[i]) - 1) / ry + 1
                            : (int)floor((P->y[i] - cfg->ymin) / dyd) + 1;
            iz = (ndim == 3) ? (orc_binary_search(g_grid.pos[2], g_grid.n[2], P->z[i]) - 1) / rz + 1
                             : (int)floor((P->z[i] - cfg->zmin) / dzd) + 1;
        } else {
            ix = (int)floor((P->x[i] - cfg->xmin) / dxd) + 1;
            iy = (int)floor((P->y[i] - cfg->ymin) / dyd) + 1;
            iz = (int)floor((P->z[i] - cfg->zmin) / dzd) + 1;
        }
        const int ip = (int)floor((log10(P->p[i]) - pmin_log) / dp_log) + 1;
        const int imu = (int)floor((P->mu[i] + 1.0) / dmu) + 1;
        if (ix < 1 || ix > nrx || iy < 1 || iy > nry || iz < 1 || iz > nrz) continue;
        if (!(ip > 0 && ip < npbins) || imu < 1 || imu > nmu) continue;
        const size_t e = (size_t)(imu - 1) + (size_t)nmu * ((size_t)(ip - 1) + (size_t)npbins *
                         ((size_t)(ix - 1) + (size_t)nrx * ((size_t)(iy - 1) + (size_t)nry * (iz - 1))));
        counts[e] += 1;
        double w = P->weight[i];
        if (spherical) {
            w = w / (P->x[i] * P->x[i]);
            if (ndim >= 2) w = w / sin(P->y[i]);
        }
        orc_fixed_add(&whi[e], &wlo[e], w);
    }
    for (size_t b = 0; b < nb; ++b) flocal[b] = orc_fixed_to_double(whi[b], wlo[b]);
}
