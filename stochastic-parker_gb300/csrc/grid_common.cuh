// Interpolation on spherical and non-uniform grids, shared by the FP64
// mover and the injection kernels (both compiled with -fmad=false).
//
// Node positions are the ghost-padded xpos_global of one rank
// (mhd_data_parallel.f90:2051-2190): memory index j holds the node at the
// reference's local index j - 1 (-1 .. n + 2).
#pragma once

#include "device_common.cuh"

namespace gpat {

// binarySearch_R (particle_module.f90:680-698) on increasing nodes: the
// number of nodes <= v, by bisection.
__device__ __forceinline__ int grid_count(const double *__restrict__ a, int n, double v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = lo + ((hi - lo) >> 1);
        if (__ldg(a + mid) > v) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// The lower interpolation corner (memory indices) and the 8 weights.
struct GridCell {
    int ix, iy, iz;
    int kx, ky, kz;   // grid_count of the position per axis (kz = 0 in 2D)
    double w[8];
};

// Whether v lies between the first and the last ghost node, where the
// search and the corner stay inside the arrays.
__device__ __forceinline__ bool grid_inside(const double *__restrict__ a, int n, double v) {
    return v >= __ldg(a + 1) && v < __ldg(a + n - 1);
}

// get_interp_paramters_spherical (particle_module.f90:705-775) for
// spherical coordinates; on a non-uniform Cartesian grid the cell found by
// binarySearch_R with the offset of :1620-1625 fed to get_interp_paramters
// (:642-674), its corner placed at the searched cell.  Returns false when
// the position is outside the ghost nodes.
__device__ __forceinline__ bool grid_cell(int ndim, int spherical, const double *__restrict__ X,
                                          int nxg, const double *__restrict__ Y, int nyg,
                                          const double *__restrict__ Z, int nzg, double x,
                                          double y, double z, GridCell &c) {
    if (!grid_inside(X, nxg, x) || (ndim > 1 && !grid_inside(Y, nyg, y)) ||
        (ndim == 3 && !grid_inside(Z, nzg, z)))
        return false;
    c.kx = grid_count(X, nxg, x);
    c.ky = (ndim > 1) ? grid_count(Y, nyg, y) : 1;   // 1D: y node 0
    c.kz = (ndim == 3) ? grid_count(Z, nzg, z) : 0;
    double rx, ry, rz, rx1, ry1, rz1;
    if (spherical) {
        c.ix = c.kx - 1;
        c.iy = c.ky - 1;
        c.iz = (ndim == 3) ? c.kz - 1 : 0;
        const double one_third = 1.0 / 3.0;
        const double xa = __ldg(X + c.ix), xb = __ldg(X + c.ix + 1);
        const double x3 = x * x * x * one_third;
        const double x3_1 = xa * xa * xa * one_third;
        const double x3_2 = xb * xb * xb * one_third;
        rx = x3 - x3_1;
        rx1 = x3_2 - x3;
        if (ndim > 1) {
            const double ctheta1 = cos(__ldg(Y + c.iy));
            const double ctheta2 = cos(__ldg(Y + c.iy + 1));
            const double ctheta = cos(y);
            ry = ctheta1 - ctheta;
            ry1 = ctheta - ctheta2;
        } else {
            ry = 0.0;
            ry1 = 1.0;
        }
        if (ndim == 3) {
            rz = z - __ldg(Z + c.iz);
            rz1 = __ldg(Z + c.iz + 1) - z;
        } else {
            rz = 0.0;
            rz1 = 1.0;
        }
        const double dv = (x3_2 - x3_1) * (ry + ry1) * (rz + rz1);
        c.w[0] = rx1 * ry1 * rz1 / dv;
        c.w[1] = rx * ry1 * rz1 / dv;
        c.w[2] = rx1 * ry * rz1 / dv;
        c.w[3] = rx * ry * rz1 / dv;
        c.w[4] = rx1 * ry1 * rz / dv;
        c.w[5] = rx * ry1 * rz / dv;
        c.w[6] = rx1 * ry * rz / dv;
        c.w[7] = rx * ry * rz / dv;
        return true;
    }
    const int lx = c.kx - 1, ly = c.ky - 1, lz = (ndim == 3) ? c.kz - 1 : 0;
    const double px = (x - __ldg(X + lx)) / (__ldg(X + lx + 1) - __ldg(X + lx));
    const double py = (ndim > 1) ? (y - __ldg(Y + ly)) / (__ldg(Y + ly + 1) - __ldg(Y + ly)) : 0.0;
    const double pz = (ndim == 3) ? (z - __ldg(Z + lz)) / (__ldg(Z + lz + 1) - __ldg(Z + lz))
                                  : 0.0;
    const int fx = (int)floor(px), fy = (ndim > 1) ? (int)floor(py) : 0;
    const int fz = (ndim == 3) ? (int)floor(pz) : 0;
    rx = (px - (double)(fx + 1)) + 1.0;
    ry = (ndim > 1) ? (py - (double)(fy + 1)) + 1.0 : 0.0;
    rz = (ndim == 3) ? (pz - (double)(fz + 1)) + 1.0 : 0.0;
    c.ix = lx + fx;
    c.iy = ly + fy;
    c.iz = (ndim == 3) ? lz + fz : 0;
    if (c.ix > nxg - 2 || (ndim > 1 && c.iy > nyg - 2) || (ndim == 3 && c.iz > nzg - 2))
        return false;
    rx1 = 1.0 - rx;
    ry1 = 1.0 - ry;
    rz1 = 1.0 - rz;
    c.w[0] = rx1 * ry1 * rz1;
    c.w[1] = rx * ry1 * rz1;
    c.w[2] = rx1 * ry * rz1;
    c.w[3] = rx * ry * rz1;
    c.w[4] = rx1 * ry1 * rz;
    c.w[5] = rx * ry1 * rz;
    c.w[6] = rx1 * ry * rz;
    c.w[7] = rx * ry * rz;
    return true;
}

}  // namespace gpat
