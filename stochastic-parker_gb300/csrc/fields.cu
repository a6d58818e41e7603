// Field preparation kernels: raw 8-variable frames -> 32-variable arrays
// with gradients (mhd_data_parallel.f90:504-610) -> packed mover records.
#include "device_common.cuh"

namespace gpat {

// Slot order of the packed records, as indices into the 32-variable cell
// (vars 0-7: vx vy vz rho bx by bz |B|; gradient of var v along d at 8+3v+d).
__constant__ int kPack2D[kRec2D] = {0, 1, 4, 5, 6, 8, 12, 20, 21, 23, 24, 26, 27, 29, 30, 3};
__constant__ int kPack3D[kRec3D] = {0, 1, 2, 4, 5, 6, 8, 12, 16, 20, 21, 22,
                                    23, 24, 25, 26, 27, 28, 29, 30, 31, 3, 7, -1};

__global__ void scatter_raw_kernel(const float *__restrict__ raw, int nvar,
                                   float *__restrict__ full, size_t ncells) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride) {
        float *dst = full + 32 * c;
        const float *src = raw + (size_t)nvar * c;
#pragma unroll 8
        for (int v = 0; v < 32; ++v) dst[v] = (v < nvar) ? src[v] : 0.0f;
    }
}

cudaError_t launch_scatter_raw_fields(const float *raw, int nvar, float *full, size_t ncells,
                                      cudaStream_t s) {
    const int threads = 256;
    const size_t blocks = (ncells + threads - 1) / threads;
    scatter_raw_kernel<<<(unsigned)(blocks < 65535 * 16 ? blocks : 65535 * 16), threads, 0, s>>>(
        raw, nvar, full, ncells);
    return cudaGetLastError();
}

// One-sided / centred difference exactly as the reference evaluates it:
// single-precision differences, scaled by the double 0.5/d, rounded to float.
__device__ __forceinline__ float grad_lo(float a0, float a1, float a2, double ih) {
    float t = -__fmul_rn(3.0f, a0);
    t = __fadd_rn(t, __fmul_rn(4.0f, a1));
    t = __fsub_rn(t, a2);
    return (float)__dmul_rn((double)t, ih);
}
__device__ __forceinline__ float grad_hi(float an, float an1, float an2, double ih) {
    float t = __fmul_rn(3.0f, an);
    t = __fsub_rn(t, __fmul_rn(4.0f, an1));
    t = __fadd_rn(t, an2);
    return (float)__dmul_rn((double)t, ih);
}
__device__ __forceinline__ float grad_c(float ap, float am, double ih) {
    return (float)__dmul_rn((double)__fsub_rn(ap, am), ih);
}

// Gradients of NVAR variables of records of STRIDE floats (value of v at
// v * VSTRIDE, its d/dx d/dy d/dz at GBASE + v * GSTEP + axis); the z
// component only in 3D.  <32, 8, 1, 8, 3>: the field records; <16, 4, 4, 1, 4>:
// the fluctuation records {db2_slab, db2_2d, lc_slab, lc_2d}.  ihx/ihy/ihz:
// per-node inverse spans of a non-uniform grid (idxh_grid of
// set_local_grid_positions, mhd_data_parallel.f90:2153-2190, as used by
// calc_fields_gradients_nonuniform :612-764), or null for 0.5 / d.
template <int STRIDE, int NVAR, int VSTRIDE, int GBASE, int GSTEP>
__global__ void gradients_kernel(float *__restrict__ a, int ndim, int nxg, int nyg, int nzg,
                                 double idxh, double idyh, double idzh,
                                 const double *__restrict__ ihx, const double *__restrict__ ihy,
                                 const double *__restrict__ ihz) {
    const size_t ncells = (size_t)nxg * nyg * nzg;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t sx = STRIDE, sy = STRIDE * (size_t)nxg, sz = STRIDE * (size_t)nxg * nyg;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride) {
        const int i = (int)(c % nxg);
        const int j = (int)((c / nxg) % nyg);
        const int k = (int)(c / ((size_t)nxg * nyg));
        float *cell = a + STRIDE * c;
        const double hx = ihx ? ihx[i] : idxh;
        const double hy = ihy ? ihy[j] : idyh;
        const double hz = ihz ? ihz[k] : idzh;
#pragma unroll
        for (int v = 0; v < NVAR; ++v) {
            const int x = v * VSTRIDE, g = GBASE + v * GSTEP;
            float d;
            if (i == 0) d = grad_lo(cell[x], cell[x + sx], cell[x + 2 * sx], hx);
            else if (i == nxg - 1) d = grad_hi(cell[x], cell[x - sx], cell[x - 2 * sx], hx);
            else d = grad_c(cell[x + sx], cell[x - sx], hx);
            cell[g] = d;
            if (nyg > 1) {
                if (j == 0) d = grad_lo(cell[x], cell[x + sy], cell[x + 2 * sy], hy);
                else if (j == nyg - 1) d = grad_hi(cell[x], cell[x - sy], cell[x - 2 * sy], hy);
                else d = grad_c(cell[x + sy], cell[x - sy], hy);
                cell[g + 1] = d;
            }
            if (nzg > 1 && ndim == 3) {
                if (k == 0) d = grad_lo(cell[x], cell[x + sz], cell[x + 2 * sz], hz);
                else if (k == nzg - 1) d = grad_hi(cell[x], cell[x - sz], cell[x - 2 * sz], hz);
                else d = grad_c(cell[x + sz], cell[x - sz], hz);
                cell[g + 2] = d;
            }
        }
    }
}

cudaError_t launch_calc_fields_gradients(float *full, int ndim, int nxg, int nyg, int nzg,
                                         double dx, double dy, double dz, cudaStream_t s,
                                         const double *const *ih) {
    const size_t ncells = (size_t)nxg * nyg * nzg;
    const int threads = 256;
    size_t blocks = (ncells + threads - 1) / threads;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    gradients_kernel<32, 8, 1, 8, 3><<<(unsigned)blocks, threads, 0, s>>>(
        full, ndim, nxg, nyg, nzg, 0.5 / dx, 0.5 / dy, 0.5 / dz, ih ? ih[0] : nullptr,
        ih ? ih[1] : nullptr, ih ? ih[2] : nullptr);
    return cudaGetLastError();
}

cudaError_t launch_calc_aux_gradients(float *aux, int ndim, int nxg, int nyg, int nzg, double dx,
                                      double dy, double dz, cudaStream_t s,
                                      const double *const *ih) {
    const size_t ncells = (size_t)nxg * nyg * nzg;
    const int threads = 256;
    size_t blocks = (ncells + threads - 1) / threads;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    gradients_kernel<16, 4, 4, 1, 4><<<(unsigned)blocks, threads, 0, s>>>(
        aux, ndim, nxg, nyg, nzg, 0.5 / dx, 0.5 / dy, 0.5 / dz, ih ? ih[0] : nullptr,
        ih ? ih[1] : nullptr, ih ? ih[2] : nullptr);
    return cudaGetLastError();
}

// One scalar field (nzg, nyg, nxg) into component `comp` of the 16-float
// fluctuation records.
__global__ void scatter_aux_kernel(const float *__restrict__ src, float *__restrict__ aux,
                                   int comp, size_t ncells) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride)
        aux[16 * c + comp] = src[c];
}

__global__ void fill_kernel(float *__restrict__ a, float v, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += stride) a[c] = v;
}

cudaError_t launch_scatter_aux(const float *src, float *aux, int comp, size_t ncells,
                               cudaStream_t s) {
    const int threads = 256;
    size_t blocks = (ncells + threads - 1) / threads;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    scatter_aux_kernel<<<(unsigned)blocks, threads, 0, s>>>(src, aux, comp, ncells);
    return cudaGetLastError();
}

cudaError_t launch_fill(float *a, float v, size_t n, cudaStream_t s) {
    const int threads = 256;
    size_t blocks = (n + threads - 1) / threads;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    if (blocks == 0) return cudaSuccess;
    fill_kernel<<<(unsigned)blocks, threads, 0, s>>>(a, v, n);
    return cudaGetLastError();
}

template <int R>
__global__ void pack_kernel(const float *__restrict__ full, float *__restrict__ rec,
                            size_t ncells) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride) {
        const float *src = full + 32 * c;
        float *dst = rec + (size_t)R * c;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int v = (R == kRec2D) ? kPack2D[r] : kPack3D[r];
            dst[r] = v >= 0 ? src[v] : 0.0f;
        }
    }
}

cudaError_t launch_pack_records(const float *full, float *rec, int ndim, size_t ncells,
                                cudaStream_t s) {
    const int threads = 256;
    size_t blocks = (ncells + threads - 1) / threads;
    if (blocks > 65535 * 16) blocks = 65535 * 16;
    if (ndim == 2) pack_kernel<kRec2D><<<(unsigned)blocks, threads, 0, s>>>(full, rec, ncells);
    else pack_kernel<kRec3D><<<(unsigned)blocks, threads, 0, s>>>(full, rec, ncells);
    return cudaGetLastError();
}

}  // namespace gpat

namespace gpat {
namespace {

// Chunk-planar copy of the packed records: float4 chunk j of every node
// contiguous, planes[j * ncells + c] = rec[c * R + 4 j .. 4 j + 3].  The
// tile mover stages these planes, so neighbouring nodes of one chunk sit in
// neighbouring shared-memory bank groups.
template <int R>
__global__ void planarize_kernel(const float4 *__restrict__ rec, float4 *__restrict__ planes,
                                 size_t ncells) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += stride) {
#pragma unroll
        for (int j = 0; j < R / 4; ++j) planes[(size_t)j * ncells + c] = rec[c * (R / 4) + j];
    }
}

}  // namespace

cudaError_t launch_planarize_records(const float *rec, float *planes, int ndim, size_t ncells,
                                     cudaStream_t s) {
    const int threads = 256;
    size_t blocks = (ncells + threads - 1) / threads;
    if (blocks > 65535 * 8) blocks = 65535 * 8;
    const float4 *r = reinterpret_cast<const float4 *>(rec);
    float4 *o = reinterpret_cast<float4 *>(planes);
    if (ndim == 2) planarize_kernel<kRec2D><<<(unsigned)blocks, threads, 0, s>>>(r, o, ncells);
    else planarize_kernel<kRec3D><<<(unsigned)blocks, threads, 0, s>>>(r, o, ncells);
    return cudaGetLastError();
}

}  // namespace gpat
