// Split-precision particle mover.
//
// Field records, interpolation, the kappa tensor, drift, noise amplitudes and
// the adaptive-dt candidates run in FP32.  The quantities that accumulate over
// thousands of steps are kept without FP64 arithmetic in the step loop:
//  - position as an integer cell index plus an FP32 offset inside the cell
//    (24 bits per cell, renormalised after every increment), which is also
//    exactly what interpolation and the boundary tests need;
//  - momentum and the particle clock as Kahan-compensated FP32 sums.
// The FP64 particle record is read once at entry and written once at exit as
// "input + accumulated change", so coordinates a call does not touch keep all
// their bits.
//
// Control flow is the reference's particle_mover_one_cycle
// (particle_module.f90:1481-1833): fine-step targets, adaptive pushes, the
// undo-and-redo landing on each target, boundaries on the half-cell-extended
// box, and the exact-box pass at the end of the interval.  Increments are the
// reference's (2u-1)*sqrt(3) variates (or Gaussian), four from one
// Philox-4x32-10 call per push.  The per-particle body is in mixed_body.cuh;
// this file holds the kernels that gather the packed field records from
// global memory (one particle per thread, and the batched persistent form).
#include "mixed_body.cuh"

#include "learned_dev.cuh"
#include "mlp_mma.cuh"

namespace gpat {

MixedConsts make_mixed_consts(const MoverArgs &a) {
    MixedConsts k{};
    k.idx = (float)(1.0 / a.dx); k.idy = (float)(1.0 / a.dy); k.idz = (float)(1.0 / a.dz);
    k.dxf = (float)a.dx; k.dyf = (float)a.dy; k.dzf = (float)a.dz;
    k.nx = a.nxg - 4; k.ny = a.nyg - 4; k.nz = a.ndim == 3 ? a.nzg - 4 : 1;
    k.dt_min = (float)a.dt_min; k.dt_max = (float)a.dt_max;
    k.dtf = (float)a.dtf; k.inv_dtf = (float)(1.0 / a.dtf);
    k.ip0 = (float)(1.0 / a.p0); k.pindex = (float)a.pindex; k.gm2 = (float)(a.gamma_turb - 2.0);
    k.kpara0 = (float)a.kpara0; k.kret = (float)a.kret;
    k.kperp0 = (float)(a.kpara0 * a.kperp_kpara);
    k.gm2_3 = (float)((a.gamma_turb - 2.0) / 3.0);
    k.pindex_perp = (float)((5.0 - a.gamma_turb) / 3.0);
    k.vdq = 1.0f / (float)(3 * a.charge);
    k.d1p0 = (float)(a.drift1 * a.p0);
    k.d2p0sq = (float)(a.drift2 * (a.p0 * a.p0));
    k.pfloor = (float)(0.25 * a.p0);
    for (int j = 0; j < 6; ++j) k.acc[j] = (float)a.acc_region[j];
    // box fraction = (x - cfg_min) / l = (cell coordinate + (min - cfg_min)/d) * d / l
    k.acc_off[0] = (float)((a.xmin - a.cfg_xmin) / a.dx);
    k.acc_off[1] = (float)((a.ymin - a.cfg_ymin) / a.dy);
    k.acc_off[2] = (float)((a.zmin - a.cfg_zmin) / a.dz);
    k.acc_scale[0] = (float)(a.dx / a.cfg_lx);
    k.acc_scale[1] = (float)(a.dy / a.cfg_ly);
    k.acc_scale[2] = (float)(a.dz / a.cfg_lz);
    return k;
}

namespace {

template <int NDIM, bool NLGC>
__global__ void __launch_bounds__(128, NDIM == 2 ? GPAT_MIXED_MINB_2D : GPAT_MIXED_MINB_3D)
    mover_mixed_kernel(const MixedRunArgs a, const MixedConsts k, const DevParticles P,
                       const int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool active = false, exited = false;
    uint32_t pushes = 0;
    if (i < n) {
        pushes = move_particle<NDIM, NLGC>(a, k, P, i, active, GlobalGather{}, a.chunk_pushes,
                                           exited);
        if (a.pause) a.pause[i] = active ? 1 : 0;
    }
    add_warp_counters(a.cnt, pushes, active, nullptr);
}

// The global-gather chunk kernel with learned splitting: as a particle
// finishes its interval in the box, the warp scores it with the network
// (tensor cores, weights staged in shared memory), adds w exp(z - z_shift)
// to the normalisation of the next interval and applies the weight window
// (split into lineage-tagged copies appended after the set, or roulette) in
// the same launch.  Warps with no finished particle skip the network.
template <int NDIM, bool NLGC>
__global__ void __launch_bounds__(128, NDIM == 2 ? GPAT_MIXED_MINB_2D : GPAT_MIXED_MINB_3D)
    mover_learned_kernel(const MixedRunArgs a, const MixedConsts k, const DevParticles P,
                         const int64_t n, const FusedLearn L) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    mma_mlp::SmemInf &S = *reinterpret_cast<mma_mlp::SmemInf *>(smem_raw);
    mma_mlp::load_smem(L.w16, S, false);
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool active = false, exited = false;
    uint32_t pushes = 0;
    if (i < n) {
        pushes = move_particle<NDIM, NLGC>(a, k, P, i, active, GlobalGather{}, a.chunk_pushes,
                                           exited);
        if (a.pause) a.pause[i] = active ? 1 : 0;
    }
    add_warp_counters(a.cnt, pushes, active, nullptr);
    const bool fin = i < n && !active && P.count_flag[i] == 1;
    if (!__any_sync(0xffffffffu, fin)) return;
    float h0[kMlpFeatures];
    if (fin) {
        float f[kMlpFeatures];
        particle_features<NDIM>(L.f, P, i, f);
        standardise(f, L.norm, L.norm + kMlpFeatures, h0);
    } else {
#pragma unroll
        for (int q = 0; q < kMlpFeatures; ++q) h0[q] = 0.0f;
    }
    const float z = mma_mlp::warp_forward(S, h0);
    if (fin) {
        const double e = fmin(fmax((double)z - L.z_shift, -60.0), 60.0);
        atomicAdd(&L.zsum[0], 1ull);
        atomic_add_fixed(&L.zsum[1], &L.zsum[2], P.weight[i] * exp(e));
        atomic_add_fixed(&L.zsum[3], &L.zsum[4], P.weight[i]);
    }
    window_split(L.s, P, i, fin, z, L.cap, L.count, a.cnt);
}

// ---------------------------------------------------------------------------
// Batched runs: one persistent launch moves the particles of up to
// kMaxBatchRuns independent runs.  Run descriptors sit in constant memory
// (a block reads its run's with uniform-index constant loads, off the L1
// path the gathers saturate); blocks take 128-particle tiles from a global
// counter across all runs, so uneven runs balance over the SMs.
// ---------------------------------------------------------------------------
__constant__ BatchRun c_batch_runs[kMaxBatchRuns];

template <int NDIM, bool NLGC, int MINB>
__global__ void __launch_bounds__(128, MINB)
    mover_mixed_batch_kernel(const int parity, const int nruns, const long long *tile_prefix,
                             const unsigned long long *run_n, unsigned long long *tile_counter,
                             const int grab, unsigned long long *nactive_total) {
    __shared__ long long s_tile;
    const long long total = tile_prefix[nruns];
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(tile_counter, (unsigned long long)grab);
        __syncthreads();
        const long long t0 = s_tile;
        if (t0 >= total) break;
        for (int g = 0; g < grab; ++g) {
            const long long t = t0 + g;
            if (t >= total) break;
            int lo = 0, hi = nruns - 1;        // last run with tile_prefix[r] <= t
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (tile_prefix[mid] <= t) lo = mid; else hi = mid - 1;
            }
            const BatchRun &d = c_batch_runs[lo];
            const int64_t i = (t - tile_prefix[lo]) * 128 + threadIdx.x;
            bool active = false, exited = false;
            uint32_t pushes = 0;
            if (i < (int64_t)run_n[lo])
                pushes = move_particle<NDIM, NLGC>(d.a, d.k, d.P[parity], i, active, GlobalGather{},
                                                  d.a.chunk_pushes, exited);
            add_warp_counters(d.a.cnt, pushes, active, nactive_total);
        }
    }
}

// Tile prefix over the runs' current particle counts, and a fresh scheduler.
__global__ void batch_prefix_kernel(const int nruns, const unsigned long long *run_n,
                                    long long *tile_prefix, unsigned long long *tile_counter,
                                    unsigned long long *nactive_total) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long acc = 0;
    for (int r = 0; r < nruns; ++r) {
        tile_prefix[r] = acc;
        acc += (long long)((run_n[r] + 127) / 128);
    }
    tile_prefix[nruns] = acc;
    *tile_counter = 0;
    *nactive_total = 0;
}

}  // namespace

MixedRunArgs mixed_run_args(const MoverArgs &a) {
    MixedRunArgs r{};
    r.rec1 = a.rec1; r.rec2 = a.rec2; r.cnt = a.cnt;
    r.dx = a.dx; r.dy = a.dy; r.dz = a.dz;
    r.xmin = a.xmin; r.ymin = a.ymin; r.zmin = a.zmin;
    r.t0 = a.t0; r.dtf = a.dtf; r.dt_fine = a.dt_fine; r.limit = a.limit;
    r.nxg = a.nxg; r.nyg = a.nyg; r.nzg = a.nzg;
    r.time_interp = a.time_interp; r.nsteps_interval = a.nsteps_interval;
    r.acc_region_flag = a.acc_region_flag; r.mag_dependency = a.mag_dependency;
    r.momentum_dependency = a.momentum_dependency; r.check_drift_2d = a.check_drift_2d;
    r.pbcx = a.pbcx; r.pbcy = a.pbcy; r.pbcz = a.pbcz; r.noise = a.noise;
    r.key0 = a.key0; r.key1 = a.key1; r.max_pushes = a.max_pushes;
    r.chunk_pushes = a.chunk_pushes;
    r.pause = a.pause;
    return r;
}

cudaError_t launch_mover_mixed(const MoverArgs &a, const MixedConsts &c, int sm_count,
                               cudaStream_t s) {
    (void)sm_count;
    if (a.n <= 0) return cudaSuccess;
    const int threads = 128;
    const int64_t blocks = (a.n + threads - 1) / threads;
    const unsigned g = (unsigned)blocks;
    const MixedRunArgs r = mixed_run_args(a);
    if (a.ndim == 2) {
        if (a.nlgc) mover_mixed_kernel<2, true><<<g, threads, 0, s>>>(r, c, a.P, a.n);
        else mover_mixed_kernel<2, false><<<g, threads, 0, s>>>(r, c, a.P, a.n);
    } else {
        if (a.nlgc) mover_mixed_kernel<3, true><<<g, threads, 0, s>>>(r, c, a.P, a.n);
        else mover_mixed_kernel<3, false><<<g, threads, 0, s>>>(r, c, a.P, a.n);
    }
    return cudaGetLastError();
}

cudaError_t launch_mover_learned(const MoverArgs &a, const MixedConsts &c, const FusedLearn &L,
                                 cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    const unsigned g = (unsigned)((a.n + 127) / 128);
    const size_t smem = sizeof(mma_mlp::SmemInf);
    const MixedRunArgs r = mixed_run_args(a);
    if (a.ndim == 2) {
        if (a.nlgc) mover_learned_kernel<2, true><<<g, 128, smem, s>>>(r, c, a.P, a.n, L);
        else mover_learned_kernel<2, false><<<g, 128, smem, s>>>(r, c, a.P, a.n, L);
    } else {
        if (a.nlgc) mover_learned_kernel<3, true><<<g, 128, smem, s>>>(r, c, a.P, a.n, L);
        else mover_learned_kernel<3, false><<<g, 128, smem, s>>>(r, c, a.P, a.n, L);
    }
    return cudaGetLastError();
}

cudaError_t upload_batch_runs(const BatchRun *runs, int nruns, cudaStream_t s) {
    if (nruns < 1 || nruns > kMaxBatchRuns) return cudaErrorInvalidValue;
    return cudaMemcpyToSymbolAsync(c_batch_runs, runs, sizeof(BatchRun) * (size_t)nruns, 0,
                                   cudaMemcpyHostToDevice, s);
}

cudaError_t launch_batch_prefix(int nruns, const unsigned long long *run_n, long long *tile_prefix,
                                unsigned long long *tile_counter,
                                unsigned long long *nactive_total, cudaStream_t s) {
    batch_prefix_kernel<<<1, 32, 0, s>>>(nruns, run_n, tile_prefix, tile_counter, nactive_total);
    return cudaGetLastError();
}

// Register-target variants the autotuner chooses from (resident 128-thread
// blocks per SM): 2D 5 / 6 / 8, 3D 4 / 5.
int batch_minb_variants(int ndim, int *out) {
    if (ndim == 2) { out[0] = 5; out[1] = 6; out[2] = 8; return 3; }
    out[0] = 4; out[1] = 5; return 2;
}

cudaError_t launch_mover_mixed_batch(int ndim, bool nlgc, int minb, int parity, int nruns,
                                     int sm_count, int grab, const long long *tile_prefix,
                                     const unsigned long long *run_n,
                                     unsigned long long *tile_counter,
                                     unsigned long long *nactive_total, cudaStream_t s) {
    const unsigned g = (unsigned)(sm_count * minb);
#define GPAT_BATCH_LAUNCH(ND, NL, MB)                                                         \
    mover_mixed_batch_kernel<ND, NL, MB><<<g, 128, 0, s>>>(parity, nruns, tile_prefix, run_n, \
                                                           tile_counter, grab, nactive_total)
    if (ndim == 2) {
        if (minb == 5) { if (nlgc) GPAT_BATCH_LAUNCH(2, true, 5); else GPAT_BATCH_LAUNCH(2, false, 5); }
        else if (minb == 6) { if (nlgc) GPAT_BATCH_LAUNCH(2, true, 6); else GPAT_BATCH_LAUNCH(2, false, 6); }
        else if (minb == 8) { if (nlgc) GPAT_BATCH_LAUNCH(2, true, 8); else GPAT_BATCH_LAUNCH(2, false, 8); }
        else return cudaErrorInvalidValue;
    } else {
        if (minb == 4) { if (nlgc) GPAT_BATCH_LAUNCH(3, true, 4); else GPAT_BATCH_LAUNCH(3, false, 4); }
        else if (minb == 5) { if (nlgc) GPAT_BATCH_LAUNCH(3, true, 5); else GPAT_BATCH_LAUNCH(3, false, 5); }
        else return cudaErrorInvalidValue;
    }
#undef GPAT_BATCH_LAUNCH
    return cudaGetLastError();
}

}  // namespace gpat
