// Split-precision mover with field bricks staged in shared memory.
//
// The particle set is binned brick-major (particles.cu, CellGrid::tile): the
// grid is cut into bricks of bx x by x bz cells, and the particles of one
// brick are contiguous, ordered by cell inside it.  A persistent grid of
// CTAs (one per SM with ~200 KB of shared memory) takes work items from a
// global counter: an item is at most `items` particles of one brick.  For
// each item the CTA brings the node records of the brick plus a halo of
// hx, hy, hz cells on every side into shared memory with one TMA tensor copy
// per field frame (cp.async.bulk.tensor, completion on an mbarrier), then
// its warps take 32-particle groups of the item and run the same
// per-particle body as the global-gather kernel (mixed_body.cuh), reading
// the corner records from shared memory, for up to one chunk of pushes.
// A particle that walks out of the staged region pauses between pushes and
// is appended to an overflow list; the overflow kernel then finishes its
// chunk with global gathers, so the number of launches per interval stays
// the chunk count however often particles cross brick faces.  Results agree
// with the global-gather mover to FP32 rounding (the same Philox increments
// for the same push; a paused particle's FP32 working state is rebuilt from
// its FP64 record, at other pushes than in the global-gather mover).
//
// Interpolation follows interp_fields (mhd_data_parallel.f90:1751-1804) with
// the same weights and summation order as the global-gather kernel; the
// control flow is particle_mover_one_cycle (particle_module.f90:1481-1833).
#include <cuda.h>
#include <cudaTypedefs.h>

#include "mixed_body.cuh"

namespace gpat {
namespace {

// Limit of one wait on a brick copy: about one second at the GB300's clock.
constexpr long long kTileWaitCycles = 2000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete; false once the
// limit has passed.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > kTileWaitCycles) return false;
    }
    return true;
}

// The staged node records of every chunk plane: box {4, sx+1, sy+1[, sz+1],
// R/4} at node (ox, oy[, oz]), chunk 0.  Node coordinates may be negative or
// run past the grid (those nodes read as zeros and are never a corner of a
// valid cell).  The innermost coordinate is 0, so the copy starts on a
// 16-byte chunk boundary.
template <int NDIM>
__device__ __forceinline__ void tma_load_brick(uint32_t dst, const CUtensorMap *m, int ox, int oy,
                                               int oz, uint32_t bar) {
    const uint64_t tm = reinterpret_cast<uint64_t>(m);
    if (NDIM == 2) {
        asm volatile(
            "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
            "l"(tm), "r"(0), "r"(ox), "r"(oy), "r"(0), "r"(bar)
            : "memory");
    } else {
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
            " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
            "l"(tm), "r"(0), "r"(ox), "r"(oy), "r"(oz), "r"(0), "r"(bar)
            : "memory");
    }
}

template <int NDIM, bool NLGC, int THREADS>
__global__ void __launch_bounds__(THREADS, 1)
    mover_tile_kernel(const MixedRunArgs a, const MixedConsts k, const DevParticles P,
                      const __grid_constant__ CUtensorMap tm1,
                      const __grid_constant__ CUtensorMap tm2, const TileSched s) {
    extern __shared__ __align__(1024) float4 s_tile[];
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ long long s_brick, s_beg, s_end;
    __shared__ unsigned int s_next;
    const uint32_t bar = smem_u32(&s_bar);
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    const long long total = s.item_prefix[s.nbricks];
    const int lane = threadIdx.x & 31;
    uint32_t parity = 0;
    long long loaded = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            const long long t = (long long)atomicAdd(s.item_counter, 1ull);
            long long b = -1, beg = 0, end = 0;
            if (t < total) {
                long long lo = 0, hi = s.nbricks - 1;   // last brick with item_prefix <= t
                while (lo < hi) {
                    const long long mid = (lo + hi + 1) >> 1;
                    if (s.item_prefix[mid] <= t) lo = mid; else hi = mid - 1;
                }
                b = lo;
                const long long bs = b == 0 ? 0 : (long long)s.incl[b * s.cpb - 1];
                const long long be = (long long)s.incl[(b + 1) * s.cpb - 1];
                beg = bs + (t - s.item_prefix[b]) * s.items;
                end = min(be, beg + (long long)s.items);
            }
            s_brick = b; s_beg = beg; s_end = end; s_next = 0u;
        }
        __syncthreads();
        const long long b = s_brick;
        if (b < 0) break;
        const int bxi = (int)(b % s.nbx), byi = (int)((b / s.nbx) % s.nby),
                  bzi = (int)(b / ((long long)s.nbx * s.nby));
        // staged region: the brick and its halo, as node origin and cells
        const int ox = bxi * s.bx - s.hx, oy = byi * s.by - s.hy, oz = bzi * s.bz - s.hz;
        const int sx = s.bx + 2 * s.hx, sy = s.by + 2 * s.hy, sz = s.bz + 2 * s.hz;
        if (b != loaded) {
            if (threadIdx.x == 0) {
                // the previous brick's generic-proxy reads come before the
                // async-proxy writes of the next copy
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(bar, a.time_interp ? 2u * s.tile_bytes : s.tile_bytes);
                tma_load_brick<NDIM>(smem_u32(s_tile), &tm1, ox, oy, oz, bar);
                if (a.time_interp)
                    tma_load_brick<NDIM>(smem_u32(s_tile + s.tile2_off), &tm2, ox, oy, oz, bar);
            }
            const bool ok = mbar_wait(bar, parity);
            parity ^= 1u;
            if (__syncthreads_or(!ok)) {
                // The copy did not complete in time: record it, give the copy
                // in flight one more bounded wait, and leave.  The item's
                // particles stay unmoved and the engine reports the status.
                if (threadIdx.x == 0) set_status(a.cnt, kStatusTileTimeout);
                mbar_wait(bar, parity ^ 1u);
                return;
            }
            loaded = b;
        }
        const TileGather g{s_tile, s_tile + s.tile2_off, ox, oy, oz, sx, sy, sz, sx + 1,
                           (sx + 1) * (sy + 1), (int)s.nodes};
        const long long beg = s_beg, end = s_end;
        for (;;) {
            unsigned int grp = 0u;
            if (lane == 0) grp = atomicAdd(&s_next, 32u);
            grp = __shfl_sync(0xffffffffu, grp, 0);
            if (beg + (long long)grp >= end) break;
            const int64_t i = beg + (long long)grp + lane;
            bool active = false, exited = false;
            uint32_t pushes = 0;
            if (i < end) {
                pushes = move_particle<NDIM, NLGC>(a, k, P, i, active, g, a.chunk_pushes, exited);
                if (a.pause) a.pause[i] = active ? 1 : 0;   // exited: set by the overflow kernel
            }
            // particles that left the staged region go to the overflow list
            const unsigned m = __ballot_sync(0xffffffffu, exited);
            if (m) {
                unsigned long long base = 0;
                if (lane == 0) base = atomicAdd(s.ovf_count, (unsigned long long)__popc(m));
                base = __shfl_sync(0xffffffffu, base, 0);
                if (exited) {
                    const unsigned long long e = base + __popc(m & ((1u << lane) - 1u));
                    s.ovf_idx[e] = i;
                    s.ovf_done[e] = pushes;
                }
            }
            add_warp_counters(a.cnt, pushes, active, nullptr);
        }
        __syncthreads();
    }
}

// The rest of the chunk of every particle that left its staged region:
// global gathers, one particle per thread, grid-stride over the list.
template <int NDIM, bool NLGC>
__global__ void __launch_bounds__(128, NDIM == 2 ? GPAT_MIXED_MINB_2D : GPAT_MIXED_MINB_3D)
    mover_overflow_kernel(const MixedRunArgs a, const MixedConsts k, const DevParticles P,
                          const long long *idx, const unsigned int *done,
                          const unsigned long long *count) {
    const long long n = (long long)*count;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = (long long)blockIdx.x * blockDim.x; base < n; base += stride) {
        const long long t = base + threadIdx.x;
        bool active = false, exited = false;
        uint32_t pushes = 0;
        if (t < n) {
            // done < chunk_pushes: a particle at its limit pauses before the exit test
            const uint32_t left = a.chunk_pushes ? a.chunk_pushes - done[t] : 0u;
            pushes = move_particle<NDIM, NLGC>(a, k, P, idx[t], active, GlobalGather{}, left,
                                               exited);
            if (a.pause) a.pause[idx[t]] = active ? 1 : 0;
        }
        add_warp_counters(a.cnt, pushes, active, nullptr);
    }
}

// Work items: brick b's particle range [incl[b cpb - 1], incl[(b + 1) cpb - 1])
// in pieces of at most `items`; item_prefix[b] = items of the bricks before b,
// item_prefix[nbricks] = all items.  One block; also resets the counter.
__global__ void __launch_bounds__(1024)
    tile_items_kernel(const unsigned int *incl, long long nbricks, int cpb, int items,
                      long long *item_prefix, unsigned long long *item_counter) {
    __shared__ long long warp_tot[32];
    const long long per = (nbricks + 1023) / 1024;
    const long long b0 = min((long long)threadIdx.x * per, nbricks);
    const long long b1 = min(b0 + per, nbricks);
    auto count = [&](long long b) -> long long {
        const long long bs = b == 0 ? 0 : (long long)incl[b * cpb - 1];
        const long long be = (long long)incl[(b + 1) * cpb - 1];
        return (be - bs + items - 1) / items;
    };
    long long mine = 0;
    for (long long b = b0; b < b1; ++b) mine += count(b);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    long long x = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long acc = 0;
        for (int w = 0; w < 32; ++w) {
            const long long c = warp_tot[w];
            warp_tot[w] = acc;
            acc += c;
        }
    }
    __syncthreads();
    long long run = warp_tot[wid] + (x - mine);
    for (long long b = b0; b < b1; ++b) {
        item_prefix[b] = run;
        run += count(b);
    }
    if (threadIdx.x == 1023) item_prefix[nbricks] = run;
    if (threadIdx.x == 0) *item_counter = 0ull;
}

template <int NDIM, bool NLGC, int THREADS>
cudaError_t launch_tile(const MixedRunArgs &r, const MixedConsts &c, const DevParticles &P,
                        const CUtensorMap &tm1, const CUtensorMap &tm2, const TileSched &s,
                        size_t smem, int sm_count, cudaStream_t st) {
    auto kern = mover_tile_kernel<NDIM, NLGC, THREADS>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, THREADS, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    kern<<<(unsigned)(sm_count * per_sm), THREADS, smem, st>>>(r, c, P, tm1, tm2, s);
    return cudaGetLastError();
}

}  // namespace

size_t tile_smem_bytes(int ndim, int sx, int sy, int sz, int time_interp, uint32_t *tile_bytes,
                       uint32_t *tile2_off) {
    const size_t rec = (size_t)((ndim == 2) ? kRec2D : kRec3D) * sizeof(float);
    const size_t nodes = (size_t)(sx + 1) * (sy + 1) * (ndim == 3 ? sz + 1 : 1);
    const size_t one = nodes * rec;
    const size_t off = (one + 127) & ~(size_t)127;   // frame 2 at a 128-byte boundary
    if (tile_bytes) *tile_bytes = (uint32_t)one;
    if (tile2_off) *tile2_off = (uint32_t)(off / sizeof(float4));
    return time_interp ? off + one : one;
}

cudaError_t encode_brick_map(CUtensorMap *m, const float *planes, int ndim, int nxg, int nyg,
                             int nzg, int sx, int sy, int sz) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q{};
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                               cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return e != cudaSuccess ? e : cudaErrorNotSupported;
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    // planes: [R/4][nzg][nyg][nxg] float4; dims innermost first
    const cuuint64_t nch = ((ndim == 2) ? kRec2D : kRec3D) / 4;
    const cuuint64_t nx = (cuuint64_t)nxg, ny = (cuuint64_t)nyg, nz = (cuuint64_t)nzg;
    cuuint64_t dims[5], strides[4];
    cuuint32_t box[5];
    const cuuint32_t elem[5] = {1, 1, 1, 1, 1};
    cuuint32_t rank;
    if (ndim == 2) {
        rank = 4;
        dims[0] = 4; dims[1] = nx; dims[2] = ny; dims[3] = nch;
        strides[0] = 16; strides[1] = 16 * nx; strides[2] = 16 * nx * ny;
        box[0] = 4; box[1] = (cuuint32_t)(sx + 1); box[2] = (cuuint32_t)(sy + 1);
        box[3] = (cuuint32_t)nch;
    } else {
        rank = 5;
        dims[0] = 4; dims[1] = nx; dims[2] = ny; dims[3] = nz; dims[4] = nch;
        strides[0] = 16; strides[1] = 16 * nx; strides[2] = 16 * nx * ny;
        strides[3] = 16 * nx * ny * nz;
        box[0] = 4; box[1] = (cuuint32_t)(sx + 1); box[2] = (cuuint32_t)(sy + 1);
        box[3] = (cuuint32_t)(sz + 1); box[4] = (cuuint32_t)nch;
    }
    const CUresult r = encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank,
                              const_cast<float *>(planes), dims, strides, box, elem,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_mover_tile(const MoverArgs &a, const MixedConsts &c, const TileSched &s,
                              const CUtensorMap &tm1, const CUtensorMap &tm2, int threads,
                              int sm_count, cudaStream_t st) {
    tile_items_kernel<<<1, 1024, 0, st>>>(s.incl, s.nbricks, s.cpb, s.items,
                                          const_cast<long long *>(s.item_prefix), s.item_counter);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (a.n <= 0) return cudaSuccess;
    const MixedRunArgs r = mixed_run_args(a);
    const size_t smem = tile_smem_bytes(a.ndim, s.bx + 2 * s.hx, s.by + 2 * s.hy,
                                        s.bz + 2 * s.hz, a.time_interp, nullptr, nullptr);
#define GPAT_TILE_LAUNCH(ND, T)                                                                  \
    (a.nlgc ? launch_tile<ND, true, T>(r, c, a.P, tm1, tm2, s, smem, sm_count, st)             \
            : launch_tile<ND, false, T>(r, c, a.P, tm1, tm2, s, smem, sm_count, st))
    e = cudaErrorInvalidValue;
    if (a.ndim == 2) {
        if (threads == 256) e = GPAT_TILE_LAUNCH(2, 256);
        if (threads == 512) e = GPAT_TILE_LAUNCH(2, 512);
    } else {
        if (threads == 256) e = GPAT_TILE_LAUNCH(3, 256);
        if (threads == 512) e = GPAT_TILE_LAUNCH(3, 512);
    }
#undef GPAT_TILE_LAUNCH
    if (e != cudaSuccess) return e;
    const unsigned g = (unsigned)(sm_count * (a.ndim == 2 ? GPAT_MIXED_MINB_2D : GPAT_MIXED_MINB_3D));
    if (a.ndim == 2) {
        if (a.nlgc) mover_overflow_kernel<2, true><<<g, 128, 0, st>>>(r, c, a.P, s.ovf_idx, s.ovf_done, s.ovf_count);
        else mover_overflow_kernel<2, false><<<g, 128, 0, st>>>(r, c, a.P, s.ovf_idx, s.ovf_done, s.ovf_count);
    } else {
        if (a.nlgc) mover_overflow_kernel<3, true><<<g, 128, 0, st>>>(r, c, a.P, s.ovf_idx, s.ovf_done, s.ovf_count);
        else mover_overflow_kernel<3, false><<<g, 128, 0, st>>>(r, c, a.P, s.ovf_idx, s.ovf_done, s.ovf_count);
    }
    return cudaGetLastError();
}

}  // namespace gpat
