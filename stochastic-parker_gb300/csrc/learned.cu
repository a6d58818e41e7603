// Learned splitting: a small MLP importance map trained on trajectories the
// mover generates, driving weighted splitting and Russian roulette.  No
// counterpart in the reference (its split_particle uses fixed momentum
// thresholds, particle_module.f90:5430-5480).
//
// Network: 8 features -> 64 -> 64 -> 64 -> 1, SiLU hidden units, a linear
// output read as the log-odds that the particle's future yield lies above a
// momentum threshold.  Weights are stored in BF16 and every product is
// accumulated in FP32; the optimizer keeps an FP32 master copy (Adam).
// Features: box-normalised x, y, z; log10(p / p0); div v; |B|; |grad B|;
// normalised time -- each standardised by the training set's mean and std.
// Every network evaluation (training, scoring, splitting) runs on the tensor
// cores through mlp_mma.cuh: BF16 weights and activations, FP32 accumulation.
#include <cuda_bf16.h>

#include <algorithm>
#include <cfloat>

#include "device_common.cuh"
#include "learned_dev.cuh"
#include "mlp_mma.cuh"

namespace gpat {
namespace {

constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kIn, kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH * kH;
constexpr int kOffW4 = kOffB3 + kH, kOffB4 = kOffW4 + kH;
static_assert(kOffB4 + 1 == kMlpParams, "parameter layout");

// Appends (features, tag_injected) of every live particle to the records.
template <int NDIM>
__global__ void record_kernel(const FeatureArgs g, const DevParticles P, int64_t n, float *feat,
                              int32_t *tags, unsigned long long *count, int64_t cap) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || P.count_flag[i] != 1) return;
    const unsigned long long slot = atomicAdd(count, 1ull);
    if ((int64_t)slot >= cap) return;
    float f[kIn];
    particle_features<NDIM>(g, P, i, f);
#pragma unroll
    for (int j = 0; j < kIn; ++j) feat[(size_t)slot * kIn + j] = f[j];
    tags[slot] = P.tag_injected[i];
}

// Final momentum by injection tag (plain runs: one particle per tag).
__global__ void final_p_kernel(const DevParticles P, int64_t n, float *p_by_tag, int64_t ntags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || P.count_flag[i] != 1) return;
    const int32_t t = P.tag_injected[i];
    if (t >= 0 && t < ntags) p_by_tag[t] = (float)P.p[i];
}

__global__ void label_kernel(const int32_t *tags, int64_t nrec, const float *p_by_tag,
                             int64_t ntags, float threshold, float *labels,
                             unsigned long long *npos) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool pos = false;
    if (i < nrec) {
        const int32_t t = tags[i];
        pos = t >= 0 && t < ntags && p_by_tag[t] > threshold;
        labels[i] = pos ? 1.0f : 0.0f;
    }
    const unsigned b = __ballot_sync(0xffffffffu, pos);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(npos, (unsigned long long)__popc(b));
}

// ---------------------------------------------------------------------------
// Training step on the tensor cores: one CTA takes 128 samples (8 warps x 16),
// runs the forward pass, the loss, and the backward pass with register-
// resident fragments, then stages the activations h0..h3 and the deltas
// d1..d3 in shared memory feature-major (BF16) and forms the weight
// gradients dW_l = d_l^T h_(l-1) as mma products whose K dimension is the
// CTA's samples; they are added to the FP32 gradient with atomics.
// ---------------------------------------------------------------------------
constexpr int kTS = 128;          // samples per CTA
constexpr int kTP = kTS + 8;      // staging row (bf16): 68 words, lanes land in distinct banks
struct TrainSmem {
    mma_mlp::Smem w;
    __nv_bfloat16 h0T[kIn * kTP];       // standardised inputs [feature][sample]
    __nv_bfloat16 hT[3][kH * kTP];      // h1, h2, h3
    __nv_bfloat16 dT[3][kH * kTP];      // d1, d2, d3
    float dz[kTS];
};

__device__ __forceinline__ void stage_frag(__nv_bfloat16 *T, const uint32_t (&a)[4][4], int row0,
                                           int g, int t) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int col = 16 * kk + 2 * t + ((e & 2) ? 8 : 0);
            const int row = row0 + g + ((e & 1) ? 8 : 0);
            const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162 *>(&a[kk][e]);
            T[col * kTP + row] = v.x;
            T[(col + 1) * kTP + row] = v.y;
        }
}

// delta = (incoming C tiles) * silu'(a) as packed A fragments.
__device__ __forceinline__ void times_dsilu(const float (&c)[8][4], const uint32_t (&ds)[4][4],
                                            uint32_t (&d)[4][4]) {
    using namespace mma_mlp;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        const float *p = c[2 * kk], *q = c[2 * kk + 1];
        d[kk][0] = pack(p[0] * lo_of(ds[kk][0]), p[1] * hi_of(ds[kk][0]));
        d[kk][1] = pack(p[2] * lo_of(ds[kk][1]), p[3] * hi_of(ds[kk][1]));
        d[kk][2] = pack(q[0] * lo_of(ds[kk][2]), q[1] * hi_of(ds[kk][2]));
        d[kk][3] = pack(q[2] * lo_of(ds[kk][3]), q[3] * hi_of(ds[kk][3]));
    }
}

// dH = D x W (W as its transposed image): C tiles over the 64 inputs of W.
__device__ __forceinline__ void back_product(const uint32_t (&d)[4][4], const __nv_bfloat16 *wt,
                                             int g, int t, float (&c)[8][4]) {
    using namespace mma_mlp;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.0f;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            uint32_t b0, b1;
            bfrag(wt, kS, 8 * nt, 16 * kk, g, t, b0, b1);
            mma16816(c[nt], d[kk], b0, b1);
        }
    }
}

// One 16 x 8 tile of dW = D^T H over the staged samples: rows i0.., columns j0..
__device__ __forceinline__ void wgrad_tile(const __nv_bfloat16 *DT, const __nv_bfloat16 *HT, int i0,
                                           int j0, int g, int t, float (&acc)[4]) {
    using namespace mma_mlp;
    acc[0] = acc[1] = acc[2] = acc[3] = 0.0f;
#pragma unroll 2
    for (int s = 0; s < kTS; s += 16) {
        uint32_t a[4];
        a[0] = *reinterpret_cast<const uint32_t *>(DT + (i0 + g) * kTP + s + 2 * t);
        a[1] = *reinterpret_cast<const uint32_t *>(DT + (i0 + g + 8) * kTP + s + 2 * t);
        a[2] = *reinterpret_cast<const uint32_t *>(DT + (i0 + g) * kTP + s + 8 + 2 * t);
        a[3] = *reinterpret_cast<const uint32_t *>(DT + (i0 + g + 8) * kTP + s + 8 + 2 * t);
        const uint32_t b0 = *reinterpret_cast<const uint32_t *>(HT + (j0 + g) * kTP + s + 2 * t);
        const uint32_t b1 = *reinterpret_cast<const uint32_t *>(HT + (j0 + g) * kTP + s + 8 + 2 * t);
        mma16816(acc, a, b0, b1);
    }
}

__device__ __forceinline__ void add_tile(float *gw, int nin, int i0, int j0, int g, int t,
                                         const float (&acc)[4]) {
    atomicAdd(&gw[(i0 + g) * nin + j0 + 2 * t], acc[0]);
    atomicAdd(&gw[(i0 + g) * nin + j0 + 2 * t + 1], acc[1]);
    atomicAdd(&gw[(i0 + g + 8) * nin + j0 + 2 * t], acc[2]);
    atomicAdd(&gw[(i0 + g + 8) * nin + j0 + 2 * t + 1], acc[3]);
}

__global__ void __launch_bounds__(256, 1) train_mma_kernel(
    const __nv_bfloat16 *w16, const float *norm, const float *x, const float *y,
    const int64_t *index, int64_t b, float *grad, float *loss) {
    using namespace mma_mlp;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem &S = *reinterpret_cast<TrainSmem *>(smem_raw);
    load_smem(w16, S.w, true);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int row0 = 16 * warp;
    const int64_t sg0 = (int64_t)blockIdx.x * kTS + row0 + g, sg1 = sg0 + 8;
    const bool v0 = sg0 < b, v1 = sg1 < b;
    const int64_t r0 = v0 ? (index ? index[sg0] : sg0) : 0, r1 = v1 ? (index ? index[sg1] : sg1) : 0;
    // standardised inputs 2t, 2t+1 of rows g and g+8 (padded samples: zero)
    const float m0 = norm[2 * t], m1 = norm[2 * t + 1];
    const float i0s = norm[kIn + 2 * t], i1s = norm[kIn + 2 * t + 1];
    float x0g = 0.0f, x1g = 0.0f, x0h = 0.0f, x1h = 0.0f;
    if (v0) { x0g = (x[r0 * kIn + 2 * t] - m0) * i0s; x1g = (x[r0 * kIn + 2 * t + 1] - m1) * i1s; }
    if (v1) { x0h = (x[r1 * kIn + 2 * t] - m0) * i0s; x1h = (x[r1 * kIn + 2 * t + 1] - m1) * i1s; }
    uint32_t a1[4];
    input_frag(x0g, x1g, x0h, x1h, a1);
    {
        const __nv_bfloat162 u = *reinterpret_cast<const __nv_bfloat162 *>(&a1[0]);
        const __nv_bfloat162 v = *reinterpret_cast<const __nv_bfloat162 *>(&a1[1]);
        S.h0T[(2 * t) * kTP + row0 + g] = u.x;
        S.h0T[(2 * t + 1) * kTP + row0 + g] = u.y;
        S.h0T[(2 * t) * kTP + row0 + g + 8] = v.x;
        S.h0T[(2 * t + 1) * kTP + row0 + g + 8] = v.y;
    }
    Stash st;
    float zr[2];
    forward_tile<true>(S.w, a1, g, t, zr, &st);
    // loss and dL/dz (lanes with t == 0 hold z of rows g and g + 8)
    float l = 0.0f, dz0 = 0.0f, dz1 = 0.0f;
    if (t == 0) {
        if (v0) {
            const float yy = y[r0], z = zr[0];
            l += fmaxf(z, 0.0f) - yy * z + log1pf(__expf(-fabsf(z)));
            dz0 = (sigm(z) - yy) / (float)b;
        }
        if (v1) {
            const float yy = y[r1], z = zr[1];
            l += fmaxf(z, 0.0f) - yy * z + log1pf(__expf(-fabsf(z)));
            dz1 = (sigm(z) - yy) / (float)b;
        }
        S.dz[row0 + g] = dz0;
        S.dz[row0 + g + 8] = dz1;
    }
    dz0 = __shfl_sync(0xffffffffu, dz0, 4 * g);
    dz1 = __shfl_sync(0xffffffffu, dz1, 4 * g);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (lane == 0 && l != 0.0f) atomicAdd(loss, l / (float)b);
    // backward: d3 = dz W4 silu'(a3); d2 = (d3 W3) silu'(a2); d1 = (d2 W2) silu'(a1)
    uint32_t d3[4][4], d2[4][4], d1[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; ++kk)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int col = 16 * kk + 2 * t + ((e & 2) ? 8 : 0);
            const float dz = (e & 1) ? dz1 : dz0;
            const uint32_t ds = st.ds[2][kk][e];
            d3[kk][e] = pack(dz * S.w.w4f[col] * lo_of(ds), dz * S.w.w4f[col + 1] * hi_of(ds));
        }
    float c[8][4];
    back_product(d3, S.w.w3t, g, t, c);
    times_dsilu(c, st.ds[1], d2);
    back_product(d2, S.w.w2t, g, t, c);
    times_dsilu(c, st.ds[0], d1);
    // stage h1..h3 and d1..d3 feature-major
    stage_frag(S.hT[0], st.h[0], row0, g, t);
    stage_frag(S.hT[1], st.h[1], row0, g, t);
    stage_frag(S.hT[2], st.h[2], row0, g, t);
    stage_frag(S.dT[0], d1, row0, g, t);
    stage_frag(S.dT[1], d2, row0, g, t);
    stage_frag(S.dT[2], d3, row0, g, t);
    __syncthreads();
    // weight gradients: dW3 and dW2 (4 x 8 tiles each, 4 per warp), dW1 (4 tiles)
    float acc[4];
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
        const int tile = 4 * warp + q, i0 = 16 * (tile >> 3), j0 = 8 * (tile & 7);
        wgrad_tile(S.dT[2], S.hT[1], i0, j0, g, t, acc);
        add_tile(grad + kOffW3, kH, i0, j0, g, t, acc);
        wgrad_tile(S.dT[1], S.hT[0], i0, j0, g, t, acc);
        add_tile(grad + kOffW2, kH, i0, j0, g, t, acc);
    }
    if (warp < 4) {
        wgrad_tile(S.dT[0], S.h0T, 16 * warp, 0, g, t, acc);
        add_tile(grad + kOffW1, kIn, 16 * warp, 0, g, t, acc);
    }
    // biases (sum of deltas over the samples) and the output layer
    const int tid = threadIdx.x;
    if (tid < 3 * kH) {
        const int layer = tid / kH, i = tid % kH;
        const __nv_bfloat16 *row = S.dT[layer] + i * kTP;
        float s = 0.0f;
        for (int k = 0; k < kTS; ++k) s += __bfloat162float(row[k]);
        const int off = layer == 0 ? kOffB1 : (layer == 1 ? kOffB2 : kOffB3);
        if (s != 0.0f) atomicAdd(&grad[off + i], s);
    } else {
        const int i = tid - 3 * kH;   // 0..63
        const __nv_bfloat16 *row = S.hT[2] + i * kTP;
        float s = 0.0f, sb = 0.0f;
        for (int k = 0; k < kTS; ++k) {
            s = fmaf(S.dz[k], __bfloat162float(row[k]), s);
            sb += S.dz[k];
        }
        if (s != 0.0f) atomicAdd(&grad[kOffW4 + i], s);
        if (i == 0 && sb != 0.0f) atomicAdd(&grad[kOffB4], sb);
    }
}

__global__ void adam_kernel(float *master, float *m1, float *m2, float *grad,
                            __nv_bfloat16 *w16, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kMlpParams) return;
    const float g = grad[k];
    const float m = b1 * m1[k] + (1.0f - b1) * g;
    const float v = b2 * m2[k] + (1.0f - b2) * g * g;
    m1[k] = m;
    m2[k] = v;
    const float w = master[k] - lr * (m * c1) / (sqrtf(v * c2) + eps);
    master[k] = w;
    w16[k] = __float2bfloat16_rn(w);
    grad[k] = 0.0f;
}

__global__ void to_bf16_kernel(const float *master, __nv_bfloat16 *w16) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < kMlpParams) w16[k] = __float2bfloat16_rn(master[k]);
}

// Forward on given feature rows (tests, scoring): each warp takes tiles of
// 16 rows.
__global__ void __launch_bounds__(128) infer_mma_kernel(const __nv_bfloat16 *w16,
                                                        const float *norm, const float *x,
                                                        int64_t n, float *z) {
    using namespace mma_mlp;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem &S = *reinterpret_cast<Smem *>(smem_raw);
    load_smem(w16, S, false);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const float m0 = norm[2 * t], m1 = norm[2 * t + 1];
    const float i0s = norm[kIn + 2 * t], i1s = norm[kIn + 2 * t + 1];
    const int64_t tiles = (n + 15) / 16;
    for (int64_t tl = (int64_t)blockIdx.x * 4 + warp; tl < tiles; tl += (int64_t)gridDim.x * 4) {
        const int64_t r0 = 16 * tl + g, r1 = r0 + 8;
        float x0g = 0.0f, x1g = 0.0f, x0h = 0.0f, x1h = 0.0f;
        if (r0 < n) { x0g = (x[r0 * kIn + 2 * t] - m0) * i0s; x1g = (x[r0 * kIn + 2 * t + 1] - m1) * i1s; }
        if (r1 < n) { x0h = (x[r1 * kIn + 2 * t] - m0) * i0s; x1h = (x[r1 * kIn + 2 * t + 1] - m1) * i1s; }
        uint32_t a1[4];
        input_frag(x0g, x1g, x0h, x1h, a1);
        float zr[2];
        forward_tile<false>(S, a1, g, t, zr, nullptr);
        if (t == 0) {
            if (r0 < n) z[r0] = zr[0];
            if (r1 < n) z[r1] = zr[1];
        }
    }
}

// ---------------------------------------------------------------------------
// Weighted splitting and roulette.  Target weight w_t = w_ref exp(-(z - z_ref))
// (importance exp(z)); the window is [w_t / sqrt(ratio), w_t sqrt(ratio)].
// Above it a particle splits into 2^j copies (j <= max_level, chosen so the
// copies land in the window), below it survives with probability w / w_t at
// weight w_t.  Both keep the expected weight.  Children get the lineage tags
// of j successive binary splits (tag + bits << split_times).
// ---------------------------------------------------------------------------
template <int NDIM>
__global__ void __launch_bounds__(128) weighted_split_kernel(
    const __nv_bfloat16 *w16, const float *norm, const FeatureArgs g, DevParticles P, int64_t n,
    int64_t cap, WSplitArgs a, unsigned long long *count, DevCounters *cnt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    mma_mlp::Smem &S = *reinterpret_cast<mma_mlp::Smem *>(smem_raw);
    mma_mlp::load_smem(w16, S, false);
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n && P.count_flag[i] == 1;
    float h0[kIn];
    if (live) {
        float f[kIn];
        particle_features<NDIM>(g, P, i, f);
        standardise(f, norm, norm + kIn, h0);
    } else {
#pragma unroll
        for (int k = 0; k < kIn; ++k) h0[k] = 0.0f;
    }
    const float z = mma_mlp::warp_forward(S, h0);   // every lane of the warp takes part
    window_split(a, P, i, live, z, cap, count, cnt);
}

// Network output of every live particle (z[i], index-aligned) and the
// maximum as an order-preserving integer.
template <int NDIM>
__global__ void __launch_bounds__(128) score_kernel(const __nv_bfloat16 *w16, const float *norm,
                                                    const FeatureArgs g, const DevParticles P,
                                                    int64_t n, float *z, int *zmax_key) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    mma_mlp::Smem &S = *reinterpret_cast<mma_mlp::Smem *>(smem_raw);
    mma_mlp::load_smem(w16, S, false);
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = i < n && P.count_flag[i] == 1;
    float h0[kIn];
    if (live) {
        float f[kIn];
        particle_features<NDIM>(g, P, i, f);
        standardise(f, norm, norm + kIn, h0);
    } else {
#pragma unroll
        for (int k = 0; k < kIn; ++k) h0[k] = 0.0f;
    }
    const float zw = mma_mlp::warp_forward(S, h0);   // every lane of the warp takes part
    if (!live) return;
    const float v = fminf(fmaxf(zw, -60.0f), 60.0f);
    z[i] = v;
    const int b = __float_as_int(v);
    atomicMax(zmax_key, b >= 0 ? b : b ^ 0x7FFFFFFF);
}

// Exact sums over live particles of z + 64, of w exp(z - zmax) and of w.
__global__ void score_sum_kernel(const DevParticles P, int64_t n, const float *z,
                                 const int *zmax_key, unsigned long long *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || P.count_flag[i] != 1) return;
    const int k = *zmax_key;
    const float zmax = __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF);
    atomicAdd(&out[0], 1ull);
    atomic_add_fixed(&out[1], &out[2], (double)z[i] + 64.0);
    atomic_add_fixed(&out[3], &out[4], P.weight[i] * exp((double)z[i] - (double)zmax));
    atomic_add_fixed(&out[5], &out[6], P.weight[i]);
}

// Sum of weights and squared weights of live particles above a momentum.
__global__ void tail_kernel(const DevParticles P, int64_t n, double pthr,
                            unsigned long long *out /* count, w hi/lo, w2 hi/lo */) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || P.count_flag[i] != 1 || !(P.p[i] > pthr)) return;
    const double w = P.weight[i];
    atomicAdd(&out[0], 1ull);
    atomic_add_fixed(&out[1], &out[2], w);
    atomic_add_fixed(&out[3], &out[4], w * w);
}

}  // namespace

size_t mlp_shared_bytes() { return sizeof(mma_mlp::Smem); }

cudaError_t mlp_set_kernel_attributes() {
    const int smem = (int)mlp_shared_bytes();
    cudaError_t e = cudaFuncSetAttribute(train_mma_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TrainSmem));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(infer_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(weighted_split_kernel<2>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(weighted_split_kernel<3>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(score_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(score_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    return e;
}

cudaError_t launch_to_bf16(const float *master, __nv_bfloat16 *w16, cudaStream_t s) {
    to_bf16_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, w16);
    return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const __nv_bfloat16 *w16, const float *norm, const float *x, int64_t n,
                             float *z, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const int64_t tiles = (n + 15) / 16;
    const unsigned blocks = (unsigned)std::min<int64_t>((tiles + 3) / 4, 65535);
    infer_mma_kernel<<<blocks, 128, mlp_shared_bytes(), s>>>(w16, norm, x, n, z);
    return cudaGetLastError();
}

cudaError_t launch_mlp_train_step(const MlpTrainBuffers &t, const __nv_bfloat16 *w16,
                                  const float *norm, const float *x, const float *y,
                                  const int64_t *index, int64_t b, float *grad, float *loss,
                                  cudaStream_t s) {
    if (b <= 0) return cudaSuccess;
    (void)t;   // the tensor-core step keeps its intermediates in shared memory
    const unsigned blocks = (unsigned)((b + kTS - 1) / kTS);
    train_mma_kernel<<<blocks, 256, sizeof(TrainSmem), s>>>(w16, norm, x, y, index, b, grad, loss);
    return cudaGetLastError();
}

cudaError_t launch_adam(float *master, float *m1, float *m2, float *grad, __nv_bfloat16 *w16,
                        float lr, int step, cudaStream_t s) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f / (1.0f - powf(b1, (float)step));
    const float c2 = 1.0f / (1.0f - powf(b2, (float)step));
    adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(master, m1, m2, grad, w16, lr, b1, b2,
                                                         1e-8f, c1, c2);
    return cudaGetLastError();
}

cudaError_t launch_record_features(const FeatureArgs &g, int ndim, const DevParticles &P, int64_t n,
                                   float *feat, int32_t *tags, unsigned long long *count,
                                   int64_t cap, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (ndim == 2) record_kernel<2><<<blocks, 256, 0, s>>>(g, P, n, feat, tags, count, cap);
    else record_kernel<3><<<blocks, 256, 0, s>>>(g, P, n, feat, tags, count, cap);
    return cudaGetLastError();
}

cudaError_t launch_label_records(const DevParticles &P, int64_t n, const int32_t *tags,
                                 int64_t nrec, float *p_by_tag, int64_t ntags, float threshold,
                                 float *labels, unsigned long long *npos, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(p_by_tag, 0, sizeof(float) * (size_t)ntags, s);
    if (e != cudaSuccess) return e;
    if (n > 0) final_p_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, n, p_by_tag, ntags);
    if (nrec > 0)
        label_kernel<<<(unsigned)((nrec + 255) / 256), 256, 0, s>>>(tags, nrec, p_by_tag, ntags,
                                                                    threshold, labels, npos);
    return cudaGetLastError();
}

cudaError_t launch_weighted_split(const __nv_bfloat16 *w16, const float *norm,
                                  const FeatureArgs &g, int ndim, const DevParticles &P,
                                  int64_t n, int64_t cap, const WSplitArgs &a,
                                  unsigned long long *count, DevCounters *cnt, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((n + 127) / 128);
    if (ndim == 2)
        weighted_split_kernel<2><<<blocks, 128, mlp_shared_bytes(), s>>>(w16, norm, g, P, n, cap,
                                                                        a, count, cnt);
    else
        weighted_split_kernel<3><<<blocks, 128, mlp_shared_bytes(), s>>>(w16, norm, g, P, n, cap,
                                                                        a, count, cnt);
    return cudaGetLastError();
}

cudaError_t launch_score(const __nv_bfloat16 *w16, const float *norm, const FeatureArgs &g,
                         int ndim, const DevParticles &P, int64_t n, float *z, int *zmax_key,
                         unsigned long long *out, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, 7 * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(zmax_key, 0x80, sizeof(int), s);   // most negative
    if (e != cudaSuccess || n <= 0) return e;
    const unsigned blocks = (unsigned)((n + 127) / 128);
    if (ndim == 2)
        score_kernel<2><<<blocks, 128, mlp_shared_bytes(), s>>>(w16, norm, g, P, n, z, zmax_key);
    else
        score_kernel<3><<<blocks, 128, mlp_shared_bytes(), s>>>(w16, norm, g, P, n, z, zmax_key);
    score_sum_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, n, z, zmax_key, out);
    return cudaGetLastError();
}

cudaError_t launch_tail(const DevParticles &P, int64_t n, double pthr, unsigned long long *out,
                        cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(out, 0, 5 * sizeof(unsigned long long), s);
    if (e != cudaSuccess || n <= 0) return e;
    tail_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P, n, pthr, out);
    return cudaGetLastError();
}

}  // namespace gpat
