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
#include <cuda_bf16.h>

#include <cfloat>

#include "device_common.cuh"

namespace gpat {
namespace {

constexpr int kIn = kMlpFeatures, kH = kMlpHidden;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kIn, kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH * kH;
constexpr int kOffW4 = kOffB3 + kH, kOffB4 = kOffW4 + kH;
static_assert(kOffB4 + 1 == kMlpParams, "parameter layout");

__device__ __forceinline__ void clone_particle(const DevParticles &P, int64_t i, int64_t j) {
    P.x[j] = P.x[i]; P.y[j] = P.y[i]; P.z[j] = P.z[i]; P.p[j] = P.p[i];
    P.v[j] = P.v[i]; P.mu[j] = P.mu[i]; P.weight[j] = P.weight[i];
    P.t[j] = P.t[i]; P.dt[j] = P.dt[i];
    P.split_times[j] = P.split_times[i]; P.count_flag[j] = P.count_flag[i];
    P.origin[j] = P.origin[i]; P.nsteps_tracked[j] = P.nsteps_tracked[i];
    P.nsteps_pushed[j] = P.nsteps_pushed[i]; P.tag_injected[j] = P.tag_injected[i];
    P.tag_splitted[j] = P.tag_splitted[i]; P.rng_ctr[j] = P.rng_ctr[i];
}

__device__ __forceinline__ float sigm(float a) { return 1.0f / (1.0f + expf(-a)); }
__device__ __forceinline__ float silu(float a) { return a * sigm(a); }
__device__ __forceinline__ float dsilu(float a) {
    const float s = sigm(a);
    return s * (1.0f + a * (1.0f - s));
}

// Weights (BF16 in global memory) -> FP32 in shared memory for one block.
__device__ __forceinline__ void load_weights(const __nv_bfloat16 *w16, float *sw) {
    for (int k = threadIdx.x; k < kMlpParams; k += blockDim.x) sw[k] = __bfloat162float(w16[k]);
    __syncthreads();
}

// Forward pass of one sample; pre-activations go to a1..a3 when given.
__device__ float mlp_forward(const float *sw, const float h0[kIn], float *a1, float *a2,
                             float *a3, int stride) {
    float h1[kH], h2[kH];
#pragma unroll 4
    for (int i = 0; i < kH; ++i) {
        float s = sw[kOffB1 + i];
#pragma unroll
        for (int j = 0; j < kIn; ++j) s = fmaf(sw[kOffW1 + i * kIn + j], h0[j], s);
        if (a1) a1[i * stride] = s;
        h1[i] = silu(s);
    }
#pragma unroll 2
    for (int i = 0; i < kH; ++i) {
        float s = sw[kOffB2 + i];
#pragma unroll 16
        for (int j = 0; j < kH; ++j) s = fmaf(sw[kOffW2 + i * kH + j], h1[j], s);
        if (a2) a2[i * stride] = s;
        h2[i] = silu(s);
    }
    float z = sw[kOffB4];
#pragma unroll 2
    for (int i = 0; i < kH; ++i) {
        float s = sw[kOffB3 + i];
#pragma unroll 16
        for (int j = 0; j < kH; ++j) s = fmaf(sw[kOffW3 + i * kH + j], h2[j], s);
        if (a3) a3[i * stride] = s;
        z = fmaf(sw[kOffW4 + i], silu(s), z);
    }
    return z;
}

__device__ __forceinline__ void standardise(const float *x, const float *mean, const float *istd,
                                            float h0[kIn]) {
#pragma unroll
    for (int j = 0; j < kIn; ++j) h0[j] = (x[j] - mean[j]) * istd[j];
}

// ---------------------------------------------------------------------------
// Features of particles, from the packed field records (FP32, trilinear).
// ---------------------------------------------------------------------------
template <int NDIM>
__device__ void particle_features(const FeatureArgs &g, const DevParticles &P, int64_t i,
                                  float f[kIn]) {
    constexpr int R = (NDIM == 2) ? kRec2D : kRec3D;
    const double px = (P.x[i] - g.xmin) * g.idx, py = (P.y[i] - g.ymin) * g.idy;
    const double pz = (NDIM == 3) ? (P.z[i] - g.zmin) * g.idz : 0.0;
    int cx = (int)floor(px), cy = (int)floor(py), cz = (NDIM == 3) ? (int)floor(pz) : 0;
    float fx = (float)(px - cx), fy = (float)(py - cy), fz = (float)(pz - cz);
    // clamp into the ghost-padded grid (a particle about to leave keeps the
    // edge values)
    const int ix = min(max(cx + 2, 0), g.nxg - 2), iy = min(max(cy + 2, 0), g.nyg - 2);
    const int iz = (NDIM == 3) ? min(max(cz + 2, 0), g.nzg - 2) : 0;
    fx = fminf(fmaxf(fx, 0.0f), 1.0f); fy = fminf(fmaxf(fy, 0.0f), 1.0f);
    fz = fminf(fmaxf(fz, 0.0f), 1.0f);
    float v[R];
#pragma unroll
    for (int k = 0; k < R; ++k) v[k] = 0.0f;
    for (int kk = 0; kk < (NDIM == 3 ? 2 : 1); ++kk)
        for (int j = 0; j < 2; ++j)
            for (int ii = 0; ii < 2; ++ii) {
                float w = (ii ? fx : 1.0f - fx) * (j ? fy : 1.0f - fy);
                if (NDIM == 3) w *= (kk ? fz : 1.0f - fz);
                const size_t cell = (size_t)(ix + ii) +
                                    (size_t)g.nxg * ((size_t)(iy + j) + (size_t)g.nyg * (iz + kk));
                const float *r = g.rec + (size_t)R * cell;
#pragma unroll
                for (int k = 0; k < R; ++k) v[k] = fmaf(__ldg(r + k), w, v[k]);
            }
    f[0] = (float)((P.x[i] - g.xmin) * g.ilx);
    f[1] = (float)((P.y[i] - g.ymin) * g.ily);
    f[2] = (NDIM == 3) ? (float)((P.z[i] - g.zmin) * g.ilz) : 0.0f;
    f[3] = (float)log10(P.p[i] * g.ip0);
    if (NDIM == 2) {   // slots: vx vy bx by bz dvx/dx dvy/dy ... db/dx(13) db/dy(14)
        f[4] = v[5] + v[6];
        f[5] = sqrtf(v[2] * v[2] + v[3] * v[3] + v[4] * v[4]);
        f[6] = sqrtf(v[13] * v[13] + v[14] * v[14]);
    } else {           // slots: vx vy vz bx by bz dvx/dx dvy/dy dvz/dz ... db/dx(18..20)
        f[4] = v[6] + v[7] + v[8];
        f[5] = sqrtf(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
        f[6] = sqrtf(v[18] * v[18] + v[19] * v[19] + v[20] * v[20]);
    }
    f[7] = g.t_norm;
}

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
// Training: forward with stored pre-activations, per-sample deltas, weight
// gradients as sample-chunked outer-product sums, Adam.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) train_forward_kernel(
    const __nv_bfloat16 *w16, const float *norm, const float *x, const float *y,
    const int64_t *index, int64_t b, float *h0s, float *a1, float *a2, float *a3, float *dz,
    float *loss) {
    extern __shared__ float sw[];
    load_weights(w16, sw);
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (s < b) {
        const int64_t r = index ? index[s] : s;
        float h0[kIn];
        standardise(x + (size_t)r * kIn, norm, norm + kIn, h0);
#pragma unroll
        for (int j = 0; j < kIn; ++j) h0s[(size_t)s * kIn + j] = h0[j];
        const float z = mlp_forward(sw, h0, a1 + s, a2 + s, a3 + s, (int)b);
        const float t = y[r];
        // BCE with logits: max(z, 0) - t z + log(1 + exp(-|z|))
        l = fmaxf(z, 0.0f) - t * z + log1pf(expf(-fabsf(z)));
        dz[s] = (sigm(z) - t) / (float)b;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0 && l != 0.0f) atomicAdd(loss, l / (float)b);
}

// d3 = dz W4 * silu'(a3), d2 = (W3^T d3) * silu'(a2), d1 = (W2^T d2) * silu'(a1);
// pre-activation arrays are overwritten by the deltas (column s of [64][b]).
__global__ void __launch_bounds__(128) train_backward_kernel(const __nv_bfloat16 *w16,
                                                             int64_t b, const float *dz,
                                                             float *a1, float *a2, float *a3,
                                                             float *h1s, float *h2s, float *h3s) {
    extern __shared__ float sw[];
    load_weights(w16, sw);
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= b) return;
    const float g = dz[s];
    float d[kH], dn[kH];
#pragma unroll 8
    for (int i = 0; i < kH; ++i) {
        const float a = a3[i * b + s];
        h3s[i * b + s] = silu(a);
        d[i] = g * sw[kOffW4 + i] * dsilu(a);
        a3[i * b + s] = d[i];
    }
#pragma unroll 4
    for (int j = 0; j < kH; ++j) {
        float acc = 0.0f;
#pragma unroll 16
        for (int i = 0; i < kH; ++i) acc = fmaf(sw[kOffW3 + i * kH + j], d[i], acc);
        const float a = a2[j * b + s];
        h2s[j * b + s] = silu(a);
        dn[j] = acc * dsilu(a);
        a2[j * b + s] = dn[j];
    }
#pragma unroll 4
    for (int j = 0; j < kH; ++j) {
        float acc = 0.0f;
#pragma unroll 16
        for (int i = 0; i < kH; ++i) acc = fmaf(sw[kOffW2 + i * kH + j], dn[i], acc);
        const float a = a1[j * b + s];
        h1s[j * b + s] = silu(a);
        a1[j * b + s] = acc * dsilu(a);
    }
}

// grad[W][i][j] += sum_s delta[i][s] * prev[j][s] (+ bias: sum_s delta[i][s])
// for one layer, over the sample chunk of this block.  Layouts [rows][b].
constexpr int kChunk = 256;
__global__ void __launch_bounds__(256) weight_grad_kernel(const float *delta, int nout,
                                                          const float *prev, int nin,
                                                          bool prev_sample_major, int64_t b,
                                                          float *gw, float *gb) {
    __shared__ float sd[kH][33], sp[kH][33];
    const int64_t s0 = (int64_t)blockIdx.x * kChunk;
    const int64_t s1 = min(s0 + kChunk, b);
    const int nent = nout * nin;
    float acc[16], accb[1] = {0.0f};
    for (int k = 0; k < 16; ++k) acc[k] = 0.0f;
    for (int64_t c = s0; c < s1; c += 32) {
        const int m = (int)min((int64_t)32, s1 - c);
        for (int k = threadIdx.x; k < kH * 32; k += blockDim.x) {
            const int row = k / 32, col = k % 32;
            float dv = 0.0f, pv = 0.0f;
            if (col < m) {
                if (row < nout) dv = delta[(size_t)row * b + c + col];
                if (row < nin)
                    pv = prev_sample_major ? prev[(size_t)(c + col) * nin + row]
                                           : prev[(size_t)row * b + c + col];
            }
            sd[row][col] = dv;
            sp[row][col] = pv;
        }
        __syncthreads();
        for (int k = 0; k < 16; ++k) {
            const int e = threadIdx.x + k * 256;
            if (e < nent) {
                const int i = e / nin, j = e % nin;
                float a = acc[k];
                for (int t = 0; t < m; ++t) a = fmaf(sd[i][t], sp[j][t], a);
                acc[k] = a;
            }
        }
        if (threadIdx.x < nout)
            for (int t = 0; t < m; ++t) accb[0] += sd[threadIdx.x][t];
        __syncthreads();
    }
    for (int k = 0; k < 16; ++k) {
        const int e = threadIdx.x + k * 256;
        if (e < nent && acc[k] != 0.0f) atomicAdd(&gw[e], acc[k]);
    }
    if (threadIdx.x < nout && accb[0] != 0.0f) atomicAdd(&gb[threadIdx.x], accb[0]);
}

// Layer-4 gradient: gw[i] = sum_s dz[s] h3[i][s], gb = sum_s dz[s].
__global__ void __launch_bounds__(256) out_grad_kernel(const float *dz, const float *h3, int64_t b,
                                                       float *gw, float *gb) {
    const int64_t s0 = (int64_t)blockIdx.x * kChunk;
    const int64_t s1 = min(s0 + kChunk, b);
    const int i = threadIdx.x;
    if (i < kH) {
        float a = 0.0f;
        for (int64_t s = s0; s < s1; ++s) a = fmaf(dz[s], h3[(size_t)i * b + s], a);
        if (a != 0.0f) atomicAdd(&gw[i], a);
    } else if (i == kH) {
        float a = 0.0f;
        for (int64_t s = s0; s < s1; ++s) a += dz[s];
        if (a != 0.0f) atomicAdd(gb, a);
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

// Forward on given feature rows (tests, scoring).
__global__ void __launch_bounds__(128) infer_kernel(const __nv_bfloat16 *w16, const float *norm,
                                                    const float *x, int64_t n, float *z) {
    extern __shared__ float sw[];
    load_weights(w16, sw);
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float h0[kIn];
    standardise(x + (size_t)s * kIn, norm, norm + kIn, h0);
    z[s] = mlp_forward(sw, h0, nullptr, nullptr, nullptr, 1);
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
    extern __shared__ float sw[];
    load_weights(w16, sw);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int j = 0;
    double w = 0.0;
    if (i < n && P.count_flag[i] == 1) {
        float f[kIn], h0[kIn];
        particle_features<NDIM>(g, P, i, f);
        standardise(f, norm, norm + kIn, h0);
        const float z = mlp_forward(sw, h0, nullptr, nullptr, nullptr, 1);
        const double wt = a.w_ref * exp(-((double)fminf(fmaxf(z, -60.0f), 60.0f) - a.z_ref));
        w = P.weight[i];
        if (w > wt * a.sqrt_ratio) {
            const int split_times = P.split_times[i];
            j = (int)ceil(log2(w / (wt * a.sqrt_ratio)));
            j = max(1, min(j, a.max_level));
            j = min(j, 30 - split_times);          // int32 lineage tags
            if (j < 1) j = 0;
        } else if (w < wt / a.sqrt_ratio) {
            const uint4 r = philox4x32_10(
                make_uint4(P.rng_ctr[i], 0x524C5454u, (uint32_t)P.tag_injected[i],
                           (uint32_t)P.tag_splitted[i]),
                a.key0, a.key1);
            const double u = u01_53(r.x, r.y);
            if (u < w / wt) {
                P.weight[i] = wt;
            } else {
                P.count_flag[i] = 0;               // removed at the next removal
                atomicAdd(&cnt->nkilled, 1ull);
            }
        }
    }
    // Warp-aggregated reservation of the children slots.
    const int lane = threadIdx.x & 31;
    const unsigned m = (j > 0) ? ((1u << j) - 1u) : 0u;
    unsigned inc = m;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    const unsigned total = __shfl_sync(0xffffffffu, inc, 31);
    unsigned long long base = 0;
    int ok = 0;
    if (lane == 31 && total > 0) {
        unsigned long long old = *(volatile unsigned long long *)count;
        for (int t = 0; t < 1024; ++t) {       // bounded compare-and-swap
            if (old + total > (unsigned long long)cap) break;
            const unsigned long long prev = atomicCAS(count, old, old + total);
            if (prev == old) { ok = 1; base = old; break; }
            old = prev;
        }
    }
    ok = __shfl_sync(0xffffffffu, ok, 31);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (!ok || j == 0) return;
    const int64_t first = (int64_t)(base + inc - m);
    const int s = P.split_times[i];
    const double wc = w / (double)(1u << j);
    P.weight[i] = wc;
    P.split_times[i] = (int8_t)(s + j);
    for (unsigned c = 1; c <= m; ++c) {
        const int64_t d = first + (int64_t)(c - 1);
        clone_particle(P, i, d);
        P.tag_splitted[d] = (int32_t)((uint32_t)P.tag_splitted[i] + (c << s));
    }
    atomicAdd(&cnt->nsplit, (unsigned long long)m);
}

// Network output of every live particle (z[i], index-aligned) and the
// maximum as an order-preserving integer.
template <int NDIM>
__global__ void __launch_bounds__(128) score_kernel(const __nv_bfloat16 *w16, const float *norm,
                                                    const FeatureArgs g, const DevParticles P,
                                                    int64_t n, float *z, int *zmax_key) {
    extern __shared__ float sw[];
    load_weights(w16, sw);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || P.count_flag[i] != 1) return;
    float f[kIn], h0[kIn];
    particle_features<NDIM>(g, P, i, f);
    standardise(f, norm, norm + kIn, h0);
    const float v = fminf(fmaxf(mlp_forward(sw, h0, nullptr, nullptr, nullptr, 1), -60.0f), 60.0f);
    z[i] = v;
    const int b = __float_as_int(v);
    atomicMax(zmax_key, b >= 0 ? b : b ^ 0x7FFFFFFF);
}

// Exact sums over live particles of z + 64 and of w exp(z - zmax).
__global__ void score_sum_kernel(const DevParticles P, int64_t n, const float *z,
                                 const int *zmax_key, unsigned long long *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || P.count_flag[i] != 1) return;
    const int k = *zmax_key;
    const float zmax = __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF);
    atomicAdd(&out[0], 1ull);
    atomic_add_fixed(&out[1], &out[2], (double)z[i] + 64.0);
    atomic_add_fixed(&out[3], &out[4], P.weight[i] * exp((double)z[i] - (double)zmax));
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

size_t mlp_shared_bytes() { return sizeof(float) * kMlpParams; }

cudaError_t mlp_set_kernel_attributes() {
    const int smem = (int)mlp_shared_bytes();
    cudaError_t e = cudaFuncSetAttribute(train_forward_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(train_backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
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
    infer_kernel<<<(unsigned)((n + 127) / 128), 128, mlp_shared_bytes(), s>>>(w16, norm, x, n, z);
    return cudaGetLastError();
}

cudaError_t launch_mlp_train_step(const MlpTrainBuffers &t, const __nv_bfloat16 *w16,
                                  const float *norm, const float *x, const float *y,
                                  const int64_t *index, int64_t b, float *grad, float *loss,
                                  cudaStream_t s) {
    const unsigned blocks = (unsigned)((b + 127) / 128);
    train_forward_kernel<<<blocks, 128, mlp_shared_bytes(), s>>>(w16, norm, x, y, index, b, t.h0,
                                                                 t.a1, t.a2, t.a3, t.dz, loss);
    train_backward_kernel<<<blocks, 128, mlp_shared_bytes(), s>>>(w16, b, t.dz, t.a1, t.a2, t.a3,
                                                                  t.h1, t.h2, t.h3);
    const unsigned chunks = (unsigned)((b + kChunk - 1) / kChunk);
    // after the backward pass a1..a3 hold the deltas d1..d3
    weight_grad_kernel<<<chunks, 256, 0, s>>>(t.a1, kH, t.h0, kIn, true, b, grad + kOffW1,
                                              grad + kOffB1);
    weight_grad_kernel<<<chunks, 256, 0, s>>>(t.a2, kH, t.h1, kH, false, b, grad + kOffW2,
                                              grad + kOffB2);
    weight_grad_kernel<<<chunks, 256, 0, s>>>(t.a3, kH, t.h2, kH, false, b, grad + kOffW3,
                                              grad + kOffB3);
    out_grad_kernel<<<chunks, 128, 0, s>>>(t.dz, t.h3, b, grad + kOffW4, grad + kOffB4);
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
    cudaError_t e = cudaMemsetAsync(out, 0, 5 * sizeof(unsigned long long), s);
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
