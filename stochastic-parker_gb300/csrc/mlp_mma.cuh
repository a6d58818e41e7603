// Tensor-core evaluation of the learned-splitting network (8 -> 64 -> 64 ->
// 64 -> 1, SiLU) with mma.sync.m16n8k16 BF16 x BF16 -> FP32.
//
// One warp carries a tile of 16 samples through all layers.  The FP32
// accumulator fragment of one layer (rows = samples, columns = units) is,
// after SiLU and rounding to BF16, exactly the A-operand fragment of the next
// layer (C tiles 2k and 2k+1 form A k-step k), so activations stay in
// registers.  Weights sit in shared memory as BF16 in the B-operand order
// (row n = output unit, K contiguous) with padded rows (stride 72 or 24
// elements) so the 8 x 4 lanes of a fragment load hit 32 distinct banks.
//
// Fragment layouts (PTX ISA, mma.m16n8k16 with .bf16): lane = 4 g + t;
//   A (16 x 16): a0 = (g, 2t..2t+1), a1 = (g+8, 2t..), a2 = (g, 2t+8..), a3 = (g+8, 2t+8..)
//   B (16 x 8):  b0 = (k 2t..2t+1, n g), b1 = (k 2t+8..2t+9, n g)
//   C (16 x 8):  c0 = (g, 2t), c1 = (g, 2t+1), c2 = (g+8, 2t), c3 = (g+8, 2t+1)
#pragma once

#include <cuda_bf16.h>

#include "gpat_internal.h"

namespace gpat {
namespace mma_mlp {

constexpr int kIn = kMlpFeatures, kH = kMlpHidden;
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kH * kIn, kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH, kOffW3 = kOffB2 + kH, kOffB3 = kOffW3 + kH * kH;
constexpr int kOffW4 = kOffB3 + kH, kOffB4 = kOffW4 + kH;

constexpr int kS = 72;    // row stride of 64-wide weight rows (bf16 elements)
constexpr int kS1 = 24;   // row stride of the layer-1 rows (8 inputs padded to 16)

// Shared-memory image of the network.  The transposed copies W2t / W3t are
// the B operands of the backward pass (dH = D W).
struct Smem {
    __nv_bfloat16 w1[kH * kS1];
    __nv_bfloat16 w2[kH * kS];
    __nv_bfloat16 w3[kH * kS];
    __nv_bfloat16 w4[8 * kS];      // row 0: W4, rows 1..7: zero (N padded to 8)
    __nv_bfloat16 w2t[kH * kS];
    __nv_bfloat16 w3t[kH * kS];
    float b1[kH], b2[kH], b3[kH], w4f[kH], b4;
};

// Inference-only image (no transposed copies, about 24 KB) for kernels whose
// shared memory competes with L1 for the field gathers.
struct SmemInf {
    __nv_bfloat16 w1[kH * kS1];
    __nv_bfloat16 w2[kH * kS];
    __nv_bfloat16 w3[kH * kS];
    __nv_bfloat16 w4[8 * kS];
    float b1[kH], b2[kH], b3[kH], w4f[kH], b4;
};

// Fills a shared image from the BF16 parameter vector (the block's threads
// share the work; the caller synchronises).  transposed: also W2t / W3t
// (Smem only).
template <class SM>
__device__ __forceinline__ void load_smem(const __nv_bfloat16 *w16, SM &s, bool transposed) {
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.0f);
    for (int e = threadIdx.x; e < kH * kS1; e += blockDim.x) {
        const int n = e / kS1, k = e % kS1;
        s.w1[e] = k < kIn ? w16[kOffW1 + n * kIn + k] : zero;
    }
    for (int e = threadIdx.x; e < kH * kS; e += blockDim.x) {
        const int n = e / kS, k = e % kS;
        const bool in = k < kH;
        s.w2[e] = in ? w16[kOffW2 + n * kH + k] : zero;
        s.w3[e] = in ? w16[kOffW3 + n * kH + k] : zero;
        if constexpr (sizeof(SM) == sizeof(Smem)) {
            if (transposed) {
                s.w2t[e] = in ? w16[kOffW2 + k * kH + n] : zero;
                s.w3t[e] = in ? w16[kOffW3 + k * kH + n] : zero;
            }
        }
    }
    for (int e = threadIdx.x; e < 8 * kS; e += blockDim.x) {
        const int n = e / kS, k = e % kS;
        s.w4[e] = (n == 0 && k < kH) ? w16[kOffW4 + k] : zero;
    }
    for (int e = threadIdx.x; e < kH; e += blockDim.x) {
        s.b1[e] = __bfloat162float(w16[kOffB1 + e]);
        s.b2[e] = __bfloat162float(w16[kOffB2 + e]);
        s.b3[e] = __bfloat162float(w16[kOffB3 + e]);
        s.w4f[e] = __bfloat162float(w16[kOffW4 + e]);
    }
    if (threadIdx.x == 0) s.b4 = __bfloat162float(w16[kOffB4]);
}

__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Two values as one BF16x2 register, the lower column in the low half.
__device__ __forceinline__ uint32_t pack(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ float lo_of(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float hi_of(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

// B fragment of rows n0..n0+7, columns k0..k0+15 of a weight image.
__device__ __forceinline__ void bfrag(const __nv_bfloat16 *w, int stride, int n0, int k0, int g,
                                      int t, uint32_t &b0, uint32_t &b1) {
    const __nv_bfloat16 *p = w + (n0 + g) * stride + k0 + 2 * t;
    b0 = *reinterpret_cast<const uint32_t *>(p);
    b1 = *reinterpret_cast<const uint32_t *>(p + 8);
}

__device__ __forceinline__ float sigm(float a) { return 1.0f / (1.0f + __expf(-a)); }
__device__ __forceinline__ float silu(float a) { return a * sigm(a); }
__device__ __forceinline__ float dsilu(float a) {
    const float s = sigm(a);
    return s * (1.0f + a * (1.0f - s));
}

// One hidden layer: c[nt] = bias + A x W^T over 64 inputs (4 k-steps).
__device__ __forceinline__ void hidden(const uint32_t (&a)[4][4], const __nv_bfloat16 *w,
                                       const float *bias, int g, int t, float (&c)[8][4]) {
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float u0 = bias[8 * nt + 2 * t], u1 = bias[8 * nt + 2 * t + 1];
        c[nt][0] = u0; c[nt][1] = u1; c[nt][2] = u0; c[nt][3] = u1;
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            uint32_t b0, b1;
            bfrag(w, kS, 8 * nt, 16 * kk, g, t, b0, b1);
            mma16816(c[nt], a[kk], b0, b1);
        }
    }
}

// SiLU of the accumulator tiles as the next layer's A fragments; with ds,
// also silu'(pre-activation) in the same packed layout (backward pass).
__device__ __forceinline__ void activate(const float (&c)[8][4], uint32_t (&a)[4][4],
                                         uint32_t (*ds)[4]) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        const float *p = c[2 * kk], *q = c[2 * kk + 1];
        a[kk][0] = pack(silu(p[0]), silu(p[1]));
        a[kk][1] = pack(silu(p[2]), silu(p[3]));
        a[kk][2] = pack(silu(q[0]), silu(q[1]));
        a[kk][3] = pack(silu(q[2]), silu(q[3]));
        if (ds) {
            ds[kk][0] = pack(dsilu(p[0]), dsilu(p[1]));
            ds[kk][1] = pack(dsilu(p[2]), dsilu(p[3]));
            ds[kk][2] = pack(dsilu(q[0]), dsilu(q[1]));
            ds[kk][3] = pack(dsilu(q[2]), dsilu(q[3]));
        }
    }
}

// Layer 1 A fragment from standardised inputs: rows g and g+8 of the tile,
// columns 2t, 2t+1 (columns 8..15 are the zero padding).
__device__ __forceinline__ void input_frag(float x0g, float x1g, float x0h, float x1h,
                                           uint32_t (&a)[4]) {
    a[0] = pack(x0g, x1g);
    a[1] = pack(x0h, x1h);
    a[2] = 0u;
    a[3] = 0u;
}

// Hidden activations h1..h3 and silu' of the pre-activations, as packed A
// fragments, kept by the training forward pass for the backward pass.
struct Stash {
    uint32_t h[3][4][4];
    uint32_t ds[3][4][4];
};

// Forward pass of one 16-sample tile.  Returns z of row g (zr[0]) and row g+8
// (zr[1]) in the lanes with t == 0.
template <bool KEEP, class SM>
__device__ __forceinline__ void forward_tile(const SM &s, const uint32_t (&a1)[4], int g, int t,
                                             float (&zr)[2], Stash *st) {
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float u0 = s.b1[8 * nt + 2 * t], u1 = s.b1[8 * nt + 2 * t + 1];
        c[nt][0] = u0; c[nt][1] = u1; c[nt][2] = u0; c[nt][3] = u1;
        uint32_t b0, b1;
        bfrag(s.w1, kS1, 8 * nt, 0, g, t, b0, b1);
        mma16816(c[nt], a1, b0, b1);
    }
    uint32_t a[4][4];
#pragma unroll
    for (int layer = 0; layer < 3; ++layer) {
        activate(c, a, KEEP ? st->ds[layer] : nullptr);
        if (KEEP) {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                for (int e = 0; e < 4; ++e) st->h[layer][kk][e] = a[kk][e];
        }
        if (layer == 0) hidden(a, s.w2, s.b2, g, t, c);
        else if (layer == 1) hidden(a, s.w3, s.b3, g, t, c);
    }
    float o[4] = {t == 0 ? s.b4 : 0.0f, 0.0f, t == 0 ? s.b4 : 0.0f, 0.0f};
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        uint32_t b0, b1;
        bfrag(s.w4, kS, 0, 16 * kk, g, t, b0, b1);
        mma16816(o, a[kk], b0, b1);
    }
    zr[0] = o[0];
    zr[1] = o[2];
}

// z of every lane's own sample: each lane holds 8 standardised inputs; lanes
// 0..15 form tile 0, lanes 16..31 tile 1.  All 32 lanes must call.
template <class SM>
__device__ __forceinline__ float warp_forward(const SM &s, const float (&x)[kIn]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t p[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) p[q] = pack(x[2 * q], x[2 * q + 1]);
    float zmine = 0.0f;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        uint32_t a1[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t rg = __shfl_sync(0xffffffffu, p[q], 16 * m + g);
            const uint32_t rh = __shfl_sync(0xffffffffu, p[q], 16 * m + g + 8);
            if (q == t) { a1[0] = rg; a1[1] = rh; }
        }
        float zr[2];
        forward_tile<false>(s, a1, g, t, zr, nullptr);
        // row r of this tile sits in lane 4 (r % 8), slot r / 8
        const int r = lane & 15;
        const float z0 = __shfl_sync(0xffffffffu, zr[0], 4 * (r & 7));
        const float z1 = __shfl_sync(0xffffffffu, zr[1], 4 * (r & 7));
        if ((lane >> 4) == m) zmine = (r < 8) ? z0 : z1;
    }
    return zmine;
}

}  // namespace mma_mlp
}  // namespace gpat
