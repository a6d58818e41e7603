// Device helpers shared by the kernels: Philox-4x32-10, 53-bit uniforms,
// exact 128-bit fixed-point accumulation, warp reductions.
#pragma once

#include <cstdint>

#include "gpat_internal.h"

namespace gpat {

// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies with a
// Weyl key schedule.
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    }
    return c;
}

// 53-bit uniform on [0,1) from two words.
__device__ __forceinline__ double u01_53(uint32_t a, uint32_t b) {
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// 24-bit uniform on [0,1) from one word (FP32 paths).
__device__ __forceinline__ float u01_24(uint32_t a) {
    return (float)(a >> 8) * (1.0f / 16777216.0f);
}

// Splits w >= 0 into 64.64 fixed point; truncates below 2^-64.
__device__ __forceinline__ void fixed_split(double w, unsigned long long &h, unsigned long long &l) {
    const double fl = floor(w);
    h = (unsigned long long)fl;
    l = __double2ull_rz((w - fl) * 18446744073709551616.0);
}

// Exact modular 128-bit atomic add (global or shared memory).
__device__ __forceinline__ void atomic_add_u128(unsigned long long *hi, unsigned long long *lo,
                                                unsigned long long h, unsigned long long l) {
    if (l) {
        const unsigned long long old = atomicAdd(lo, l);
        if (old + l < old) h += 1ull;
    }
    if (h) atomicAdd(hi, h);
}

__device__ __forceinline__ void atomic_add_fixed(unsigned long long *hi, unsigned long long *lo,
                                                 double w) {
    unsigned long long h, l;
    fixed_split(w, h, l);
    atomic_add_u128(hi, lo, h, l);
}

__device__ __forceinline__ void add_u128(unsigned long long &h, unsigned long long &l,
                                         unsigned long long bh, unsigned long long bl) {
    const unsigned long long o = l;
    l += bl;
    h += bh + (l < o ? 1ull : 0ull);
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// 128-bit sum over the full warp (every lane gets the total).
__device__ __forceinline__ void warp_sum_u128(unsigned long long &h, unsigned long long &l) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long oh = __shfl_xor_sync(0xffffffffu, h, o);
        const unsigned long long ol = __shfl_xor_sync(0xffffffffu, l, o);
        add_u128(h, l, oh, ol);
    }
}

__device__ __forceinline__ void set_status(DevCounters *c, unsigned int bit) {
    atomicOr(&c->status, bit);
}

}  // namespace gpat
