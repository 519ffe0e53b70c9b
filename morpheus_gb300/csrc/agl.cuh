// almost-Goldilocks field q = 2^64 - 2^32 - 31 (cuda_almost_goldilocks/almost_goldilocks.cuh)
// and the ChaCha8 matrix PRG of the Ajtai commitment
// (cuda_almost_goldilocks/ajtai_chacha8.cuh:60-178), device side.
#pragma once
#include "gl.cuh"

namespace gb {

constexpr u64 AGL_Q = 0xFFFFFFFEFFFFFFE1ull;
constexpr u64 AGL_C = 0x10000001Full;  // 2^64 mod q = 2^32 + 31

__host__ __device__ __forceinline__ u64 agl_canon(u64 a) { return a >= AGL_Q ? a - AGL_Q : a; }

__device__ __forceinline__ u64 agl_add(u64 a, u64 b) {
    u64 s = a + b;
    if (s < a) {
        s += AGL_C;
        if (s < AGL_C) s += AGL_C;
    }
    return s;
}
__device__ __forceinline__ u64 agl_sub(u64 a, u64 b) {
    u64 d = a - b;
    if (a < b) {
        u64 t = d - AGL_C;
        if (d < AGL_C) t -= AGL_C;
        d = t;
    }
    return d;
}
// x = lo + 2^64 hi == lo + c hi, applied until the high part vanishes
__device__ __forceinline__ u64 agl_reduce(u64 lo, u64 hi) {
    u64 p_lo = hi * AGL_C, p_hi = __umul64hi(hi, AGL_C);  // hi * c < 2^97
    u64 r = lo + p_lo;
    p_hi += (r < lo);
    // p_hi < 2^34: p_hi * c < 2^67 -> split once more
    u64 q_lo = p_hi * AGL_C, q_hi = __umul64hi(p_hi, AGL_C);
    u64 r2 = r + q_lo;
    q_hi += (r2 < r);
    return agl_add(r2, q_hi * AGL_C);
}
__device__ __forceinline__ u64 agl_mul(u64 a, u64 b) {
    u64 lo, hi;
    gl_mul128(a, b, lo, hi);
    return agl_reduce(lo, hi);
}

// Ext2 of the almost-Goldilocks field: c0 + c1 X, X^2 = 3 (cuda_almost_goldilocks/almost_extension.cuh:31-32)
struct ae2 {
    u64 c0, c1;
};
__device__ __forceinline__ ae2 ae2_make(u64 a, u64 b) {
    ae2 r;
    r.c0 = a;
    r.c1 = b;
    return r;
}
__device__ __forceinline__ ae2 ae2_add(ae2 a, ae2 b) { return ae2_make(agl_add(a.c0, b.c0), agl_add(a.c1, b.c1)); }
__device__ __forceinline__ ae2 ae2_sub(ae2 a, ae2 b) { return ae2_make(agl_sub(a.c0, b.c0), agl_sub(a.c1, b.c1)); }
// Karatsuba: three base multiplies
__device__ __forceinline__ ae2 ae2_mul(ae2 a, ae2 b) {
    u64 m0 = agl_mul(a.c0, b.c0), m1 = agl_mul(a.c1, b.c1);
    u64 m2 = agl_mul(agl_add(a.c0, a.c1), agl_add(b.c0, b.c1));
    u64 m1x3 = agl_add(agl_add(m1, m1), m1);
    return ae2_make(agl_add(m0, m1x3), agl_sub(agl_sub(m2, m0), m1));
}
__device__ __forceinline__ ae2 ae2_canon(ae2 a) { return ae2_make(agl_canon(a.c0), agl_canon(a.c1)); }

// ---------------------------------------------------------------------------
// ChaCha8 block: 8 rounds (4 double rounds) of the ChaCha quarter-round network over
// constants | key[8] | counter | nonce[3]; output = state + input.
// ---------------------------------------------------------------------------
__device__ __forceinline__ u32 rotl32(u32 x, int n) { return __funnelshift_l(x, x, n); }

#define GB_QR(a, b, c, d)                        \
    a += b; d ^= a; d = rotl32(d, 16);           \
    c += d; b ^= c; b = rotl32(b, 12);           \
    a += b; d ^= a; d = rotl32(d, 8);            \
    c += d; b ^= c; b = rotl32(b, 7);

__device__ __forceinline__ void chacha8_block_dev(const u32* key, u32 counter, u32 n0, u32 n1, u32 n2, u32* out) {
    u32 s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                 key[4],      key[5],      key[6],      key[7],      counter, n0, n1, n2};
    u32 x[16];
#pragma unroll
    for (int i = 0; i < 16; i++) x[i] = s[i];
#pragma unroll
    for (int dr = 0; dr < 4; dr++) {
        GB_QR(x[0], x[4], x[8], x[12]);
        GB_QR(x[1], x[5], x[9], x[13]);
        GB_QR(x[2], x[6], x[10], x[14]);
        GB_QR(x[3], x[7], x[11], x[15]);
        GB_QR(x[0], x[5], x[10], x[15]);
        GB_QR(x[1], x[6], x[11], x[12]);
        GB_QR(x[2], x[7], x[8], x[13]);
        GB_QR(x[3], x[4], x[9], x[14]);
    }
#pragma unroll
    for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}
#undef GB_QR

// 8 coefficients of M[row, j] (block blk of 8): the block's 8 words if all are < q,
// otherwise words < q taken in order from counters blk, blk + 8, blk + 16, ...
__device__ __forceinline__ void ajtai_prg_block(const u32* key, u32 row, u64 j, u32 blk, u64* out) {
    u32 buf[16];
    chacha8_block_dev(key, blk, row, (u32)j, (u32)(j >> 32), buf);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        out[k] = ((u64)buf[2 * k + 1] << 32) | buf[2 * k];
        ok = ok && out[k] < AGL_Q;
    }
    if (ok) return;
    int written = 0;
    for (int k = 0; k < 8; k++) out[k] = 0;
    for (u32 retry = 0; retry < 16 && written < 8; retry++) {
        chacha8_block_dev(key, blk + retry * 8u, row, (u32)j, (u32)(j >> 32), buf);
        for (int k = 0; k < 8 && written < 8; k++) {
            u64 v = ((u64)buf[2 * k + 1] << 32) | buf[2 * k];
            if (v < AGL_Q) out[written++] = v;
        }
    }
}

}  // namespace gb
