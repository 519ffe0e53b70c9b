// Goldilocks (p = 2^64 - 2^32 + 1) and its quadratic extension F_p[X]/(X^2 - 7)
// on the device.
//
// Representation: any u64 in [0, 2^64) congruent to the value (the "non-canonical"
// form the reference kernels use, cuda/goldilocks.cuh:182-311).
// Values leave the device canonicalised only where a caller compares or
// hashes them on the host; inside kernels the cheaper non-canonical form is kept.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gb {

typedef uint64_t u64;
typedef uint32_t u32;

constexpr u64 GL_P = 0xFFFFFFFF00000001ull;
constexpr u64 GL_EPS = 0xFFFFFFFFull;  // 2^64 mod p

__host__ __device__ __forceinline__ u64 gl_canon(u64 a) { return a >= GL_P ? a - GL_P : a; }

// a + b; a carry out of 2^64 is worth 2^64 - p = EPS.  A second carry is possible only
// when both inputs are non-canonical and close to 2^64.
__device__ __forceinline__ u64 gl_add(u64 a, u64 b) {
    u64 s = a + b;
    if (s < a) {
        s += GL_EPS;
        if (s < GL_EPS) s += GL_EPS;
    }
    return s;
}

__device__ __forceinline__ u64 gl_sub(u64 a, u64 b) {
    u64 d = a - b;
    if (a < b) {
        u64 t = d - GL_EPS;
        if (d < GL_EPS) t -= GL_EPS;
        d = t;
    }
    return d;
}

__device__ __forceinline__ u64 gl_neg(u64 a) {
    a = gl_canon(a);
    return a ? GL_P - a : 0;
}

// 128-bit x = lo + 2^64 (h1 2^32 + h0) == lo - h1 + h0 (2^32 - 1)   (2^96 == -1 mod p)
__device__ __forceinline__ u64 gl_reduce(u64 lo, u64 hi) {
    u64 h1 = hi >> 32;
    u64 h0 = hi & GL_EPS;
    u64 t0 = lo - h1;
    if (lo < h1) t0 -= GL_EPS;
    u64 t1 = (h0 << 32) - h0;
    u64 r = t0 + t1;
    if (r < t1) r += GL_EPS;
    return r;
}

__device__ __forceinline__ u64 gl_mul(u64 a, u64 b) { return gl_reduce(a * b, __umul64hi(a, b)); }

// x^2 from 32-bit limbs: x0^2 + 2 x0 x1 2^32 + x1^2 2^64 (three wide multiplies).
__device__ __forceinline__ u64 gl_sqr(u64 x) {
    u32 x0 = (u32)x, x1 = (u32)(x >> 32);
    u64 p00 = (u64)x0 * x0;
    u64 p01 = (u64)x0 * x1;
    u64 p11 = (u64)x1 * x1;
    // cross = 2 * p01 is up to 65 bits
    u64 c_lo = p01 << 33;
    u64 c_hi = p01 >> 31;
    u64 lo = p00 + c_lo;
    u64 hi = p11 + c_hi + (lo < p00 ? 1ull : 0ull);
    return gl_reduce(lo, hi);
}

// 7 a = 8 a - a; the three bits shifted out of 8a are worth EPS each.
__device__ __forceinline__ u64 gl_mul7(u64 a) {
    u64 ovf = a >> 61;
    u64 eight = gl_add(a << 3, ovf * GL_EPS);
    return gl_sub(eight, a);
}

__device__ __forceinline__ u64 gl_double(u64 a) { return gl_add(a, a); }

__device__ __forceinline__ u64 gl_pow(u64 a, u64 e) {
    u64 r = 1;
    while (e) {
        if (e & 1) r = gl_mul(r, a);
        a = gl_sqr(a);
        e >>= 1;
    }
    return r;
}

// Fermat inverse; 0 maps to 0
__device__ __forceinline__ u64 gl_inv(u64 a) { return gl_pow(a, GL_P - 2); }

// ---------------------------------------------------------------------------
// Ext2: c0 + c1 X, X^2 = 7
// ---------------------------------------------------------------------------
struct e2 {
    u64 c0, c1;
};

__device__ __forceinline__ e2 e2_make(u64 c0, u64 c1) {
    e2 r;
    r.c0 = c0;
    r.c1 = c1;
    return r;
}
__device__ __forceinline__ e2 e2_add(e2 a, e2 b) { return e2_make(gl_add(a.c0, b.c0), gl_add(a.c1, b.c1)); }
__device__ __forceinline__ e2 e2_sub(e2 a, e2 b) { return e2_make(gl_sub(a.c0, b.c0), gl_sub(a.c1, b.c1)); }
// Karatsuba: three base multiplies
__device__ __forceinline__ e2 e2_mul(e2 a, e2 b) {
    u64 m0 = gl_mul(a.c0, b.c0);
    u64 m1 = gl_mul(a.c1, b.c1);
    u64 m2 = gl_mul(gl_add(a.c0, a.c1), gl_add(b.c0, b.c1));
    return e2_make(gl_add(m0, gl_mul7(m1)), gl_sub(gl_sub(m2, m0), m1));
}
__device__ __forceinline__ e2 e2_mul_base(e2 a, u64 s) { return e2_make(gl_mul(a.c0, s), gl_mul(a.c1, s)); }
__device__ __forceinline__ e2 e2_canon(e2 a) { return e2_make(gl_canon(a.c0), gl_canon(a.c1)); }
__device__ __forceinline__ e2 e2_zero() { return e2_make(0, 0); }

// 128-bit vector load/store of one Ext2 element (16-byte aligned)
__device__ __forceinline__ e2 e2_ld(const u64* p) {
    ulonglong2 v = *reinterpret_cast<const ulonglong2*>(p);
    return e2_make(v.x, v.y);
}
__device__ __forceinline__ void e2_st(u64* p, e2 a) {
    ulonglong2 v;
    v.x = a.c0;
    v.y = a.c1;
    *reinterpret_cast<ulonglong2*>(p) = v;
}

// warp reduction of one field element (lane 0 ends with the sum)
__device__ __forceinline__ u64 gl_warp_sum(u64 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = gl_add(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace gb
