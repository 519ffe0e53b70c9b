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

// Full 64 x 64 -> 128-bit product from 32-bit multiply-adds with carry chains (full-rate
// IMAD work; the 64-bit multiply-high would go through the slower wide-multiply path).
__device__ __forceinline__ void gl_mul128(u64 a, u64 b, u64& lo, u64& hi) {
    u32 a0 = (u32)a, a1 = (u32)(a >> 32), b0 = (u32)b, b1 = (u32)(b >> 32);
    u32 r0, r1, r2, r3;
    asm("{\n\t"
        "mul.lo.u32 %0, %4, %6;\n\t"
        "mul.hi.u32 %1, %4, %6;\n\t"
        "mad.lo.cc.u32 %1, %4, %7, %1;\n\t"
        "madc.hi.u32 %2, %4, %7, 0;\n\t"
        "mad.lo.cc.u32 %1, %5, %6, %1;\n\t"
        "madc.hi.cc.u32 %2, %5, %6, %2;\n\t"
        "madc.hi.u32 %3, %5, %7, 0;\n\t"
        "mad.lo.cc.u32 %2, %5, %7, %2;\n\t"
        "addc.u32 %3, %3, 0;\n\t"
        "}"
        : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
        : "r"(a0), "r"(a1), "r"(b0), "r"(b1));
    lo = ((u64)r1 << 32) | r0;
    hi = ((u64)r3 << 32) | r2;
}

// 128-bit x = lo + 2^64 (h1 2^32 + h0) == lo - h1 + h0 (2^32 - 1)   (2^96 == -1 mod p),
// with 32-bit carry chains: a borrow of lo - h1 is worth -EPS, a carry of the final sum +EPS
// (neither correction can wrap again).  Any (lo, hi) in, a u64 congruent to x out.
__device__ __forceinline__ u64 gl_reduce(u64 lo, u64 hi) {
    u32 l0 = (u32)lo, l1 = (u32)(lo >> 32), h0 = (u32)hi, h1 = (u32)(hi >> 32);
    u32 s0, s1;
    asm("{\n\t.reg .u32 b, t0, t1, c, m;\n\t"
        "sub.cc.u32 %0, %2, %5;\n\t"
        "subc.cc.u32 %1, %3, 0;\n\t"
        "subc.u32 b, 0, 0;\n\t"
        "sub.cc.u32 %0, %0, b;\n\t"
        "subc.u32 %1, %1, 0;\n\t"
        "sub.cc.u32 t0, 0, %4;\n\t"
        "subc.u32 t1, %4, 0;\n\t"
        "add.cc.u32 %0, %0, t0;\n\t"
        "addc.cc.u32 %1, %1, t1;\n\t"
        "addc.u32 c, 0, 0;\n\t"
        "sub.u32 m, 0, c;\n\t"
        "add.cc.u32 %0, %0, m;\n\t"
        "addc.u32 %1, %1, 0;\n\t}"
        : "=r"(s0), "=r"(s1)
        : "r"(l0), "r"(l1), "r"(h0), "r"(h1));
    return ((u64)s1 << 32) | s0;
}

__device__ __forceinline__ u64 gl_mul(u64 a, u64 b) {
    u64 lo, hi;
    gl_mul128(a, b, lo, hi);
    return gl_reduce(lo, hi);
}

// x^2 = a0^2 + 2 a0 a1 2^32 + a1^2 2^64 (x = a1 2^32 + a0): the cross product once, doubled by
// shifts, so 6 multiply-adds instead of 8 and three more ALU steps.  The one-thread Poseidon2
// kernels are bound by the multiply-add (fmaheavy) pipe with the ALU pipe below it, so the trade
// pays there.
__device__ __forceinline__ void gl_sqr128(u64 x, u64& lo, u64& hi) {
    u32 a0 = (u32)x, a1 = (u32)(x >> 32);
    u32 r0, r1, r2, r3;
    asm("{\n\t.reg .u32 c0, c1, d0, d1, d2;\n\t"
        "mul.lo.u32 c0, %4, %5;\n\t"
        "mul.hi.u32 c1, %4, %5;\n\t"
        "shl.b32 d0, c0, 1;\n\t"
        "shf.l.wrap.b32 d1, c0, c1, 1;\n\t"
        "shr.u32 d2, c1, 31;\n\t"
        "mul.lo.u32 %0, %4, %4;\n\t"
        "mul.hi.u32 %1, %4, %4;\n\t"
        "add.cc.u32 %1, %1, d0;\n\t"
        "madc.lo.cc.u32 %2, %5, %5, d1;\n\t"
        "madc.hi.u32 %3, %5, %5, d2;\n\t"
        "}"
        : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
        : "r"(a0), "r"(a1));
    lo = ((u64)r1 << 32) | r0;
    hi = ((u64)r3 << 32) | r2;
}

__device__ __forceinline__ u64 gl_sqr(u64 x) {
    u64 lo, hi;
    gl_sqr128(x, lo, hi);
    return gl_reduce(lo, hi);
}

// ---------------------------------------------------------------------------
// Lazy sums: lo + 2^64 hi with a small hi, reduced once (linear layers, dot products).
// ---------------------------------------------------------------------------
struct glw {
    u64 lo;
    u32 hi;
};
__device__ __forceinline__ glw glw_of(u64 x) {
    glw r;
    r.lo = x;
    r.hi = 0u;
    return r;
}
__device__ __forceinline__ glw glw_add(glw a, glw b) {
    glw r;
    asm("add.cc.u64 %0, %2, %4;\n\taddc.u32 %1, %3, %5;"
        : "=l"(r.lo), "=r"(r.hi)
        : "l"(a.lo), "r"(a.hi), "l"(b.lo), "r"(b.hi));
    return r;
}
__device__ __forceinline__ glw glw_add(glw a, u64 b) {
    glw r;
    asm("add.cc.u64 %0, %2, %4;\n\taddc.u32 %1, %3, 0;" : "=l"(r.lo), "=r"(r.hi) : "l"(a.lo), "r"(a.hi), "l"(b));
    return r;
}
// lo + hi EPS for hi < 2^32: one carry at most, worth EPS, after which no carry is possible
// (the wrapped sum is below hi EPS <= 2^64 - 2^32)
__device__ __forceinline__ u64 glw_reduce(glw a) {
    u64 t = ((u64)a.hi << 32) - a.hi;
    u64 r;
    u32 c;
    asm("add.cc.u64 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=l"(r), "=r"(c) : "l"(a.lo), "l"(t));
    return r + (u64)(0u - c);
}
// Three-word lazy sums of full 128-bit products: lo + 2^64 hi + 2^128 top.
// 2^128 == -2^32 (mod p) (2^64 == 2^32 - 1, squared), so the value reduces to
// gl_reduce(lo, hi) - top 2^32.
struct gl3 {
    u64 lo, hi;
    u32 top;
};
__device__ __forceinline__ gl3 gl3_zero() {
    gl3 r;
    r.lo = r.hi = 0;
    r.top = 0;
    return r;
}
__device__ __forceinline__ void gl3_add_prod(gl3& a, u64 x, u64 y) {
    u64 lo, hi;
    gl_mul128(x, y, lo, hi);
    asm("add.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, %4;\n\taddc.u32 %2, %2, 0;"
        : "+l"(a.lo), "+l"(a.hi), "+r"(a.top)
        : "l"(lo), "l"(hi));
}
__device__ __forceinline__ void gl3_add(gl3& a, u64 x) {
    asm("add.cc.u64 %0, %0, %3;\n\taddc.cc.u64 %1, %1, 0;\n\taddc.u32 %2, %2, 0;"
        : "+l"(a.lo), "+l"(a.hi), "+r"(a.top)
        : "l"(x));
}
// lo + 2^64 (h1 2^32 + h0) + 2^128 top == lo - (top 2^32 + h1) + h0 (2^32 - 1)  (2^128 == -2^32):
// gl_reduce with the top word as the high half of the subtracted word.  For top <= 2^32 - 2 a
// borrow still leaves at least EPS, so one -EPS correction remains enough.
__device__ __forceinline__ u64 gl3_reduce(gl3 a) {
    u32 l0 = (u32)a.lo, l1 = (u32)(a.lo >> 32), h0 = (u32)a.hi, h1 = (u32)(a.hi >> 32);
    u32 s0, s1;
    asm("{\n\t.reg .u32 b, t0, t1, c, m;\n\t"
        "sub.cc.u32 %0, %2, %5;\n\t"
        "subc.cc.u32 %1, %3, %6;\n\t"
        "subc.u32 b, 0, 0;\n\t"
        "sub.cc.u32 %0, %0, b;\n\t"
        "subc.u32 %1, %1, 0;\n\t"
        "sub.cc.u32 t0, 0, %4;\n\t"
        "subc.u32 t1, %4, 0;\n\t"
        "add.cc.u32 %0, %0, t0;\n\t"
        "addc.cc.u32 %1, %1, t1;\n\t"
        "addc.u32 c, 0, 0;\n\t"
        "sub.u32 m, 0, c;\n\t"
        "add.cc.u32 %0, %0, m;\n\t"
        "addc.u32 %1, %1, 0;\n\t}"
        : "=r"(s0), "=r"(s1)
        : "r"(l0), "r"(l1), "r"(h0), "r"(h1), "r"(a.top));
    return ((u64)s1 << 32) | s0;
}

// a b + c reduced, for b < p: the product's high word is then below 2^64 - 2^32, so adding
// c (hi < 2^32) cannot carry out of 128 bits
__device__ __forceinline__ u64 gl_mul_add(u64 a, u64 b, glw c) {
    u64 lo, hi;
    gl_mul128(a, b, lo, hi);
    asm("add.cc.u64 %0, %0, %2;\n\taddc.u64 %1, %1, %3;" : "+l"(lo), "+l"(hi) : "l"(c.lo), "l"((u64)c.hi));
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
