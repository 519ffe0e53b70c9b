// Per-pair device arithmetic of the product sumcheck, shared by the per-call driver
// (sumcheck.cu) and the round-synchronous batch engine (lockstep.cu).
#pragma once
#include "gl.cuh"

namespace gb {

__device__ __forceinline__ bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

// Pair (p[0], p[1]) of base elements; vector load when the address allows it.
__device__ __forceinline__ void ld_pair(const u64* p, bool vec, u64& a, u64& b) {
    if (vec) {
        ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p));
        a = v.x;
        b = v.y;
    } else {
        a = __ldg(p);
        b = __ldg(p + 1);
    }
}
__device__ __forceinline__ e2 ld_e2(const u64* p, bool vec) {
    if (vec) {
        ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(p));
        return e2_make(v.x, v.y);
    }
    return e2_make(__ldg(p), __ldg(p + 1));
}
__device__ __forceinline__ void st_e2(u64* p, e2 a, bool vec) {
    if (vec) e2_st(p, a);
    else {
        p[0] = a.c0;
        p[1] = a.c1;
    }
}

// Accumulate prod_i (e_i + c delta_i) for c = 0..D into acc (base field).
template <int D>
__device__ __forceinline__ void accum_base(const u64 (&e)[D], const u64 (&dl)[D], u64 (&acc)[D + 1]) {
    u64 v[D];
#pragma unroll
    for (int i = 0; i < D; i++) v[i] = e[i];
#pragma unroll
    for (int c = 0; c <= D; c++) {
        u64 prod = v[0];
#pragma unroll
        for (int i = 1; i < D; i++) prod = gl_mul(prod, v[i]);
        acc[c] = gl_add(acc[c], prod);
        if (c < D) {
#pragma unroll
            for (int i = 0; i < D; i++) v[i] = gl_add(v[i], dl[i]);
        }
    }
}

// Same over Ext2; acc is laid out [c][c0, c1].
template <int D>
__device__ __forceinline__ void accum_e2(const e2 (&e)[D], const e2 (&dl)[D], u64 (&acc)[2 * (D + 1)]) {
    e2 v[D];
#pragma unroll
    for (int i = 0; i < D; i++) v[i] = e[i];
#pragma unroll
    for (int c = 0; c <= D; c++) {
        e2 prod = v[0];
#pragma unroll
        for (int i = 1; i < D; i++) prod = e2_mul(prod, v[i]);
        acc[2 * c] = gl_add(acc[2 * c], prod.c0);
        acc[2 * c + 1] = gl_add(acc[2 * c + 1], prod.c1);
        if (c < D) {
#pragma unroll
            for (int i = 0; i < D; i++) v[i] = e2_add(v[i], dl[i]);
        }
    }
}

}  // namespace gb
