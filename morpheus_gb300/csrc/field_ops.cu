// Element-wise batch field operations of the two crates' ABI (goldilocks-cuda-rs/src/ffi.rs:105-131,
// :163-265, :633-639; almost-goldilocks-cuda-rs/src/ffi.rs:95-140; goldilocks-cuda-rs/cuda/wrapper.cu
// :180-858, :1790-1815; almost wrapper.cu:420-640) over
//   Goldilocks p = 2^64 - 2^32 + 1:  base, Ext2 = F_p[X]/(X^2 - 7), Ext5 = F_p[X]/(X^5 - 3)
//   almost-Goldilocks q = 2^64 - 2^32 - 31:  base, Ext2 = F_q[X]/(X^2 - 3)
// (cuda/extension.cuh, cuda_almost_goldilocks/almost_extension.cuh).  One thread per element,
// canonical outputs.  Inverses of zero are zero (Fermat / norm-based, as the reference).
// add, sub, mul and inverse of the Goldilocks base and Ext2 forms are in runtime.cu.
#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "../../include/goldilocks_cuda_wrapper.h"
#include "agl.cuh"
#include "common.cuh"
#include "gl.cuh"

namespace gb {

// ---------------------------------------------------------------- base fields
struct BGl {
    static __device__ __forceinline__ u64 add(u64 a, u64 b) { return gl_add(a, b); }
    static __device__ __forceinline__ u64 sub(u64 a, u64 b) { return gl_sub(a, b); }
    static __device__ __forceinline__ u64 mul(u64 a, u64 b) { return gl_mul(a, b); }
    static __device__ __forceinline__ u64 canon(u64 a) { return gl_canon(a); }
    static __device__ __forceinline__ u64 neg(u64 a) { return gl_neg(a); }
    static __device__ __forceinline__ u64 inv(u64 a) { return gl_inv(gl_canon(a)); }
};
struct BAgl {
    static __device__ __forceinline__ u64 add(u64 a, u64 b) { return agl_add(a, b); }
    static __device__ __forceinline__ u64 sub(u64 a, u64 b) { return agl_sub(a, b); }
    static __device__ __forceinline__ u64 mul(u64 a, u64 b) { return agl_mul(a, b); }
    static __device__ __forceinline__ u64 canon(u64 a) { return agl_canon(a); }
    static __device__ __forceinline__ u64 neg(u64 a) {
        a = agl_canon(a);
        return a ? AGL_Q - a : 0;
    }
    static __device__ __forceinline__ u64 inv(u64 a) {  // a^(q - 2)
        u64 r = 1, b = agl_canon(a), e = AGL_Q - 2;
        while (e) {
            if (e & 1) r = agl_mul(r, b);
            b = agl_mul(b, b);
            e >>= 1;
        }
        return r;
    }
};

// ---------------------------------------------------------------- elements of degree D over B
// X^D = NR; FROB[i] = NR^(i (p - 1) / D), the Frobenius a -> a^p acting on coefficient i.
template <class B, int D, u64 NR>
struct Ext {
    u64 c[D];
    static constexpr int W = D;
    static __device__ __forceinline__ Ext ld(const u64* p, size_t i) {
        Ext x;
#pragma unroll
        for (int k = 0; k < D; k++) x.c[k] = p[D * i + k];
        return x;
    }
    __device__ __forceinline__ void st(u64* p, size_t i) const {
#pragma unroll
        for (int k = 0; k < D; k++) p[D * i + k] = B::canon(c[k]);
    }
    static __device__ __forceinline__ Ext one() {
        Ext x;
#pragma unroll
        for (int k = 0; k < D; k++) x.c[k] = k == 0;
        return x;
    }
    friend __device__ __forceinline__ Ext operator+(Ext a, Ext b) {
#pragma unroll
        for (int k = 0; k < D; k++) a.c[k] = B::add(a.c[k], b.c[k]);
        return a;
    }
    friend __device__ __forceinline__ Ext operator-(Ext a, Ext b) {
#pragma unroll
        for (int k = 0; k < D; k++) a.c[k] = B::sub(a.c[k], b.c[k]);
        return a;
    }
    __device__ __forceinline__ Ext neg() const {
        Ext r;
#pragma unroll
        for (int k = 0; k < D; k++) r.c[k] = B::neg(c[k]);
        return r;
    }
    __device__ __forceinline__ Ext scale(u64 s) const {
        Ext r;
#pragma unroll
        for (int k = 0; k < D; k++) r.c[k] = B::mul(c[k], s);
        return r;
    }
    // schoolbook product, the wrapped terms times NR
    friend __device__ __forceinline__ Ext operator*(Ext a, Ext b) {
        Ext r;
#pragma unroll
        for (int k = 0; k < D; k++) {
            u64 lo = 0, hi = 0;
#pragma unroll
            for (int i = 0; i < D; i++) {
                const int j = k - i;
                if (j >= 0) lo = B::add(lo, B::mul(a.c[i], b.c[j]));
                else hi = B::add(hi, B::mul(a.c[i], b.c[j + D]));
            }
            r.c[k] = B::add(lo, B::mul(hi, NR));
        }
        return r;
    }
    __device__ __forceinline__ Ext frob(const u64* fr) const {
        Ext r;
#pragma unroll
        for (int k = 0; k < D; k++) r.c[k] = k ? B::mul(c[k], fr[k]) : c[k];
        return r;
    }
    // a^-1 = a^(p + ... + p^(D-1)) / N(a), N(a) = a^(1 + p + ... + p^(D-1)) in the base field
    __device__ __forceinline__ Ext inv(const u64* fr) const {
        if (D == 1) {
            Ext r;
            r.c[0] = B::inv(c[0]);
            return r;
        }
        Ext conj = frob(fr), f = conj;
        for (int k = 2; k < D; k++) {
            f = f.frob(fr);
            conj = conj * f;
        }
        const u64 n = ((*this) * conj).c[0];
        return conj.scale(B::inv(n));
    }
    __device__ __forceinline__ Ext pow(u64 e) const {
        Ext r = one(), b = *this;
        while (e) {
            if (e & 1) r = r * b;
            b = b * b;
            e >>= 1;
        }
        return r;
    }
};

using GlE2 = Ext<BGl, 2, 7>;
using GlE5 = Ext<BGl, 5, 3>;
using AglE2 = Ext<BAgl, 2, 3>;
using GlE1 = Ext<BGl, 1, 0>;
using AglE1 = Ext<BAgl, 1, 0>;

// Frobenius multipliers: -1 for both quadratic extensions (7 and 3 are non-residues), and the
// powers of 3^((p - 1)/5) for Ext5 (the test suite checks these against the definition)
__constant__ u64 c_frob_gl2[2] = {1, GL_P - 1};
__constant__ u64 c_frob_agl2[2] = {1, AGL_Q - 1};
__constant__ u64 c_frob_gl5[5] = {1, 1041288259238279555ull, 15820824984080659046ull, 211587555138949697ull,
                                  1373043270956696022ull};
__constant__ u64 c_frob_none[1] = {1};

template <class T>
__device__ __forceinline__ const u64* frob_table();
template <>
__device__ __forceinline__ const u64* frob_table<GlE2>() { return c_frob_gl2; }
template <>
__device__ __forceinline__ const u64* frob_table<GlE5>() { return c_frob_gl5; }
template <>
__device__ __forceinline__ const u64* frob_table<AglE2>() { return c_frob_agl2; }
template <>
__device__ __forceinline__ const u64* frob_table<GlE1>() { return c_frob_none; }
template <>
__device__ __forceinline__ const u64* frob_table<AglE1>() { return c_frob_none; }

enum EwOp { EW_ADD, EW_SUB, EW_MUL, EW_DIV, EW_NEG, EW_SQR, EW_DBL, EW_INV, EW_EXP, EW_MULS, EW_FROB, EW_CONJ, EW_SACC };

template <class T, int OP>
__global__ void ew_kernel(const u64* __restrict__ a, const u64* __restrict__ b, u64 s0, u64 s1, u64* __restrict__ r,
                          size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const T x = T::ld(a, i);
        T z;
        if constexpr (OP == EW_ADD) z = x + T::ld(b, i);
        else if constexpr (OP == EW_SUB) z = x - T::ld(b, i);
        else if constexpr (OP == EW_MUL) z = x * T::ld(b, i);
        else if constexpr (OP == EW_DIV) z = x * T::ld(b, i).inv(frob_table<T>());
        else if constexpr (OP == EW_NEG) z = x.neg();
        else if constexpr (OP == EW_SQR) z = x * x;
        else if constexpr (OP == EW_DBL) z = x + x;
        else if constexpr (OP == EW_INV) z = x.inv(frob_table<T>());
        else if constexpr (OP == EW_EXP) z = x.pow(s0);
        else if constexpr (OP == EW_MULS) z = x.scale(s0);
        else if constexpr (OP == EW_FROB || OP == EW_CONJ) z = x.frob(frob_table<T>());  // quadratic: a0 - a1 X
        else {  // EW_SACC (quadratic): r += (s0 + s1 X) x
            static_assert(T::W == 2, "scale-accumulate is the Ext2 form");
            T s;
            s.c[0] = s0;
            s.c[1] = s1;
            z = T::ld(r, i) + s * x;
        }
        z.st(r, i);
    }
}

template <class T, int OP>
static int ew(const u64* a, const u64* b, u64 s0, u64 s1, u64* r, int n, const char* name) {
    if (n < 0 || (n > 0 && (!a || !r))) return GB_EINVAL;
    if (n == 0) return GB_OK;
    ew_kernel<T, OP><<<grid_for((size_t)n, 256), 256, 0, stream()>>>(a, b, s0, s1, r, (size_t)n);
    return check_launch(name);
}

// base <-> extension: lift (c0 = v, the rest 0) or take c0
__global__ void ew_lift_kernel(const u64* __restrict__ in, u64* __restrict__ out, int w, size_t n, bool to_ext, u64 q) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (to_ext) {
            const u64 v = in[i];
            out[w * i] = v >= q ? v - q : v;
            for (int k = 1; k < w; k++) out[w * i + k] = 0;
        } else {
            const u64 v = in[w * i];
            out[i] = v >= q ? v - q : v;
        }
    }
}
static int ew_lift(const u64* in, u64* out, int w, int n, bool to_ext, u64 q, const char* name) {
    if (n < 0 || (n > 0 && (!in || !out))) return GB_EINVAL;
    if (n == 0) return GB_OK;
    ew_lift_kernel<<<grid_for((size_t)n, 256), 256, 0, stream()>>>(in, out, w, (size_t)n, to_ext, q);
    return check_launch(name);
}

static int zero_words(void* p, size_t words) {
    if (!p && words) return GB_EINVAL;
    if (!words) return GB_OK;
    GB_CUDA_TRY(cudaMemsetAsync(p, 0, words * 8, stream()));
    return GB_OK;
}

}  // namespace gb

using namespace gb;

#define EW1(NAME, T, OP) \
    int NAME(const uint64_t* a, uint64_t* r, int n) { return ew<T, OP>(a, nullptr, 0, 0, r, n, #NAME); }
#define EW2(NAME, T, OP) \
    int NAME(const uint64_t* a, const uint64_t* b, uint64_t* r, int n) { return ew<T, OP>(a, b, 0, 0, r, n, #NAME); }
#define EWS(NAME, T, OP) \
    int NAME(uint64_t s, const uint64_t* a, uint64_t* r, int n) { return ew<T, OP>(a, nullptr, s, 0, r, n, #NAME); }
#define EWE(NAME, T, OP) \
    int NAME(const uint64_t* a, uint64_t e, uint64_t* r, int n) { return ew<T, OP>(a, nullptr, e, 0, r, n, #NAME); }

extern "C" {

// ---- Goldilocks base (ffi.rs:163-183) ----
EW2(gl_batch_div, GlE1, EW_DIV)
EWS(gl_batch_mul_scalar, GlE1, EW_MULS)
EW1(gl_batch_neg, GlE1, EW_NEG)
EW1(gl_batch_square, GlE1, EW_SQR)
EW1(gl_batch_double, GlE1, EW_DBL)
EWE(gl_batch_exp, GlE1, EW_EXP)
// ---- Goldilocks Ext2 (ffi.rs:214-230) ----
EW1(ext2_batch_inverse_ffi, GlE2, EW_INV)
EWS(ext2_batch_mul_scalar_ffi, GlE2, EW_MULS)
EW1(ext2_batch_neg_ffi, GlE2, EW_NEG)
EW1(ext2_batch_square_ffi, GlE2, EW_SQR)
EW1(ext2_batch_frobenius_ffi, GlE2, EW_FROB)
EW1(ext2_batch_conjugate_ffi, GlE2, EW_CONJ)
EWE(ext2_batch_exp_ffi, GlE2, EW_EXP)
int ext2_scale_accumulate_ffi(uint64_t s0, uint64_t s1, const uint64_t* d_src, uint64_t* d_acc, int n) {
    return ew<GlE2, EW_SACC>(d_src, nullptr, s0, s1, d_acc, n, "ext2_scale_accumulate_ffi");
}
// ---- Goldilocks Ext5 (ffi.rs:236-270) ----
EW2(ext5_batch_add_ffi, GlE5, EW_ADD)
EW2(ext5_batch_sub_ffi, GlE5, EW_SUB)
EW2(ext5_batch_mul_ffi, GlE5, EW_MUL)
EW1(ext5_batch_inverse_ffi, GlE5, EW_INV)
EWS(ext5_batch_mul_scalar_ffi, GlE5, EW_MULS)
EW1(ext5_batch_neg_ffi, GlE5, EW_NEG)
EW1(ext5_batch_square_ffi, GlE5, EW_SQR)
EW1(ext5_batch_frobenius_ffi, GlE5, EW_FROB)
EWE(ext5_batch_exp_ffi, GlE5, EW_EXP)
// ---- conversions (ffi.rs:274-280) ----
int gl_to_ext2_batch_ffi(const uint64_t* in, uint64_t* out, int n) { return ew_lift(in, out, 2, n, true, GL_P, "gl_to_ext2_batch_ffi"); }
int ext2_to_gl_batch_ffi(const uint64_t* in, uint64_t* out, int n) { return ew_lift(in, out, 2, n, false, GL_P, "ext2_to_gl_batch_ffi"); }
int gl_to_ext5_batch_ffi(const uint64_t* in, uint64_t* out, int n) { return ew_lift(in, out, 5, n, true, GL_P, "gl_to_ext5_batch_ffi"); }
int ext5_to_gl_batch_ffi(const uint64_t* in, uint64_t* out, int n) { return ew_lift(in, out, 5, n, false, GL_P, "ext5_to_gl_batch_ffi"); }
// ---- buffers (ffi.rs:105, :131) ----
int gl_memset_zero(uint64_t* d_buf, size_t n_u64) { return zero_words(d_buf, n_u64); }
int gl_zero_buffer(uint64_t* d_buf, int n) { return n < 0 ? GB_EINVAL : zero_words(d_buf, (size_t)n); }

// ---- almost-Goldilocks base and Ext2 (almost-goldilocks-cuda-rs/src/ffi.rs:95-140) ----
EW2(agl_batch_add_ffi, AglE1, EW_ADD)
EW2(agl_batch_sub_ffi, AglE1, EW_SUB)
EW2(agl_batch_mul_ffi, AglE1, EW_MUL)
EW2(agl_batch_div_ffi, AglE1, EW_DIV)
EW1(agl_batch_inverse_ffi, AglE1, EW_INV)
EWS(agl_batch_mul_scalar_ffi, AglE1, EW_MULS)
EW1(agl_batch_neg_ffi, AglE1, EW_NEG)
EW1(agl_batch_square_ffi, AglE1, EW_SQR)
EW1(agl_batch_double_ffi, AglE1, EW_DBL)
EWE(agl_batch_exp_ffi, AglE1, EW_EXP)
EW2(aext2_batch_add_ffi, AglE2, EW_ADD)
EW2(aext2_batch_sub_ffi, AglE2, EW_SUB)
EW2(aext2_batch_mul_ffi, AglE2, EW_MUL)
EW1(aext2_batch_inverse_ffi, AglE2, EW_INV)
EWS(aext2_batch_mul_scalar_ffi, AglE2, EW_MULS)
EW1(aext2_batch_neg_ffi, AglE2, EW_NEG)
EW1(aext2_batch_square_ffi, AglE2, EW_SQR)
EW1(aext2_batch_frobenius_ffi, AglE2, EW_FROB)
EW1(aext2_batch_conjugate_ffi, AglE2, EW_CONJ)
EWE(aext2_batch_exp_ffi, AglE2, EW_EXP)
int aext2_scale_accumulate_ffi(uint64_t s0, uint64_t s1, const uint64_t* d_src, uint64_t* d_acc, int n) {
    return ew<AglE2, EW_SACC>(d_src, nullptr, s0, s1, d_acc, n, "aext2_scale_accumulate_ffi");
}
int agl_to_aext2_batch_ffi(const uint64_t* in, uint64_t* out, int n) { return ew_lift(in, out, 2, n, true, AGL_Q, "agl_to_aext2_batch_ffi"); }
int aext2_to_agl_batch_ffi(const uint64_t* in, uint64_t* out, int n) { return ew_lift(in, out, 2, n, false, AGL_Q, "aext2_to_agl_batch_ffi"); }
int agl_zero_buffer_ffi(uint64_t* d_buf, int n) { return n < 0 ? GB_EINVAL : zero_words(d_buf, (size_t)n); }

}  // extern "C"
