// Multilinear product sumcheck: the reference-ABI round/fold kernels and the
// fused whole-proof driver.
//
// Round k of the protocol (zk-torch-3/src/sumcheck/linear_prover.rs:66-118,
// cuda/sumcheck_prover.cuh:37-151): for c = 0..d,
//     s_k(c) = sum_y prod_i (p_i[2y] + c (p_i[2y+1] - p_i[2y])),
// then every p_i is folded with the round challenge r:
//     p_i[y] <- p_i[2y] + r (p_i[2y+1] - p_i[2y]).
//
// Fused driver layout: round 0 reads the caller's base-field polynomials
// directly (one 128-bit load per (poly, pair)) -- the reference lifts them to
// Ext2 on the host first, which doubles round-0 traffic.  Each later round is a
// single launch that folds the previous level with r_{k-1} (writing the folded
// level, 128-bit stores) and accumulates round k's message from the folded
// values still in registers, so the folded level is written once and never
// re-read within the round.  The message is reduced inside the launch (last
// block finishes), leaving d+1 canonical values for a 16*(d+1)-byte copy.
#include <vector>

#include "../../include/goldilocks_cuda_wrapper.h"
#include "common.cuh"
#include "host_field.hpp"
#include "reduce.cuh"
#include "sc_device.cuh"

namespace gb {

constexpr int SC_MAX_D = 8;

// ---------------------------------------------------------------------------
// Reference-ABI kernels (per-block partials, stride = original size)
// ---------------------------------------------------------------------------
template <int D, bool EXT>
__global__ void __launch_bounds__(RED_THREADS) ref_round_msg_kernel(const u64* __restrict__ polys, u64* __restrict__ partial,
                                                                    size_t stride, size_t half) {
    constexpr int W = EXT ? 2 * (D + 1) : (D + 1);
    u64 acc[W];
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = 0;
    const bool vec = aligned16(polys) && ((stride & 1) == 0);
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        if constexpr (EXT) {
            e2 e[D], dl[D];
#pragma unroll
            for (int i = 0; i < D; i++) {
                const u64* p = polys + (size_t)i * 2 * stride + 4 * y;
                e[i] = ld_e2(p, vec);
                dl[i] = e2_sub(ld_e2(p + 2, vec), e[i]);
            }
            accum_e2<D>(e, dl, acc);
        } else {
            u64 e[D], dl[D];
#pragma unroll
            for (int i = 0; i < D; i++) {
                u64 a, b;
                ld_pair(polys + (size_t)i * stride + 2 * y, vec, a, b);
                e[i] = a;
                dl[i] = gl_sub(b, a);
            }
            accum_base<D>(e, dl, acc);
        }
    }
    block_partials<W>(acc, partial);
}

template <bool EXT>
__global__ void ref_fold_kernel(const u64* __restrict__ in, u64* __restrict__ out, u64 r0, u64 r1, int d, size_t stride,
                                size_t half) {
    size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (y >= half) return;
    for (int i = 0; i < d; i++) {
        if constexpr (EXT) {
            const u64* p = in + (size_t)i * 2 * stride + 4 * y;
            e2 a = e2_make(p[0], p[1]), b = e2_make(p[2], p[3]);
            e2 f = e2_add(a, e2_mul(e2_make(r0, r1), e2_sub(b, a)));
            u64* q = out + (size_t)i * 2 * stride + 2 * y;
            q[0] = f.c0;
            q[1] = f.c1;
        } else {
            const u64* p = in + (size_t)i * stride + 2 * y;
            out[(size_t)i * stride + y] = gl_add(p[0], gl_mul(r0, gl_sub(p[1], p[0])));
        }
    }
}

// ---------------------------------------------------------------------------
// Fused driver kernels
// ---------------------------------------------------------------------------

// Round 0 on base-field inputs: message only (EXT decides the output width).
template <int D, bool EXT>
__global__ void __launch_bounds__(RED_THREADS) sc_round0_kernel(const u64* __restrict__ polys, size_t stride, size_t half,
                                                                u64* __restrict__ partials, u64* __restrict__ msg,
                                                                unsigned* __restrict__ counter) {
    constexpr int W = EXT ? 2 * (D + 1) : (D + 1);
    u64 acc[W];
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = 0;
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        u64 e[D], dl[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
            u64 a, b;
            ld_pair(polys + (size_t)i * stride + 2 * y, true, a, b);
            e[i] = a;
            dl[i] = gl_sub(b, a);
        }
        if constexpr (EXT) {
            u64 bacc[D + 1];
#pragma unroll
            for (int c = 0; c <= D; c++) bacc[c] = 0;
            accum_base<D>(e, dl, bacc);
#pragma unroll
            for (int c = 0; c <= D; c++) acc[2 * c] = gl_add(acc[2 * c], bacc[c]);
        } else {
            accum_base<D>(e, dl, acc);
        }
    }
    grid_reduce_finish<W>(acc, partials, msg, counter);
}

// Round 0 on Ext2 inputs (CpuLinearSumcheckProverExt2): message only.
template <int D>
__global__ void __launch_bounds__(RED_THREADS) sc_round0_e2in_kernel(const u64* __restrict__ polys, size_t stride,
                                                                     size_t half, u64* __restrict__ partials,
                                                                     u64* __restrict__ msg, unsigned* __restrict__ counter) {
    constexpr int W = 2 * (D + 1);
    u64 acc[W];
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = 0;
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        e2 e[D], dl[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
            const u64* p = polys + (size_t)i * 2 * stride + 4 * y;
            e[i] = ld_e2(p, true);
            dl[i] = e2_sub(ld_e2(p + 2, true), e[i]);
        }
        accum_e2<D>(e, dl, acc);
    }
    grid_reduce_finish<W>(acc, partials, msg, counter);
}

// Round k >= 1, Ext2 challenge: fold level k-1 (base if BASE_IN) with r, store the folded
// level, accumulate round k's message.  quarter = number of output pairs.
template <int D, bool BASE_IN>
__global__ void __launch_bounds__(RED_THREADS) sc_fold_round_e2_kernel(const u64* __restrict__ in, size_t in_stride,
                                                                       u64* __restrict__ out, size_t out_stride,
                                                                       size_t quarter, u64 r0, u64 r1,
                                                                       u64* __restrict__ partials, u64* __restrict__ msg,
                                                                       unsigned* __restrict__ counter) {
    constexpr int W = 2 * (D + 1);
    u64 acc[W];
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = 0;
    const e2 r = e2_make(r0, r1);
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < quarter; y += (size_t)gridDim.x * blockDim.x) {
        e2 e[D], dl[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
            e2 a, b;
            if constexpr (BASE_IN) {
                const u64* p = in + (size_t)i * in_stride + 4 * y;
                u64 x0, x1, x2, x3;
                ld_pair(p, true, x0, x1);
                ld_pair(p + 2, true, x2, x3);
                u64 d0 = gl_sub(x1, x0), d1 = gl_sub(x3, x2);
                a = e2_make(gl_add(x0, gl_mul(r0, d0)), gl_mul(r1, d0));
                b = e2_make(gl_add(x2, gl_mul(r0, d1)), gl_mul(r1, d1));
            } else {
                const u64* p = in + (size_t)i * 2 * in_stride + 8 * y;
                e2 x0 = ld_e2(p, true), x1 = ld_e2(p + 2, true), x2 = ld_e2(p + 4, true), x3 = ld_e2(p + 6, true);
                a = e2_add(x0, e2_mul(r, e2_sub(x1, x0)));
                b = e2_add(x2, e2_mul(r, e2_sub(x3, x2)));
            }
            u64* q = out + (size_t)i * 2 * out_stride + 4 * y;
            e2_st(q, a);
            e2_st(q + 2, b);
            e[i] = a;
            dl[i] = e2_sub(b, a);
        }
        accum_e2<D>(e, dl, acc);
    }
    grid_reduce_finish<W>(acc, partials, msg, counter);
}

// Round k >= 2 (Ext2 input) for D <= 4 with lazy arithmetic:
//   fold  a = x0 + r (x1 - x0) per coordinate as ONE three-word multiply-accumulate,
//         c0 = x0.c0 + r0 d0 + (7 r1) d1,  c1 = x0.c1 + r0 d1 + r1 d0  (d = x1 - x0; r0, r1,
//         7 r1 canonical, so each product is below 2^128 - 2^96), reduced once;
//   message: s(c) = sum_y prod_i v_i(c): the product of the first D-1 factors is reduced, the
//         last multiplication is accumulated as raw 128-bit products (schoolbook:
//         A += p0 q0 + p1 (7 q1), C += p0 q1 + p1 q0), reduced once per thread.
// Same outputs (mod p) as sc_fold_round_e2_kernel<D, false>.
template <int D>
__global__ void __launch_bounds__(RED_THREADS) sc_fold_round_e2_lazy_kernel(const u64* __restrict__ in, size_t in_stride,
                                                                            u64* __restrict__ out, size_t out_stride,
                                                                            size_t quarter, u64 r0_, u64 r1_,
                                                                            u64* __restrict__ partials,
                                                                            u64* __restrict__ msg,
                                                                            unsigned* __restrict__ counter) {
    constexpr int W = 2 * (D + 1);
    const u64 r0 = gl_canon(r0_), r1 = gl_canon(r1_), r1x7 = gl_canon(gl_mul7(r1));
    gl3 A[D + 1], C[D + 1];
#pragma unroll
    for (int c = 0; c <= D; c++) A[c] = C[c] = gl3_zero();
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < quarter; y += (size_t)gridDim.x * blockDim.x) {
        e2 e[D], dl[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
            const u64* p = in + (size_t)i * 2 * in_stride + 8 * y;
            e2 x[4] = {ld_e2(p, true), ld_e2(p + 2, true), ld_e2(p + 4, true), ld_e2(p + 6, true)};
            e2 f[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                u64 d0 = gl_sub(x[2 * h + 1].c0, x[2 * h].c0), d1 = gl_sub(x[2 * h + 1].c1, x[2 * h].c1);
                gl3 c0 = gl3_zero(), c1 = gl3_zero();
                c0.lo = x[2 * h].c0;
                c1.lo = x[2 * h].c1;
                gl3_add_prod(c0, r0, d0);
                gl3_add_prod(c0, r1x7, d1);
                gl3_add_prod(c1, r0, d1);
                gl3_add_prod(c1, r1, d0);
                f[h] = e2_make(gl3_reduce(c0), gl3_reduce(c1));
            }
            u64* q = out + (size_t)i * 2 * out_stride + 4 * y;
            e2_st(q, f[0]);
            e2_st(q + 2, f[1]);
            e[i] = f[0];
            dl[i] = e2_sub(f[1], f[0]);
        }
        e2 v[D];
#pragma unroll
        for (int i = 0; i < D; i++) v[i] = e[i];
#pragma unroll
        for (int c = 0; c <= D; c++) {
            e2 pre = v[0];
#pragma unroll
            for (int i = 1; i + 1 < D; i++) pre = e2_mul(pre, v[i]);
            if constexpr (D == 1) {
                gl3_add(A[c], pre.c0);
                gl3_add(C[c], pre.c1);
            } else {
                const e2 last = v[D - 1];
                gl3_add_prod(A[c], pre.c0, last.c0);
                gl3_add_prod(A[c], pre.c1, gl_mul7(last.c1));
                gl3_add_prod(C[c], pre.c0, last.c1);
                gl3_add_prod(C[c], pre.c1, last.c0);
            }
            if (c < D) {
#pragma unroll
                for (int i = 0; i < D; i++) v[i] = e2_add(v[i], dl[i]);
            }
        }
    }
    u64 acc[W];
#pragma unroll
    for (int c = 0; c <= D; c++) {
        acc[2 * c] = gl3_reduce(A[c]);
        acc[2 * c + 1] = gl3_reduce(C[c]);
    }
    grid_reduce_finish<W>(acc, partials, msg, counter);
}

// D == 2: the lazy round with the next pair's loads issued before the current pair is folded
// (register double buffering; two resident blocks per SM leave room for the extra registers).
// Same outputs as sc_fold_round_e2_lazy_kernel.
template <int D>  // D == 2 only (the message's last factor is the second polynomial)
__global__ void __launch_bounds__(RED_THREADS, 2) sc_fold_round_e2_pf_kernel(const u64* __restrict__ in, size_t in_stride, u64* __restrict__ out,
                                                          size_t out_stride, size_t quarter, u64 r0_, u64 r1_,
                                                          u64* __restrict__ partials, u64* __restrict__ msg,
                                                          unsigned* __restrict__ counter) {
    static_assert(D == 2, "the prefetching fold round is the degree-2 form");
    constexpr int W = 2 * (D + 1);
    const u64 r0 = gl_canon(r0_), r1 = gl_canon(r1_), r1x7 = gl_canon(gl_mul7(r1));
    gl3 A[D + 1], C[D + 1];
#pragma unroll
    for (int c = 0; c <= D; c++) A[c] = C[c] = gl3_zero();
    const size_t step = (size_t)gridDim.x * blockDim.x;
    size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    e2 nx[D][4];
    if (y < quarter) {
#pragma unroll
        for (int i = 0; i < D; i++) {
            const u64* p = in + (size_t)i * 2 * in_stride + 8 * y;
#pragma unroll
            for (int k = 0; k < 4; k++) nx[i][k] = ld_e2(p + 2 * k, true);
        }
    }
    for (; y < quarter; y += step) {
        e2 x[D][4];
#pragma unroll
        for (int i = 0; i < D; i++)
#pragma unroll
            for (int k = 0; k < 4; k++) x[i][k] = nx[i][k];
        const size_t yn = y + step;
        if (yn < quarter) {
#pragma unroll
            for (int i = 0; i < D; i++) {
                const u64* p = in + (size_t)i * 2 * in_stride + 8 * yn;
#pragma unroll
                for (int k = 0; k < 4; k++) nx[i][k] = ld_e2(p + 2 * k, true);
            }
        }
        e2 e[D], f1[D], dl[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
            e2 f[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                u64 d0 = gl_sub(x[i][2 * h + 1].c0, x[i][2 * h].c0), d1 = gl_sub(x[i][2 * h + 1].c1, x[i][2 * h].c1);
                gl3 c0 = gl3_zero(), c1 = gl3_zero();
                c0.lo = x[i][2 * h].c0;
                c1.lo = x[i][2 * h].c1;
                gl3_add_prod(c0, r0, d0);
                gl3_add_prod(c0, r1x7, d1);
                gl3_add_prod(c1, r0, d1);
                gl3_add_prod(c1, r1, d0);
                f[h] = e2_make(gl3_reduce(c0), gl3_reduce(c1));
            }
            u64* q = out + (size_t)i * 2 * out_stride + 4 * y;
            e2_st(q, f[0]);
            e2_st(q + 2, f[1]);
            e[i] = f[0];
            f1[i] = f[1];
            dl[i] = e2_sub(f[1], f[0]);
        }
        // the product at 0, at 1, and its leading coefficient (the product of the slopes)
        const e2 pts[3][2] = {{e[0], e[1]}, {f1[0], f1[1]}, {dl[0], dl[1]}};
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const e2 pre = pts[c][0], last = pts[c][1];
            gl3_add_prod(A[c], pre.c0, last.c0);
            gl3_add_prod(A[c], pre.c1, gl_mul7(last.c1));
            gl3_add_prod(C[c], pre.c0, last.c1);
            gl3_add_prod(C[c], pre.c1, last.c0);
        }
    }
    // s(2) = 2 s(1) - s(0) + 2 lead (the second difference of a quadratic is twice its lead)
    u64 acc[W];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        acc[2 * c] = gl3_reduce(A[c]);
        acc[2 * c + 1] = gl3_reduce(C[c]);
    }
#pragma unroll
    for (int k = 0; k < 2; k++) acc[4 + k] = gl_sub(gl_add(gl_double(acc[2 + k]), gl_double(acc[4 + k])), acc[k]);
    grid_reduce_finish<W>(acc, partials, msg, counter);
}

// Round k >= 1, base-field challenge (LinearSumcheckProver).
template <int D>
__global__ void __launch_bounds__(RED_THREADS) sc_fold_round_base_kernel(const u64* __restrict__ in, size_t in_stride,
                                                                         u64* __restrict__ out, size_t out_stride,
                                                                         size_t quarter, u64 r,
                                                                         u64* __restrict__ partials, u64* __restrict__ msg,
                                                                         unsigned* __restrict__ counter) {
    constexpr int W = D + 1;
    u64 acc[W];
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = 0;
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < quarter; y += (size_t)gridDim.x * blockDim.x) {
        u64 e[D], dl[D];
#pragma unroll
        for (int i = 0; i < D; i++) {
            const u64* p = in + (size_t)i * in_stride + 4 * y;
            u64 x0, x1, x2, x3;
            ld_pair(p, true, x0, x1);
            ld_pair(p + 2, true, x2, x3);
            u64 a = gl_add(x0, gl_mul(r, gl_sub(x1, x0)));
            u64 b = gl_add(x2, gl_mul(r, gl_sub(x3, x2)));
            ulonglong2 v;
            v.x = a;
            v.y = b;
            *reinterpret_cast<ulonglong2*>(out + (size_t)i * out_stride + 2 * y) = v;
            e[i] = a;
            dl[i] = gl_sub(b, a);
        }
        accum_base<D>(e, dl, acc);
    }
    grid_reduce_finish<W>(acc, partials, msg, counter);
}

// Final fold of the last pair of every polynomial; canonical outputs.
// EXT_CH: Ext2 challenge; BASE_IN: the pair is base-field (n == 1).
template <bool EXT_CH, bool BASE_IN>
__global__ void sc_final_kernel(const u64* __restrict__ in, size_t in_stride, int d, u64 r0, u64 r1,
                                u64* __restrict__ finals) {
    int i = threadIdx.x;
    if (i >= d) return;
    if constexpr (!EXT_CH) {
        const u64* p = in + (size_t)i * in_stride;
        finals[i] = gl_canon(gl_add(p[0], gl_mul(r0, gl_sub(p[1], p[0]))));
    } else if constexpr (BASE_IN) {
        const u64* p = in + (size_t)i * in_stride;
        u64 dd = gl_sub(p[1], p[0]);
        finals[2 * i] = gl_canon(gl_add(p[0], gl_mul(r0, dd)));
        finals[2 * i + 1] = gl_canon(gl_mul(r1, dd));
    } else {
        const u64* p = in + (size_t)i * 2 * in_stride;
        e2 a = e2_make(p[0], p[1]), b = e2_make(p[2], p[3]);
        e2 f = e2_canon(e2_add(a, e2_mul(e2_make(r0, r1), e2_sub(b, a))));
        finals[2 * i] = f.c0;
        finals[2 * i + 1] = f.c1;
    }
}

// ---------------------------------------------------------------------------
// dispatch helpers
// ---------------------------------------------------------------------------
template <template <int> class F, typename... A>
static int dispatch_d(int d, A... args) {
    switch (d) {
        case 1: return F<1>::run(args...);
        case 2: return F<2>::run(args...);
        case 3: return F<3>::run(args...);
        case 4: return F<4>::run(args...);
        case 5: return F<5>::run(args...);
        case 6: return F<6>::run(args...);
        case 7: return F<7>::run(args...);
        case 8: return F<8>::run(args...);
        default: return GB_EINVAL;
    }
}

template <bool EXT>
struct RefRound {
    template <int D>
    struct K {
        static int run(const u64* polys, u64* partial, size_t stride, size_t half, int blocks) {
            ref_round_msg_kernel<D, EXT><<<blocks, RED_THREADS, 0, stream()>>>(polys, partial, stride, half);
            return check_launch("sumcheck_round_message");
        }
    };
};

template <int D>
struct Round0E2 {
    static int run(const u64* polys, size_t stride, size_t half, unsigned grid, u64* part, u64* msg, unsigned* ctr) {
        sc_round0_kernel<D, true><<<grid, RED_THREADS, 0, stream()>>>(polys, stride, half, part, msg, ctr);
        return check_launch("sc_round0");
    }
};
template <int D>
struct Round0E2In {
    static int run(const u64* polys, size_t stride, size_t half, unsigned grid, u64* part, u64* msg, unsigned* ctr) {
        sc_round0_e2in_kernel<D><<<grid, RED_THREADS, 0, stream()>>>(polys, stride, half, part, msg, ctr);
        return check_launch("sc_round0_e2in");
    }
};
template <int D>
struct Round0Base {
    static int run(const u64* polys, size_t stride, size_t half, unsigned grid, u64* part, u64* msg, unsigned* ctr) {
        sc_round0_kernel<D, false><<<grid, RED_THREADS, 0, stream()>>>(polys, stride, half, part, msg, ctr);
        return check_launch("sc_round0");
    }
};
template <int D>
struct FoldRoundE2 {
    static int run(bool base_in, const u64* in, size_t in_stride, u64* out, size_t out_stride, size_t quarter,
                   unsigned grid, u64 r0, u64 r1, u64* part, u64* msg, unsigned* ctr) {
        if (base_in)
            sc_fold_round_e2_kernel<D, true><<<grid, RED_THREADS, 0, stream()>>>(in, in_stride, out, out_stride, quarter,
                                                                                 r0, r1, part, msg, ctr);
        else if constexpr (D == 2)
            sc_fold_round_e2_pf_kernel<D><<<grid, RED_THREADS, 0, stream()>>>(in, in_stride, out, out_stride, quarter,
                                                                              r0, r1, part, msg, ctr);
        else if constexpr (D <= 4)
            sc_fold_round_e2_lazy_kernel<D><<<grid, RED_THREADS, 0, stream()>>>(in, in_stride, out, out_stride, quarter,
                                                                                r0, r1, part, msg, ctr);
        else
            sc_fold_round_e2_kernel<D, false><<<grid, RED_THREADS, 0, stream()>>>(in, in_stride, out, out_stride, quarter,
                                                                                  r0, r1, part, msg, ctr);
        return check_launch("sc_fold_round_e2");
    }
};
template <int D>
struct FoldRoundBase {
    static int run(const u64* in, size_t in_stride, u64* out, size_t out_stride, size_t quarter, unsigned grid, u64 r,
                   u64* part, u64* msg, unsigned* ctr) {
        sc_fold_round_base_kernel<D><<<grid, RED_THREADS, 0, stream()>>>(in, in_stride, out, out_stride, quarter, r, part,
                                                                         msg, ctr);
        return check_launch("sc_fold_round_base");
    }
};

// Grid size for a round over `work` items: enough blocks to fill the GPU, at most one
// item per thread when work is small.
static unsigned round_grid(size_t work) {
    size_t cap = (size_t)num_sms() * 4;
    size_t need = (work + RED_THREADS - 1) / RED_THREADS;
    if (need < 1) need = 1;
    return (unsigned)(need < cap ? need : cap);
}

// Pinned host staging reused by the calling thread.
static u64* pinned_staging(size_t words) { return thread_pinned(0, words); }

// Device workspace of one proof.
struct ScWork {
    u64* base = nullptr;  // caller-independent aligned copy of the inputs (when needed)
    u64* a = nullptr;     // ping
    u64* b = nullptr;     // pong
    u64* partials = nullptr;
    unsigned* counter = nullptr;
    ~ScWork() {
        cudaStream_t s = stream();
        if (base) cudaFreeAsync(base, s);
        if (a) cudaFreeAsync(a, s);
        if (b) cudaFreeAsync(b, s);
        if (partials) cudaFreeAsync(partials, s);
        if (counter) cudaFreeAsync(counter, s);
    }
};

// ext: Ext2 challenges and messages; in_ext (with ext): the polynomials themselves are Ext2,
// [d][2^n][c0, c1].
static int prove(gb_transcript* t, int n, int d, const u64* d_polys, const u64* h_polys, bool ext, bool in_ext,
                 u64* h_msgs, u64* h_ch, u64* h_finals, u64* h_final_eval) {
    using namespace host;
    if (!t || n < 0 || n > 40 || d < 1 || d > SC_MAX_D || (!d_polys == !h_polys) || !h_msgs || !h_ch || !h_finals ||
        !h_final_eval) {
        set_error_msg("gb_sumcheck_prove: invalid argument");
        return GB_EINVAL;
    }
    cudaStream_t s = stream();
    const size_t N = (size_t)1 << n;
    const int W = ext ? 2 : 1;  // words per value in messages / challenges
    tr_append_u64(t, "num_var", (u64)n);
    tr_append_u64(t, "num_poly", (u64)d);

    ScWork w;
    const u64* polys = d_polys;
    const int IW = in_ext ? 2 : 1;  // words per input value
    if (h_polys || (((uintptr_t)d_polys) & 15)) {
        GB_CUDA_TRY(cudaMallocAsync(&w.base, N * d * IW * 8, s));
        GB_CUDA_TRY(cudaMemcpyAsync(w.base, h_polys ? (const void*)h_polys : (const void*)d_polys, N * d * IW * 8,
                                    h_polys ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, s));
        polys = w.base;
    }
    u64* stage = pinned_staging(2 * (SC_MAX_D + 1) + 2 * SC_MAX_D);
    // the round kernels write each message (and the final values) straight into the pinned
    // staging through its device address, so reading it back is a stream synchronisation
    void* stage_dev = nullptr;
    if (!stage || cudaHostGetDevicePointer(&stage_dev, stage, 0) != cudaSuccess) {
        set_error_msg("gb_sumcheck_prove: pinned staging allocation failed");
        return GB_ECUDA;
    }
    u64* msg_out = (u64*)stage_dev;
    const unsigned max_grid = round_grid(N / 2 > 0 ? N / 2 : 1);
    GB_CUDA_TRY(cudaMallocAsync(&w.partials, (size_t)max_grid * 2 * (SC_MAX_D + 1) * 8, s));
    GB_CUDA_TRY(cudaMallocAsync(&w.counter, sizeof(unsigned), s));
    GB_CUDA_TRY(cudaMemsetAsync(w.counter, 0, sizeof(unsigned), s));
    const size_t lvl_stride = N / 2 > 0 ? N / 2 : 1;  // elements per poly in the ping/pong buffers
    if (n >= 2) {
        size_t words = lvl_stride * d * (ext ? 2 : 1);
        GB_CUDA_TRY(cudaMallocAsync(&w.a, words * 8, s));
        GB_CUDA_TRY(cudaMallocAsync(&w.b, words * 8, s));
    }

    std::vector<u64> finals(2 * d, 0);
    if (n == 0) {
        // no rounds: the single evaluation of every polynomial is its final value
        GB_CUDA_TRY(cudaMemcpyAsync(stage, polys, (size_t)d * IW * 8, cudaMemcpyDeviceToHost, s));
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        for (int i = 0; i < d; i++)
            for (int c = 0; c < IW; c++) finals[W * i + c] = canon(stage[IW * i + c]);
    } else {
        u64 r0 = 0, r1 = 0;
        const u64* cur = polys;
        size_t cur_stride = N;
        bool base_in = !in_ext;
        u64* bufs[2] = {w.a, w.b};
        int pp = 0;
        for (int k = 0; k < n; k++) {
            const size_t level = N >> k;  // elements of the level this round's message is taken over
            int rc;
            if (k == 0) {
                unsigned g = round_grid(level / 2);
                rc = in_ext ? dispatch_d<Round0E2In>(d, cur, cur_stride, level / 2, g, w.partials, msg_out, w.counter)
                     : ext  ? dispatch_d<Round0E2>(d, cur, cur_stride, level / 2, g, w.partials, msg_out, w.counter)
                            : dispatch_d<Round0Base>(d, cur, cur_stride, level / 2, g, w.partials, msg_out, w.counter);
            } else {
                u64* dst = bufs[pp];
                size_t quarter = level / 2;  // output pairs
                unsigned g = round_grid(quarter);
                rc = ext ? dispatch_d<FoldRoundE2>(d, base_in, cur, cur_stride, dst, lvl_stride, quarter, g, r0, r1,
                                                   w.partials, msg_out, w.counter)
                         : dispatch_d<FoldRoundBase>(d, cur, cur_stride, dst, lvl_stride, quarter, g, r0, w.partials, msg_out,
                                                     w.counter);
                cur = dst;
                cur_stride = lvl_stride;
                base_in = false;
                pp ^= 1;
            }
            if (rc) return rc;
            const int words = W * (d + 1);
            // the first message's label does not depend on the message: absorb it while the
            // round runs on the device (the absorb sequence is unchanged)
            tr_label(t, "round_message");
            GB_CUDA_TRY(cudaStreamSynchronize(s));
            u64* m = h_msgs + (size_t)k * words;
            for (int i = 0; i < words; i++) m[i] = stage[i];
            if (ext) {
                tr_absorb(t, m[0]);
                tr_absorb(t, m[1]);
                for (int c = 1; c <= d; c++) tr_append_ext2(t, "round_message", E2{m[2 * c], m[2 * c + 1]});
                E2 ch = tr_challenge_ext2(t, "challenge");
                r0 = ch.c0;
                r1 = ch.c1;
                h_ch[2 * k] = r0;
                h_ch[2 * k + 1] = r1;
            } else {
                tr_absorb(t, m[0]);
                for (int c = 1; c <= d; c++) tr_append_u64(t, "round_message", m[c]);
                r0 = tr_challenge(t, "challenge");
                h_ch[k] = r0;
            }
        }
        if (ext) {
            if (base_in)
                sc_final_kernel<true, true><<<1, 32, 0, s>>>(cur, cur_stride, d, r0, r1, msg_out);
            else
                sc_final_kernel<true, false><<<1, 32, 0, s>>>(cur, cur_stride, d, r0, r1, msg_out);
        } else {
            sc_final_kernel<false, true><<<1, 32, 0, s>>>(cur, cur_stride, d, r0, r1, msg_out);
        }
        GB_LAUNCH_CHECK("sc_final");
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        for (int i = 0; i < W * d; i++) finals[i] = stage[i];
    }
    for (int i = 0; i < W * d; i++) h_finals[i] = finals[i];
    if (ext) {
        E2 fe{1, 0};
        for (int i = 0; i < d; i++) fe = e2mul(fe, E2{finals[2 * i], finals[2 * i + 1]});
        h_final_eval[0] = fe.c0;
        h_final_eval[1] = fe.c1;
    } else {
        u64 fe = 1;
        for (int i = 0; i < d; i++) fe = mul(fe, finals[i]);
        h_final_eval[0] = fe;
    }
    return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int sumcheck_round_message_ffi(const uint64_t* d_polys, uint64_t* d_partial, int d, size_t original_size, size_t half,
                               int num_blocks) {
    if (num_blocks <= 0 || d < 1 || d > SC_MAX_D) return GB_EINVAL;
    int rc = dispatch_d<RefRound<false>::K>(d, d_polys, d_partial, original_size, half, num_blocks);
    return rc ? rc : sync_stream("sumcheck_round_message_ffi");
}

int sumcheck_round_message_ext2_ffi(const uint64_t* d_polys, uint64_t* d_partial, int d, size_t original_size,
                                    size_t half, int num_blocks) {
    if (num_blocks <= 0 || d < 1 || d > SC_MAX_D) return GB_EINVAL;
    int rc = dispatch_d<RefRound<true>::K>(d, d_polys, d_partial, original_size, half, num_blocks);
    return rc ? rc : sync_stream("sumcheck_round_message_ext2_ffi");
}

int sumcheck_fold_ffi(const uint64_t* d_input, uint64_t* d_output, uint64_t challenge, int d, size_t original_size,
                      size_t half) {
    if (d < 1) return GB_EINVAL;
    if (half == 0) return GB_OK;
    ref_fold_kernel<false><<<grid_for(half, 256), 256, 0, stream()>>>(d_input, d_output, challenge, 0, d, original_size,
                                                                       half);
    GB_LAUNCH_CHECK("sumcheck_fold_ffi");
    return sync_stream("sumcheck_fold_ffi");
}

int sumcheck_fold_ext2_ffi(const uint64_t* d_input, uint64_t* d_output, uint64_t c0, uint64_t c1, int d,
                           size_t original_size, size_t half) {
    if (d < 1) return GB_EINVAL;
    if (half == 0) return GB_OK;
    ref_fold_kernel<true><<<grid_for(half, 256), 256, 0, stream()>>>(d_input, d_output, c0, c1, d, original_size, half);
    GB_LAUNCH_CHECK("sumcheck_fold_ext2_ffi");
    return sync_stream("sumcheck_fold_ext2_ffi");
}

int gb_sumcheck_prove_ext2(gb_transcript* t, int n, int d, const uint64_t* d_polys, const uint64_t* h_polys,
                           uint64_t* h_msgs, uint64_t* h_challenges, uint64_t* h_finals, uint64_t* h_final_eval) {
    return prove(t, n, d, d_polys, h_polys, true, false, h_msgs, h_challenges, h_finals, h_final_eval);
}

int gb_sumcheck_prove_ext2_polys(gb_transcript* t, int n, int d, const uint64_t* d_polys, const uint64_t* h_polys,
                                 uint64_t* h_msgs, uint64_t* h_challenges, uint64_t* h_finals, uint64_t* h_final_eval) {
    return prove(t, n, d, d_polys, h_polys, true, true, h_msgs, h_challenges, h_finals, h_final_eval);
}

size_t gb_sumcheck_round_workspace_words(void) {
    return (size_t)num_sms() * 4 * 2 * (SC_MAX_D + 1) + 2;
}

int gb_sumcheck_fold_round_ext2(const uint64_t* d_in, int in_base, size_t in_stride, uint64_t* d_out,
                                size_t out_stride, int d, size_t pairs_out, uint64_t r0, uint64_t r1, uint64_t* d_msg,
                                uint64_t* d_work) {
    if (d < 1 || d > SC_MAX_D || pairs_out == 0 || !d_work || !d_msg) return GB_EINVAL;
    unsigned g = round_grid(pairs_out);
    u64* partials = d_work;
    unsigned* counter = reinterpret_cast<unsigned*>(d_work + (size_t)num_sms() * 4 * 2 * (SC_MAX_D + 1));
    return dispatch_d<FoldRoundE2>(d, in_base != 0, d_in, in_stride, d_out, out_stride, pairs_out, g, r0, r1, partials,
                                   d_msg, counter);
}

int gb_sumcheck_prove_base(gb_transcript* t, int n, int d, const uint64_t* d_polys, const uint64_t* h_polys,
                           uint64_t* h_msgs, uint64_t* h_challenges, uint64_t* h_finals, uint64_t* h_final_eval) {
    return prove(t, n, d, d_polys, h_polys, false, false, h_msgs, h_challenges, h_finals, h_final_eval);
}

}  // extern "C"
