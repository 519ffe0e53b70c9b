// Basefold commit / open on the device: reference-ABI kernels
// (goldilocks-cuda-rs/src/ffi.rs:416-545, wrapper.cu:1223-1600) and the
// whole-proof drivers gb_basefold_*.
//
// Commit.  The reference interpolates evaluations to monomial coefficients
// (per variable (e0, e1) -> (e0, e1 - e0)), repeats every coefficient 2^lr times,
// applies n +-1 butterfly layers on bits lr..n+lr-1 and bit-reverses
// (cuda/basefold.cuh:103-205).  Per variable the two steps compose to
//     T = [[1,1],[1,-1]] [[1,0],[-1,1]] = [[0,1],[2,-1]]:  (e0, e1) -> (e1, 2 e0 - e1),
// and because the repetition bits end up as the top bits after the reversal,
//     codeword[j] = u[bitrev_n(j mod 2^n)],  u = T^(x)n (evals).
// The codeword is 2^lr copies of one block, so its Merkle tree consists of 2^lr
// identical subtrees: one is hashed, the others are copied (merkle.cu).
//
// Open (BasefoldCommitment::open_ext2, basefold.rs:578-870).  Round r's sumcheck
// oracle (c0, c1, c2) over the pairs of the folded eq / bh tables comes from one
// launch that also folds both tables with the previous challenge; the codeword
// fold of round r writes the folded codeword and hashes its leaves in the same
// launch.  Per round the host receives 10 canonical words (oracle + root), runs the
// transcript and launches the next round.  Queries are gathered by one kernel.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/goldilocks_cuda_wrapper.h"
#include "basefold.cuh"
#include "host_field.hpp"
#include "merkle.cuh"
#include "bf_device.cuh"
#include "reduce.cuh"

namespace gb {

// ===========================================================================
// 2x2 per-variable transforms applied to K consecutive bits [b, b+K) in registers
// MAT 0: T = (e1, 2 e0 - e1)   1: Moebius (e0, e1 - e0)   2: WHT (e0 + e1, e0 - e1)
// ===========================================================================
template <int MAT, int K>
__global__ void bf_transform_pass_kernel(const u64* __restrict__ in, u64* __restrict__ out, int b, size_t groups) {
    size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (g >= groups) return;
    bf_transform_group<MAT, K>(in, out, b, g);
}

// apply the transform on all n bits; in may equal out
template <int MAT>
static int bf_transform(const u64* in, u64* out, int n) {
    cudaStream_t s = stream();
    size_t N = (size_t)1 << n;
    if (n == 0) {
        if (in != out) GB_CUDA_TRY(cudaMemcpyAsync(out, in, 8, cudaMemcpyDeviceToDevice, s));
        return GB_OK;
    }
    const u64* src = in;
    for (int b = 0; b < n;) {
        int k = n - b >= 4 ? 4 : n - b;
        size_t groups = N >> k;
        switch (k) {
            case 4: bf_transform_pass_kernel<MAT, 4><<<grid_for(groups, 128), 128, 0, s>>>(src, out, b, groups); break;
            case 3: bf_transform_pass_kernel<MAT, 3><<<grid_for(groups, 128), 128, 0, s>>>(src, out, b, groups); break;
            case 2: bf_transform_pass_kernel<MAT, 2><<<grid_for(groups, 128), 128, 0, s>>>(src, out, b, groups); break;
            default: bf_transform_pass_kernel<MAT, 1><<<grid_for(groups, 128), 128, 0, s>>>(src, out, b, groups); break;
        }
        GB_LAUNCH_CHECK("bf_transform_pass_kernel");
        src = out;
        b += k;
    }
    return GB_OK;
}


// out[j] = in[bitrev_n(j mod 2^n)] for j < 2^(n+reps_log)
__global__ void bitrev_replicate_kernel(const u64* __restrict__ in, u64* __restrict__ out, int n, size_t total) {
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= total) return;
    size_t m = j & (((size_t)1 << n) - 1);
    out[j] = __ldg(in + bitrev_dev(m, n));
}

template <int W>
__global__ void bit_reverse_inplace_kernel(u64* __restrict__ data, int log_n) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >> log_n) return;
    size_t j = bitrev_dev(i, log_n);
    if (i < j) {
#pragma unroll
        for (int k = 0; k < W; k++) {
            u64 t = data[W * i + k];
            data[W * i + k] = data[W * j + k];
            data[W * j + k] = t;
        }
    }
}

// ===========================================================================
// reference-ABI elementwise kernels (sumcheck interp / eval / fold)
// ===========================================================================
template <bool EXT>
__global__ void sc_interp_kernel(u64* __restrict__ d, size_t pairs) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= pairs) return;
    if (EXT) {
        u64* p = d + 4 * i;
        p[2] = gl_sub(p[2], p[0]);
        p[3] = gl_sub(p[3], p[1]);
    } else {
        d[2 * i + 1] = gl_sub(d[2 * i + 1], d[2 * i]);
    }
}

// out[i] = data[2i] + ch * data[2i+1]; MODE 0 base/base, 1 base data + Ext2 ch, 2 Ext2
template <int MODE>
__global__ void sc_eval_kernel(const u64* __restrict__ d, u64 c0, u64 c1, u64* __restrict__ out, size_t pairs) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= pairs) return;
    if (MODE == 0) {
        out[i] = gl_add(d[2 * i], gl_mul(c0, d[2 * i + 1]));
    } else if (MODE == 1) {
        u64 a = d[2 * i], b = d[2 * i + 1];
        out[2 * i] = gl_add(a, gl_mul(c0, b));
        out[2 * i + 1] = gl_mul(c1, b);
    } else {
        const u64* p = d + 4 * i;
        e2 r = e2_add(e2_make(p[0], p[1]), e2_mul(e2_make(c0, c1), e2_make(p[2], p[3])));
        out[2 * i] = r.c0;
        out[2 * i + 1] = r.c1;
    }
}

template <int MODE>
__global__ void bf_fold_kernel(const u64* __restrict__ cw, const u64* __restrict__ tab, u64 c0, u64 c1,
                               u64* __restrict__ out, size_t pairs) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= pairs) return;
    fold_pair<MODE>(cw, i, tab[2 * i], tab[2 * i + 1], c0, c1, out + (MODE == 0 ? i : 2 * i));
}

// Reference product kernels: per-block partials of c0 = sum eq_e bh_e,
// c1 = sum (eq_e bh_o + eq_o bh_e), c2 = sum eq_o bh_o on interp'd (value, diff) pairs.
// EQ_EXT/BH_EXT select Ext2 operands.
template <bool EQ_EXT, bool BH_EXT>
__device__ __forceinline__ void product_terms(const u64* eq, const u64* bh, size_t i, u64 (&acc)[6]) {
    e2 ee, eo, be, bo;
    if (EQ_EXT) {
        ee = e2_make(eq[4 * i], eq[4 * i + 1]);
        eo = e2_make(eq[4 * i + 2], eq[4 * i + 3]);
    } else {
        ee = e2_make(eq[2 * i], 0);
        eo = e2_make(eq[2 * i + 1], 0);
    }
    if (BH_EXT) {
        be = e2_make(bh[4 * i], bh[4 * i + 1]);
        bo = e2_make(bh[4 * i + 2], bh[4 * i + 3]);
    } else {
        be = e2_make(bh[2 * i], 0);
        bo = e2_make(bh[2 * i + 1], 0);
    }
    e2 t0, t1, t2;
    if (!EQ_EXT && !BH_EXT) {
        t0 = e2_make(gl_mul(ee.c0, be.c0), 0);
        t1 = e2_make(gl_add(gl_mul(ee.c0, bo.c0), gl_mul(eo.c0, be.c0)), 0);
        t2 = e2_make(gl_mul(eo.c0, bo.c0), 0);
    } else if (!BH_EXT) {
        t0 = e2_mul_base(ee, be.c0);
        t1 = e2_add(e2_mul_base(ee, bo.c0), e2_mul_base(eo, be.c0));
        t2 = e2_mul_base(eo, bo.c0);
    } else {
        t0 = e2_mul(ee, be);
        t1 = e2_add(e2_mul(ee, bo), e2_mul(eo, be));
        t2 = e2_mul(eo, bo);
    }
    acc[0] = gl_add(acc[0], t0.c0);
    acc[1] = gl_add(acc[1], t0.c1);
    acc[2] = gl_add(acc[2], t1.c0);
    acc[3] = gl_add(acc[3], t1.c1);
    acc[4] = gl_add(acc[4], t2.c0);
    acc[5] = gl_add(acc[5], t2.c1);
}

__device__ __forceinline__ void write_c_partials(const u64 (&acc)[6], bool ext, u64* p0, u64* p1, u64* p2) {
    if (threadIdx.x) return;
    if (ext) {
        p0[2 * blockIdx.x] = acc[0];
        p0[2 * blockIdx.x + 1] = acc[1];
        p1[2 * blockIdx.x] = acc[2];
        p1[2 * blockIdx.x + 1] = acc[3];
        p2[2 * blockIdx.x] = acc[4];
        p2[2 * blockIdx.x + 1] = acc[5];
    } else {
        p0[blockIdx.x] = acc[0];
        p1[blockIdx.x] = acc[2];
        p2[blockIdx.x] = acc[4];
    }
}

template <bool EQ_EXT, bool BH_EXT>
__global__ void __launch_bounds__(RED_THREADS) sc_product_kernel(const u64* __restrict__ eq, const u64* __restrict__ bh,
                                                                 u64* p0, u64* p1, u64* p2, size_t pairs) {
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs; i += (size_t)gridDim.x * blockDim.x)
        product_terms<EQ_EXT, BH_EXT>(eq, bh, i, acc);
    block_reduce<6>(acc);
    write_c_partials(acc, EQ_EXT || BH_EXT, p0, p1, p2);
}

// fused_sumcheck_round_ext2_kernel semantics (basefold.cuh:654-735): eval at ch, interp, product
__global__ void __launch_bounds__(RED_THREADS) sc_fused_round_ref_kernel(const u64* __restrict__ eq_in,
                                                                         const u64* __restrict__ bh_in, u64 c0, u64 c1,
                                                                         u64* __restrict__ eq_out, u64* __restrict__ bh_out,
                                                                         u64* p0, u64* p1, u64* p2, size_t pairs) {
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    const e2 ch = e2_make(c0, c1);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs; i += (size_t)gridDim.x * blockDim.x) {
        const u64* q = eq_in + 8 * i;
        const u64* h = bh_in + 8 * i;
        e2 ea = e2_add(e2_make(q[0], q[1]), e2_mul(ch, e2_make(q[2], q[3])));
        e2 eb = e2_add(e2_make(q[4], q[5]), e2_mul(ch, e2_make(q[6], q[7])));
        e2 ba = e2_add(e2_make(h[0], h[1]), e2_mul(ch, e2_make(h[2], h[3])));
        e2 bb = e2_add(e2_make(h[4], h[5]), e2_mul(ch, e2_make(h[6], h[7])));
        e2 eo = e2_sub(eb, ea), bo = e2_sub(bb, ba);
        e2_st(eq_out + 4 * i, ea);
        e2_st(eq_out + 4 * i + 2, eo);
        e2_st(bh_out + 4 * i, ba);
        e2_st(bh_out + 4 * i + 2, bo);
        e2 t0 = e2_mul(ea, ba), t1 = e2_add(e2_mul(ea, bo), e2_mul(eo, ba)), t2 = e2_mul(eo, bo);
        acc[0] = gl_add(acc[0], t0.c0);
        acc[1] = gl_add(acc[1], t0.c1);
        acc[2] = gl_add(acc[2], t1.c0);
        acc[3] = gl_add(acc[3], t1.c1);
        acc[4] = gl_add(acc[4], t2.c0);
        acc[5] = gl_add(acc[5], t2.c1);
    }
    block_reduce<6>(acc);
    write_c_partials(acc, true, p0, p1, p2);
}

template <bool MIXED>
__global__ void __launch_bounds__(RED_THREADS) dot_product_kernel(const u64* __restrict__ a, const u64* __restrict__ b,
                                                                  u64* __restrict__ out, size_t n) {
    u64 acc[2] = {0, 0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (MIXED) {
            e2 v = e2_mul_base(e2_make(b[2 * i], b[2 * i + 1]), a[i]);
            acc[0] = gl_add(acc[0], v.c0);
            acc[1] = gl_add(acc[1], v.c1);
        } else {
            acc[0] = gl_add(acc[0], gl_mul(a[i], b[i]));
        }
    }
    block_reduce<2>(acc);
    if (threadIdx.x == 0) {
        if (MIXED) {
            out[2 * blockIdx.x] = acc[0];
            out[2 * blockIdx.x + 1] = acc[1];
        } else {
            out[blockIdx.x] = acc[0];
        }
    }
}

// ===========================================================================
// open_ext2 driver kernels
// ===========================================================================

// Round 0 oracle on (bh base, eq Ext2) at full size: acc = (c0, s1, c2) with
// s1 = sum eq_o bh_o = c0 + c1 + c2.  Also the pairs' eval = c0 + s1.
// BH_BASE: base evaluations (a commitment's); else Ext2 (a batch opening's combined ones).
template <bool BH_BASE>
__global__ void __launch_bounds__(RED_THREADS) open_round0_kernel(const u64* __restrict__ bh, const u64* __restrict__ eq,
                                                                  size_t pairs, u64* __restrict__ partials,
                                                                  u64* __restrict__ out, unsigned* __restrict__ counter) {
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < pairs; i += (size_t)gridDim.x * blockDim.x) {
        if (BH_BASE) open_round0_item(bh, eq, i, acc);
        else open_round0_e2_item(bh, eq, i, acc);
    }
    grid_reduce_finish<6>(acc, partials, out, counter);
}

// Round r >= 1: fold eq (Ext2) and bh (base when BH_BASE) with ch = (c0, c1) from the
// previous level, store the folded level, accumulate (c0, s1, c2) over its pairs.
template <bool BH_BASE>
__global__ void __launch_bounds__(RED_THREADS) open_round_kernel(const u64* __restrict__ eq_in, const u64* __restrict__ bh_in,
                                                                 u64* __restrict__ eq_out, u64* __restrict__ bh_out,
                                                                 size_t quarter, u64 c0, u64 c1,
                                                                 u64* __restrict__ partials, u64* __restrict__ out,
                                                                 unsigned* __restrict__ counter) {
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    const e2 ch = e2_make(c0, c1);
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < quarter; y += (size_t)gridDim.x * blockDim.x)
        open_round_item<BH_BASE>(eq_in, bh_in, eq_out, bh_out, y, ch, acc);
    grid_reduce_finish<6>(acc, partials, out, counter);
}

// Codeword fold of one round fused with hashing the folded codeword's leaves:
// leaf i = P2(f[2i], f[2i+1]) with f[k] = fold(cw[2k], cw[2k+1], table[k]).
// BASE_IN: the input codeword is the base-field committed one (mixed fold).
template <bool BASE_IN, int T>
__global__ void P2_BOUNDS(T) fold_hash_leaves_kernel(const u64* __restrict__ cw, const u64* __restrict__ tab,
                                                               u64 c0, u64 c1, u64* __restrict__ folded,
                                                               u64* __restrict__ tree, size_t leaves) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= leaves) return;
    e2 f0, f1;
    fold_leaf_item<BASE_IN>(cw, tab, i, c0, c1, f0, f1);
    e2_st(folded + 4 * i, f0);
    e2_st(folded + 4 * i + 2, f1);
    u64 s[8] = {f0.c0, f0.c1, f1.c0, f1.c1, 0, 0, 0, 0};
    p2_permute<4>(s);
    st_digest(tree + 4 * i, s);
}

// Same in the pair form (p2_permute_pair): lane 0 of a pair folds and holds the leaf's four
// elements, lane 1 the zero half of the state.
template <bool BASE_IN, int T>
__global__ void P2_PAIR_BOUNDS(T) fold_hash_leaves_pair_kernel(const u64* __restrict__ cw,
                                                               const u64* __restrict__ tab, u64 c0, u64 c1,
                                                               u64* __restrict__ folded, u64* __restrict__ tree,
                                                               size_t leaves) {
    const size_t i = (blockIdx.x * (size_t)T + threadIdx.x) >> 1;
    const int h = threadIdx.x & 1;
    const bool live = i < leaves;
    u64 s[4] = {0, 0, 0, 0};
    if (h == 0) {
        e2 f0, f1;
        fold_leaf_item<BASE_IN>(cw, tab, live ? i : 0, c0, c1, f0, f1);
        if (live) {
            e2_st(folded + 4 * i, f0);
            e2_st(folded + 4 * i + 2, f1);
        }
        s[0] = f0.c0;
        s[1] = f0.c1;
        s[2] = f1.c0;
        s[3] = f1.c1;
    }
    p2_permute_pair(s, h);
    if (live && h == 0) st_digest(tree + 4 * i, s);
}

// Same with 8 lanes per leaf (latency-bound rounds, see mk_coop_below): every lane of a
// group folds both elements, lane l takes state element l, lanes 0..3 store.
template <bool BASE_IN>
__global__ void __launch_bounds__(256) fold_hash_leaves_coop_kernel(const u64* __restrict__ cw,
                                                                    const u64* __restrict__ tab, u64 c0, u64 c1,
                                                                    u64* __restrict__ folded, u64* __restrict__ tree,
                                                                    size_t leaves) {
    pdl_enter();
    size_t g = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 3;
    const int l = threadIdx.x & 7;
    const bool live = g < leaves;
    const size_t i = live ? g : 0;
    e2 f0, f1;
    fold_leaf_item<BASE_IN>(cw, tab, i, c0, c1, f0, f1);
    u64 x = l == 0 ? f0.c0 : l == 1 ? f0.c1 : l == 2 ? f1.c0 : l == 3 ? f1.c1 : 0;
    if (live && l < 4) folded[4 * g + l] = x;
    P2Lane c = p2_lane_consts(l);
    x = p2_permute_coop(x, l, c);
    if (live && l < 4) tree[4 * g + l] = x;
}

// Final fold (no tree): Ext2 codeword of 2*pairs elements -> pairs elements, canonical.
__global__ void fold_final_kernel(const u64* __restrict__ cw, const u64* __restrict__ tab, u64 c0, u64 c1,
                                  u64* __restrict__ out, size_t pairs, bool base_in) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= pairs) return;
    u64 o[2];
    if (base_in) fold_pair<1>(cw, i, tab[2 * i], tab[2 * i + 1], c0, c1, o);
    else fold_pair<2>(cw, i, tab[2 * i], tab[2 * i + 1], c0, c1, o);
    out[2 * i] = gl_canon(o[0]);
    out[2 * i + 1] = gl_canon(o[1]);
}

__global__ void query_gather_kernel(QueryJob job, const u64* __restrict__ leaf_idx, int num_queries, size_t per_query,
                                    u64* __restrict__ out) {
    int q = blockIdx.x;
    if (q >= num_queries) return;
    query_gather_block(job, leaf_idx[q], out + (size_t)q * per_query);
}

// ===========================================================================
// batch opening kernels (batch_open_ext2, basefold.rs:1202-1532)
// ===========================================================================

// One scaled source of a linear combination: src (base) times (c0, c1).
struct BoTerm {
    const u64* src;
    u64 c0, c1;
};

// g_p[k] = sum of the point's terms c0 * src[k]  (blockIdx.y = point; terms start[p] .. start[p+1])
__global__ void bo_accum_g_kernel(const BoTerm* __restrict__ terms, const int* __restrict__ start, size_t N,
                                  u64* __restrict__ g) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= N) return;
    const int p = blockIdx.y;
    gl3 a = gl3_zero();
    for (int j = start[p]; j < start[p + 1]; j++) gl3_add_prod(a, terms[j].c0, __ldg(terms[j].src + k));
    g[(size_t)p * N + k] = gl3_reduce(a);
}

// Outer sumcheck round 0 over all points at once (blockIdx.y = point): g_p base at g + p N,
// eq_p Ext2 at eq + 2 p N; one message summed over every point's pairs.
__global__ void __launch_bounds__(RED_THREADS) bo_round0_kernel(const u64* __restrict__ g, const u64* __restrict__ eq,
                                                                size_t N, u64* __restrict__ partials,
                                                                u64* __restrict__ out, unsigned* __restrict__ counter) {
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    const u64* gp = g + (size_t)blockIdx.y * N;
    const u64* ep = eq + (size_t)blockIdx.y * 2 * N;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < N / 2; i += (size_t)gridDim.x * blockDim.x)
        open_round0_item(gp, ep, i, acc);
    grid_reduce_finish_n<6>(acc, partials, out, counter, blockIdx.y * gridDim.x + blockIdx.x, gridDim.x * gridDim.y);
}

// Outer round k >= 1 over all points: fold eq_p, g_p (base when BH_BASE) with ch; strides in words.
template <bool BH_BASE>
__global__ void __launch_bounds__(RED_THREADS) bo_round_kernel(const u64* __restrict__ eq_in, size_t eq_stride,
                                                               const u64* __restrict__ g_in, size_t g_stride,
                                                               u64* __restrict__ eq_out, u64* __restrict__ g_out,
                                                               size_t out_stride, size_t quarter, u64 c0, u64 c1,
                                                               u64* __restrict__ partials, u64* __restrict__ out,
                                                               unsigned* __restrict__ counter) {
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    const e2 ch = e2_make(c0, c1);
    const size_t p = blockIdx.y;
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < quarter; y += (size_t)gridDim.x * blockDim.x)
        open_round_item<BH_BASE>(eq_in + p * eq_stride, g_in + p * g_stride, eq_out + p * out_stride,
                                 g_out + p * out_stride, y, ch, acc);
    grid_reduce_finish_n<6>(acc, partials, out, counter, blockIdx.y * gridDim.x + blockIdx.x, gridDim.x * gridDim.y);
}

// Combined Ext2 codeword sum_j scalar_j cw_j fused with its leaf hashes: leaf i = P2(ccw[2i] || ccw[2i+1]).
// (Up to 64 registers: the four three-word accumulators do not fit the P2_BOUNDS budget.)
template <int T>
__global__ void __launch_bounds__(T, (T) == 512 ? 2 : 4) bo_combine_leaves_kernel(const BoTerm* __restrict__ terms, int num_terms,
                                                                u64* __restrict__ ccw, u64* __restrict__ tree,
                                                                size_t leaves) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= leaves) return;
    gl3 a[4] = {gl3_zero(), gl3_zero(), gl3_zero(), gl3_zero()};
    for (int j = 0; j < num_terms; j++) {
        const BoTerm tm = terms[j];
        ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(tm.src) + i);
        gl3_add_prod(a[0], tm.c0, v.x);
        gl3_add_prod(a[1], tm.c1, v.x);
        gl3_add_prod(a[2], tm.c0, v.y);
        gl3_add_prod(a[3], tm.c1, v.y);
    }
    u64 s[8] = {gl3_reduce(a[0]), gl3_reduce(a[1]), gl3_reduce(a[2]), gl3_reduce(a[3]), 0, 0, 0, 0};
    e2_st(ccw + 4 * i, e2_make(s[0], s[1]));
    e2_st(ccw + 4 * i + 2, e2_make(s[2], s[3]));
    p2_permute<4>(s);
    st_digest(tree + 4 * i, s);
}

// Combined Ext2 evaluations sum_j scalar_j evals_j (natural order).
__global__ void bo_combine_evals_kernel(const BoTerm* __restrict__ terms, int num_terms, u64* __restrict__ out,
                                        size_t N) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= N) return;
    gl3 a0 = gl3_zero(), a1 = gl3_zero();
    for (int j = 0; j < num_terms; j++) {
        const BoTerm tm = terms[j];
        const u64 v = __ldg(tm.src + k);
        gl3_add_prod(a0, tm.c0, v);
        gl3_add_prod(a1, tm.c1, v);
    }
    e2_st(out + 2 * k, e2_make(gl3_reduce(a0), gl3_reduce(a1)));
}

// Individual query (q, j) (block q * E + j): the committed pair of evaluation j's codeword at the
// query's leaf and its authentication path, canonical: 2 + 4 depth words.
__global__ void bo_indiv_query_kernel(const u64* const* __restrict__ cws, const u64* const* __restrict__ trees,
                                      const u64* __restrict__ leaf_idx, int num_evals, int depth, size_t leaves0,
                                      u64* __restrict__ out) {
    const int q = blockIdx.x / num_evals, j = blockIdx.x % num_evals;
    const size_t leaf = leaf_idx[q];
    u64* d = out + (size_t)blockIdx.x * (2 + 4 * (size_t)depth);
    if (threadIdx.x == 0) {
        d[0] = gl_canon(cws[j][2 * leaf]);
        d[1] = gl_canon(cws[j][2 * leaf + 1]);
    }
    for (int l = threadIdx.x; l < depth; l += blockDim.x) {
        size_t off = 0, sz = leaves0;
        for (int k = 0; k < l; k++) {
            off += sz;
            sz >>= 1;
        }
        const u64* dg = trees[j] + 4 * (off + ((leaf >> l) ^ 1));
        for (int k = 0; k < 4; k++) d[2 + 4 * l + k] = gl_canon(dg[k]);
    }
}

// ===========================================================================
// host side
// ===========================================================================
static inline size_t path_words_total(int n, int lr) {
    size_t s = 0;
    for (int r = 0; r < n; r++) s += (size_t)(n + lr - 1 - r);
    return s * 4;
}
static inline size_t proof_len(int n, int lr, int q) {
    size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    return 2 + (size_t)n * 6 + (size_t)(n - 1) * 4 + ((size_t)2 << lr) + (size_t)q * per_q;
}

static unsigned red_grid(size_t work) {
    size_t cap = (size_t)num_sms() * 4;
    size_t need = (work + RED_THREADS - 1) / RED_THREADS;
    if (need < 1) need = 1;
    return (unsigned)(need < cap ? need : cap);
}

struct DevMem {
    std::vector<void*> ptrs;
    template <typename T>
    int alloc(T** p, size_t bytes) {
        void* q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, bytes < 16 ? 16 : bytes, stream());
        if (e != cudaSuccess) {
            set_error("cudaMallocAsync", e);
            return GB_ECUDA;
        }
        ptrs.push_back(q);
        *p = (T*)q;
        return GB_OK;
    }
    ~DevMem() {
        for (void* p : ptrs) cudaFreeAsync(p, stream());
    }
};

static u64* pinned(size_t words) { return thread_pinned(1, words); }
// Device address of pinned staging: the kernels write each round's record there directly, so
// reading it back takes a stream synchronisation and no copy.
static u64* mapped(u64* host) {
    void* d = nullptr;
    return host && cudaHostGetDevicePointer(&d, host, 0) == cudaSuccess ? (u64*)d : nullptr;
}

#define RC_TRY(x)                 \
    do {                          \
        int _r = (x);             \
        if (_r) return _r;        \
    } while (0)

// commit from device evaluations (natural order) into a new commitment object
static int commit_device(const u64* d_evals, int n, int lr, BfCommitment* c) {
    cudaStream_t s = stream();
    size_t N = (size_t)1 << n, L = N << lr, leaves = L / 2;
    c->num_vars = n;
    c->log_rate = lr;
    GB_CUDA_TRY(cudaMallocAsync(&c->d_evals, N * 8, s));
    GB_CUDA_TRY(cudaMallocAsync(&c->d_codeword, L * 8, s));
    GB_CUDA_TRY(cudaMallocAsync(&c->d_tree, (2 * leaves - 1) * 32, s));
    GB_CUDA_TRY(cudaMemcpyAsync(c->d_evals, d_evals, N * 8, cudaMemcpyDeviceToDevice, s));
    u64* u = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&u, N * 8, s));
    int rc = bf_transform<0>(d_evals, u, n);
    if (!rc) {
        bitrev_replicate_kernel<<<grid_for(L, 256), 256, 0, s>>>(u, c->d_codeword, n, L);
        rc = check_launch("bitrev_replicate_kernel");
    }
    cudaFreeAsync(u, s);
    RC_TRY(rc);
    RC_TRY(merkle_tree_gl_replicated(c->d_codeword, c->d_tree, leaves, n >= 1 ? lr : 0));
    u64* st = pinned(4);
    if (!st) return GB_ECUDA;
    GB_CUDA_TRY(cudaMemcpyAsync(st, c->d_tree + (2 * leaves - 2) * 4, 32, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    for (int k = 0; k < 4; k++) c->root[k] = gl_canon(st[k]);
    return GB_OK;
}

static void commitment_free(BfCommitment* c) {
    cudaStream_t s = stream();
    if (c->d_evals) cudaFreeAsync(c->d_evals, s);
    if (c->d_codeword) cudaFreeAsync(c->d_codeword, s);
    if (c->d_tree) cudaFreeAsync(c->d_tree, s);
    c->d_evals = c->d_codeword = c->d_tree = nullptr;
}

__global__ void table_weights_kernel(const u64* __restrict__ x1, u64* __restrict__ ent, size_t total) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= total) return;
    u64 x0 = ent[2 * i];
    ent[2 * i + 1] = gl_canon(gl_inv(gl_canon(gl_sub(x1[i], x0))));
}

static int table_create(int num_vars, int log_rate, int num_rounds, u64 seed, BfTable* t) {
    if (num_vars < 1 || log_rate < 0 || num_rounds < 1 || num_rounds > num_vars + log_rate || num_vars + log_rate > 40)
        return GB_EINVAL;
    t->num_vars = num_vars;
    t->log_rate = log_rate;
    t->num_rounds = num_rounds;
    t->seed = seed;
    size_t total = 0;
    t->level_offsets.clear();
    for (int i = 0; i < num_rounds; i++) {
        t->level_offsets.push_back(total);
        total += (size_t)1 << (num_vars + log_rate - i - 1);
    }
    t->total = total;
    // xorshift64 (13, 7, 17), every draw reduced mod p; x1 redrawn while equal to x0
    // (goldilocks-cuda-rs/src/basefold.rs:281-321).  The draws are sequential; the
    // inversions run on the device.
    std::vector<u64> host(2 * total);
    std::vector<u64> x1s(total);
    u64 st = seed;
    auto next = [&st]() {
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        return st % GL_P;
    };
    for (size_t k = 0; k < total; k++) {
        u64 x0 = next(), x1 = next();
        while (x1 == x0) x1 = next();
        host[2 * k] = x0;
        x1s[k] = x1;
    }
    cudaStream_t s = stream();
    u64* d_x1 = nullptr;
    GB_CUDA_TRY(cudaMalloc(&t->d_entries, total * 16));
    GB_CUDA_TRY(cudaMallocAsync(&d_x1, total * 8, s));
    GB_CUDA_TRY(cudaMemcpyAsync(t->d_entries, host.data(), total * 16, cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(d_x1, x1s.data(), total * 8, cudaMemcpyHostToDevice, s));
    table_weights_kernel<<<grid_for(total, 256), 256, 0, s>>>(d_x1, t->d_entries, total);
    GB_LAUNCH_CHECK("table_weights_kernel");
    cudaFreeAsync(d_x1, s);
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
}

// The rounds and queries of open_ext2 from its eq table onwards (basefold.rs:640-870), shared by
// the single opening (base evaluations and codeword) and the inner phase of a batch opening
// (their Ext2 linear combinations).
struct OpenRounds {
    const u64* bh;  // round-0 evaluations, natural order: base, or Ext2 when !bh_base
    bool bh_base;
    const u64* cw;  // round-0 codeword, 2^(n+lr) elements: base, or Ext2 when !cw_base
    bool cw_base;
    const u64* tree;  // its Merkle tree
    int n, lr;
};

// A second stream of the calling thread (created on first use, per device), with two events for
// ordering it against the thread's launch stream.
struct HelperStream {
    cudaStream_t s = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    int dev = -1;
    ~HelperStream() { release(); }
    void release() {
        for (auto& e : ev)
            if (e) cudaEventDestroy(e), e = nullptr;
        if (s) cudaStreamDestroy(s), s = nullptr;
    }
    int get(cudaStream_t* out) {
        int d = 0;
        GB_CUDA_TRY(cudaGetDevice(&d));
        if (!s || d != dev) {
            release();
            dev = d;
            GB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            for (auto& e : ev) GB_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        *out = s;
        return GB_OK;
    }
};
static thread_local HelperStream t_helper;

// Writes eval (2 words), n oracles, n-1 folded roots, the final codeword (2^lr Ext2) and the
// queries; *d_leaf_idx receives the device array of the query leaves (num_queries > 0).
static int open_rounds(const OpenRounds& in, const BfTable* tab, const u64* eq, gb_transcript* t, int num_queries,
                       u64* p_eval, u64* p_oracles, u64* p_roots, u64* p_final, u64* p_queries, DevMem& m,
                       u64** d_leaf_idx) {
    using namespace host;
    cudaStream_t s = stream();
    const int n = in.n, lr = in.lr;
    const size_t N = (size_t)1 << n, L = N << lr;
    u64 *eqA, *eqB, *bhA, *bhB, *partials;
    unsigned* counter;
    RC_TRY(m.alloc(&eqA, N * 8));  // N/2 Ext2
    RC_TRY(m.alloc(&eqB, N * 8));
    RC_TRY(m.alloc(&bhA, N * 8));
    RC_TRY(m.alloc(&bhB, N * 8));
    const unsigned gmax = red_grid(N / 2);
    RC_TRY(m.alloc(&partials, (size_t)gmax * 6 * 8));
    RC_TRY(m.alloc(&counter, 16));
    GB_CUDA_TRY(cudaMemsetAsync(counter, 0, 16, s));
    // folded codewords r = 0..n-1 (L >> (r+1) Ext2 each) and trees r = 0..n-2
    std::vector<u64*> fcw(n), ftree(n - 1);
    for (int r = 0; r < n; r++) RC_TRY(m.alloc(&fcw[r], (L >> (r + 1)) * 16));
    for (int r = 0; r + 1 < n; r++) {
        size_t leaves = (L >> (r + 1)) / 2;
        RC_TRY(m.alloc(&ftree[r], (2 * leaves - 1) * 32));
    }
    u64* stage = pinned(64);
    u64* rec = mapped(stage);  // records: oracle words 0..5, root 8..11
    if (!rec) return GB_ECUDA;

    // Round rd + 1's eq/bh fold and oracle (open_round_kernel) need only round rd's challenge, as do
    // round rd's codeword fold and tree: they run on the helper stream s2, beside the tree, and the
    // host reads the round's record once both streams are idle.  s2 starts after the work already
    // queued on s, and s waits for s2 before this function returns (on every path), so the caller's
    // later work and frees stay ordered after it.
    cudaStream_t s2 = nullptr;
    RC_TRY(t_helper.get(&s2));
    GB_CUDA_TRY(cudaEventRecord(t_helper.ev[0], s));
    GB_CUDA_TRY(cudaStreamWaitEvent(s2, t_helper.ev[0], 0));
    struct JoinHelper {
        cudaStream_t s, s2;
        cudaEvent_t ev;
        ~JoinHelper() {
            if (cudaEventRecord(ev, s2) == cudaSuccess) cudaStreamWaitEvent(s, ev, 0);
        }
    } join{s, s2, t_helper.ev[1]};
    auto read_rec = [&](int) -> int {  // the record's words are in `stage` once both streams are idle
        GB_CUDA_TRY(cudaStreamSynchronize(s2));
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        return GB_OK;
    };
    auto put_oracle = [&](int r) {
        // stage: c0 (2), s1 (2), c2 (2) -> c1 = s1 - c0 - c2
        E2 c0{stage[0], stage[1]}, s1{stage[2], stage[3]}, c2{stage[4], stage[5]};
        E2 c1 = e2sub(e2sub(s1, c0), c2);
        u64* o = p_oracles + (size_t)r * 6;
        o[0] = c0.c0;
        o[1] = c0.c1;
        o[2] = c1.c0;
        o[3] = c1.c1;
        o[4] = c2.c0;
        o[5] = c2.c1;
        tr_append_ext2(t, "", c0);
        tr_append_ext2(t, "", c1);
        tr_append_ext2(t, "", c2);
        return s1;
    };

    // round 0 oracle over (bh, eq); eval = c0 + s1
    if (in.bh_base)
        open_round0_kernel<true><<<red_grid(N / 2), RED_THREADS, 0, s>>>(in.bh, eq, N / 2, partials, rec, counter);
    else
        open_round0_kernel<false><<<red_grid(N / 2), RED_THREADS, 0, s>>>(in.bh, eq, N / 2, partials, rec, counter);
    GB_LAUNCH_CHECK("open_round0_kernel");
    RC_TRY(read_rec(6));
    {
        E2 c0{stage[0], stage[1]};
        E2 s1 = put_oracle(0);
        E2 ev = e2add(c0, s1);
        p_eval[0] = ev.c0;
        p_eval[1] = ev.c1;
    }

    const u64* eq_cur = eq;
    const u64* bh_cur = in.bh;
    u64* eq_bufs[2] = {eqA, eqB};
    u64* bh_bufs[2] = {bhA, bhB};
    int pp_i = 0;
    size_t sc = N;  // current sumcheck table size
    for (int rd = 0; rd < n; rd++) {
        E2 ch = tr_challenge_ext2(t, "");
        if (rd < n - 1) {
            size_t quarter = sc / 4;  // output pairs of the folded level
            u64* eo = eq_bufs[pp_i];
            u64* bo = bh_bufs[pp_i];
            unsigned g = red_grid(quarter);
            if (rd == 0 && in.bh_base)
                open_round_kernel<true><<<g, RED_THREADS, 0, s2>>>(eq_cur, bh_cur, eo, bo, quarter, ch.c0, ch.c1,
                                                                   partials, rec, counter);
            else
                open_round_kernel<false><<<g, RED_THREADS, 0, s2>>>(eq_cur, bh_cur, eo, bo, quarter, ch.c0, ch.c1,
                                                                    partials, rec, counter);
            GB_LAUNCH_CHECK("open_round_kernel");
            eq_cur = eo;
            bh_cur = bo;
            pp_i ^= 1;
            sc /= 2;
        }
        const u64* lvl = tab->d_entries + 2 * tab->level_offsets[rd];
        const u64* cw_in = rd == 0 ? in.cw : fcw[rd - 1];
        const bool base_in = rd == 0 && in.cw_base;
        size_t pairs = L >> (rd + 1);
        if (rd < n - 1) {
            size_t leaves = pairs / 2;
            const P2Form form = p2_form(leaves);
            if (form == P2_PAIR) {
                const int th = p2_pair_threads(leaves);
                const unsigned g = grid_for(2 * leaves, th);
                if (base_in && th == 256)
                    fold_hash_leaves_pair_kernel<true, 256><<<g, th, 0, s>>>(cw_in, lvl, ch.c0, ch.c1, fcw[rd],
                                                                             ftree[rd], leaves);
                else if (base_in)
                    fold_hash_leaves_pair_kernel<true, 128><<<g, th, 0, s>>>(cw_in, lvl, ch.c0, ch.c1, fcw[rd],
                                                                             ftree[rd], leaves);
                else if (th == 256)
                    fold_hash_leaves_pair_kernel<false, 256><<<g, th, 0, s>>>(cw_in, lvl, ch.c0, ch.c1, fcw[rd],
                                                                              ftree[rd], leaves);
                else
                    fold_hash_leaves_pair_kernel<false, 128><<<g, th, 0, s>>>(cw_in, lvl, ch.c0, ch.c1, fcw[rd],
                                                                              ftree[rd], leaves);
            } else if (form == P2_COOP) {
                int th = coop_threads(leaves);
                unsigned g = grid_for(leaves * 8, th);
                if (base_in)
                    GB_CUDA_TRY(launch_pdl(fold_hash_leaves_coop_kernel<true>, g, th, s, cw_in, lvl, ch.c0, ch.c1,
                                           fcw[rd], ftree[rd], leaves));
                else
                    GB_CUDA_TRY(launch_pdl(fold_hash_leaves_coop_kernel<false>, g, th, s, cw_in, lvl, ch.c0, ch.c1,
                                           fcw[rd], ftree[rd], leaves));
            } else {
                const unsigned g = grid_for(leaves, P2_WIDE);
                if (base_in)
                    fold_hash_leaves_kernel<true, P2_WIDE><<<g, P2_WIDE, 0, s>>>(cw_in, lvl, ch.c0, ch.c1, fcw[rd],
                                                                                 ftree[rd], leaves);
                else
                    fold_hash_leaves_kernel<false, P2_WIDE><<<g, P2_WIDE, 0, s>>>(cw_in, lvl, ch.c0, ch.c1, fcw[rd],
                                                                                  ftree[rd], leaves);
            }
            GB_LAUNCH_CHECK("fold_hash_leaves_kernel");
            RC_TRY(merkle_build_from_leaves(ftree[rd], leaves, rec + 8));
            RC_TRY(read_rec(12));
            put_oracle(rd + 1);
            u64* root = p_roots + (size_t)rd * 4;
            for (int k = 0; k < 4; k++) {
                root[k] = canon(stage[8 + k]);
                tr_append_u64(t, "", root[k]);
            }
        } else {
            fold_final_kernel<<<grid_for(pairs, 128), 128, 0, s>>>(cw_in, lvl, ch.c0, ch.c1, fcw[rd], pairs, base_in);
            GB_LAUNCH_CHECK("fold_final_kernel");
        }
    }
    // final codeword (2^lr Ext2)
    GB_CUDA_TRY(cudaMemcpyAsync(p_final, fcw[n - 1], ((size_t)2 << lr) * 8, cudaMemcpyDeviceToHost, s));

    // query phase: indices from the transcript, one gather launch
    const size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    if (num_queries > 0) {
        std::vector<u64> idx(num_queries);
        for (int q = 0; q < num_queries; q++) idx[q] = tr_challenge(t, "") % (u64)(L / 2);
        u64 *d_idx, *d_out;
        const u64** d_ptrs;
        RC_TRY(m.alloc(&d_idx, (size_t)num_queries * 8));
        RC_TRY(m.alloc(&d_out, (size_t)num_queries * per_q * 8));
        RC_TRY(m.alloc(&d_ptrs, (size_t)2 * n * sizeof(u64*)));
        std::vector<const u64*> ptrs(2 * n, nullptr);
        for (int r = 0; r + 1 < n; r++) {
            ptrs[r] = fcw[r];
            ptrs[n + r] = ftree[r];
        }
        GB_CUDA_TRY(cudaMemcpyAsync(d_idx, idx.data(), (size_t)num_queries * 8, cudaMemcpyHostToDevice, s));
        GB_CUDA_TRY(cudaMemcpyAsync(d_ptrs, ptrs.data(), ptrs.size() * sizeof(u64*), cudaMemcpyHostToDevice, s));
        QueryJob job{in.cw, in.tree, d_ptrs, d_ptrs + n, n, lr, !in.cw_base};
        query_gather_kernel<<<num_queries, 128, 0, s>>>(job, d_idx, num_queries, per_q, d_out);
        GB_LAUNCH_CHECK("query_gather_kernel");
        GB_CUDA_TRY(cudaMemcpyAsync(p_queries, d_out, (size_t)num_queries * per_q * 8, cudaMemcpyDeviceToHost, s));
        if (d_leaf_idx) *d_leaf_idx = d_idx;
    }
    return GB_OK;
}

static bool table_covers(const BfTable* tab, int n, int lr) {
    return tab && tab->d_entries && tab->num_rounds >= n && tab->log_rate == lr && tab->num_vars >= n;
}

// BasefoldCommitment::open_ext2 (basefold.rs:578-870) into the flat proof layout.
static int open_ext2(const BfCommitment* c, const BfTable* tab, const u64* h_point, gb_transcript* t, int num_queries,
                     u64* h_proof) {
    using namespace host;
    const int n = c->num_vars, lr = c->log_rate;
    if (n < 2 || num_queries < 0 || !table_covers(tab, n, lr)) {
        set_error_msg("gb_basefold_open_ext2: table does not cover this commitment (or num_vars < 2)");
        return GB_EINVAL;
    }
    cudaStream_t s = stream();
    const size_t N = (size_t)1 << n;
    DevMem m;
    u64 *d_point, *eq;
    RC_TRY(m.alloc(&d_point, (size_t)n * 16));
    RC_TRY(m.alloc(&eq, N * 16));

    u64* p_eval = h_proof;
    u64* p_oracles = h_proof + 2;
    u64* p_roots = p_oracles + (size_t)n * 6;
    u64* p_final = p_roots + (size_t)(n - 1) * 4;
    u64* p_queries = p_final + ((size_t)2 << lr);

    // transcript preamble
    for (int k = 0; k < 4; k++) tr_append_u64(t, "", c->root[k]);
    std::vector<u64> pt(2 * n);
    for (int i = 0; i < n; i++) {
        pt[2 * i] = canon(h_point[2 * i]);
        pt[2 * i + 1] = canon(h_point[2 * i + 1]);
        tr_append_ext2(t, "", E2{pt[2 * i], pt[2 * i + 1]});
    }
    GB_CUDA_TRY(cudaMemcpyAsync(d_point, pt.data(), (size_t)n * 16, cudaMemcpyHostToDevice, s));
    RC_TRY(eq_table(d_point, n, true, eq));
    OpenRounds in{c->d_evals, true, c->d_codeword, true, c->d_tree, n, lr};
    RC_TRY(open_rounds(in, tab, eq, t, num_queries, p_eval, p_oracles, p_roots, p_final, p_queries, m, nullptr));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
}

static inline size_t batch_proof_len(int n, int lr, int q, int num_evals) {
    size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    size_t indiv = 2 + (size_t)(n + lr - 1) * 4;
    return (size_t)n * 6 + 4 + 2 + (size_t)n * 6 + (size_t)(n - 1) * 4 + ((size_t)2 << lr) + (size_t)q * per_q +
           (size_t)q * num_evals * indiv;
}

// batch_open_ext2 (basefold.rs:1202-1532).  Outer sumcheck over sum_p eq_p g_p with every point's
// pairs in one launch per round (blockIdx.y = point); the combined codeword is formed and its
// leaves hashed in one launch; the inner phase runs the open rounds on the combined Ext2
// codeword and evaluations at the outer challenges r.
static int batch_open_ext2(BfCommitment* const* comms, int num_comms, const u64* h_points, int num_points,
                           const int* ev_poly, const int* ev_point, const u64* ev_vals, int num_evals,
                           const BfTable* tab, gb_transcript* t, int num_queries, u64* h_proof) {
    using namespace host;
    if (!comms || num_comms < 1 || !h_points || num_points < 1 || !ev_poly || !ev_point || !ev_vals ||
        num_evals < 1 || num_queries < 0 || !t || !h_proof) {
        set_error_msg("gb_basefold_batch_open_ext2: empty or null argument");
        return GB_EINVAL;
    }
    for (int c = 0; c < num_comms; c++)
        if (!comms[c]) return GB_EINVAL;
    const int n = comms[0]->num_vars, lr = comms[0]->log_rate;
    for (int c = 1; c < num_comms; c++)
        if (comms[c]->num_vars != n || comms[c]->log_rate != lr) {
            set_error_msg("gb_basefold_batch_open_ext2: commitments differ in num_vars or log_rate");
            return GB_EINVAL;
        }
    for (int i = 0; i < num_evals; i++)
        if (ev_poly[i] < 0 || ev_poly[i] >= num_comms || ev_point[i] < 0 || ev_point[i] >= num_points) {
            set_error_msg("gb_basefold_batch_open_ext2: evaluation index out of range");
            return GB_EINVAL;
        }
    if (n < 2 || !table_covers(tab, n, lr)) {
        set_error_msg("gb_basefold_batch_open_ext2: table does not cover the commitments (or num_vars < 2)");
        return GB_EINVAL;
    }
    cudaStream_t s = stream();
    const size_t N = (size_t)1 << n, L = N << lr, P = (size_t)num_points, E = (size_t)num_evals;
    u64* p_outer = h_proof;
    u64* p_croot = p_outer + (size_t)n * 6;
    u64* p_ieval = p_croot + 4;
    u64* p_inner = p_ieval + 2;
    u64* p_roots = p_inner + (size_t)n * 6;
    u64* p_final = p_roots + (size_t)(n - 1) * 4;
    u64* p_cq = p_final + ((size_t)2 << lr);
    const size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    u64* p_iq = p_cq + (size_t)num_queries * per_q;

    // 1. transcript: roots, points, claimed values
    std::vector<u64> pts(P * n * 2);
    for (size_t k = 0; k < pts.size(); k++) pts[k] = canon(h_points[k]);
    for (int c = 0; c < num_comms; c++)
        for (int k = 0; k < 4; k++) tr_append_u64(t, "", comms[c]->root[k]);
    for (size_t k = 0; k < P * n; k++) tr_append_ext2(t, "", E2{pts[2 * k], pts[2 * k + 1]});
    for (int i = 0; i < num_evals; i++) tr_append_ext2(t, "", E2{canon(ev_vals[2 * i]), canon(ev_vals[2 * i + 1])});
    // 2. weights eq(t, i), t_0 on the top index bit (basefold.rs:3008-3026)
    int ell = 0;
    while (((size_t)1 << ell) < E) ell++;
    if (E <= 1) ell = 1;
    std::vector<u64> w((size_t)1 << ell, 0);
    w[0] = 1;
    for (int i = 0; i < ell; i++) {
        u64 ti = tr_challenge(t, "");
        u64 omt = sub(1, ti);
        for (size_t j = (size_t)1 << i; j-- > 0;) {
            u64 v = w[j];
            w[2 * j] = mul(v, omt);
            w[2 * j + 1] = mul(v, ti);
        }
    }

    DevMem m;
    u64 *d_pts, *g, *eq, *eqA, *eqB, *gA, *gB, *partials;
    unsigned* counter;
    BoTerm* d_terms;
    int* d_start;
    RC_TRY(m.alloc(&d_pts, P * n * 16));
    RC_TRY(m.alloc(&g, P * N * 8));
    RC_TRY(m.alloc(&eq, P * N * 16));
    RC_TRY(m.alloc(&eqA, P * N * 8));  // per point N/2 Ext2 (stride N words)
    RC_TRY(m.alloc(&eqB, P * N * 8));
    RC_TRY(m.alloc(&gA, P * N * 8));
    RC_TRY(m.alloc(&gB, P * N * 8));
    const unsigned gx = (unsigned)std::max<size_t>(1, (red_grid(N / 2) + P - 1) / P);
    RC_TRY(m.alloc(&partials, (size_t)gx * P * 6 * 8));
    RC_TRY(m.alloc(&counter, 16));
    RC_TRY(m.alloc(&d_terms, E * sizeof(BoTerm)));
    RC_TRY(m.alloc(&d_start, (P + 1) * sizeof(int)));
    GB_CUDA_TRY(cudaMemsetAsync(counter, 0, 16, s));
    GB_CUDA_TRY(cudaMemcpyAsync(d_pts, pts.data(), P * n * 16, cudaMemcpyHostToDevice, s));
    u64* stage = pinned(64);
    u64* rec = mapped(stage);  // records: oracle words 0..5, root 8..11
    if (!rec) return GB_ECUDA;

    // 3. g_p = sum over the point's evaluations of w_i evals_i (terms grouped by point)
    std::vector<BoTerm> terms;
    std::vector<int> start(P + 1, 0);
    for (size_t p = 0; p < P; p++) {
        start[p] = (int)terms.size();
        for (size_t i = 0; i < E; i++)
            if ((size_t)ev_point[i] == p) terms.push_back(BoTerm{comms[ev_poly[i]]->d_evals, w[i], 0});
    }
    start[P] = (int)terms.size();
    GB_CUDA_TRY(cudaMemcpyAsync(d_terms, terms.data(), E * sizeof(BoTerm), cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(d_start, start.data(), (P + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    bo_accum_g_kernel<<<dim3(grid_for(N, 256), (unsigned)P), 256, 0, s>>>(d_terms, d_start, N, g);
    GB_LAUNCH_CHECK("bo_accum_g_kernel");
    // 4. eq tables
    for (size_t p = 0; p < P; p++) RC_TRY(eq_table(d_pts + p * n * 2, n, true, eq + p * N * 2));

    // 5-7. outer sumcheck: n oracles, n challenges r
    auto read_rec = [&](int) -> int {  // the record's words are in `stage` once the stream is idle
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        return GB_OK;
    };
    auto put_oracle = [&](u64* o) {
        E2 c0{stage[0], stage[1]}, s1{stage[2], stage[3]}, c2{stage[4], stage[5]};
        E2 c1 = e2sub(e2sub(s1, c0), c2);
        o[0] = c0.c0;
        o[1] = c0.c1;
        o[2] = c1.c0;
        o[3] = c1.c1;
        o[4] = c2.c0;
        o[5] = c2.c1;
        tr_append_ext2(t, "", c0);
        tr_append_ext2(t, "", c1);
        tr_append_ext2(t, "", c2);
    };
    std::vector<E2> r(n);
    bo_round0_kernel<<<dim3(gx, (unsigned)P), RED_THREADS, 0, s>>>(g, eq, N, partials, rec, counter);
    GB_LAUNCH_CHECK("bo_round0_kernel");
    RC_TRY(read_rec(6));
    put_oracle(p_outer);
    r[0] = tr_challenge_ext2(t, "");
    {
        const u64* eq_cur = eq;
        const u64* g_cur = g;
        size_t eq_stride = 2 * N, g_stride = N;
        u64* eq_bufs[2] = {eqA, eqB};
        u64* g_bufs[2] = {gA, gB};
        size_t sc = N;
        for (int rd = 1; rd < n; rd++) {
            const size_t quarter = sc / 4;
            const unsigned gq = (unsigned)std::max<size_t>(1, (red_grid(quarter) + P - 1) / P);
            u64* eo = eq_bufs[rd & 1];
            u64* go = g_bufs[rd & 1];
            if (rd == 1)
                bo_round_kernel<true><<<dim3(gq, (unsigned)P), RED_THREADS, 0, s>>>(
                    eq_cur, eq_stride, g_cur, g_stride, eo, go, N, quarter, r[rd - 1].c0, r[rd - 1].c1, partials, rec,
                    counter);
            else
                bo_round_kernel<false><<<dim3(gq, (unsigned)P), RED_THREADS, 0, s>>>(
                    eq_cur, eq_stride, g_cur, g_stride, eo, go, N, quarter, r[rd - 1].c0, r[rd - 1].c1, partials, rec,
                    counter);
            GB_LAUNCH_CHECK("bo_round_kernel");
            RC_TRY(read_rec(6));
            put_oracle(p_outer + (size_t)rd * 6);
            r[rd] = tr_challenge_ext2(t, "");
            eq_cur = eo;
            g_cur = go;
            eq_stride = g_stride = N;
            sc /= 2;
        }
    }

    // 8. scalars eq(r, point_i) w_i; combined codeword (+ leaves) and evaluations
    std::vector<E2> eqr(P);
    for (size_t p = 0; p < P; p++) {
        E2 acc{1, 0}, one{1, 0};
        for (int i = 0; i < n; i++) {
            E2 pi{pts[(p * n + i) * 2], pts[(p * n + i) * 2 + 1]};
            E2 term = e2add(e2mul(r[i], pi), e2mul(e2sub(one, r[i]), e2sub(one, pi)));
            acc = e2mul(acc, term);
        }
        eqr[p] = acc;
    }
    std::vector<BoTerm> cw_terms(E), ev_terms(E);
    for (size_t i = 0; i < E; i++) {
        E2 sc = e2mul(eqr[ev_point[i]], E2{w[i], 0});
        cw_terms[i] = BoTerm{comms[ev_poly[i]]->d_codeword, sc.c0, sc.c1};
        ev_terms[i] = BoTerm{comms[ev_poly[i]]->d_evals, sc.c0, sc.c1};
    }
    BoTerm *d_cw_terms, *d_ev_terms;
    u64 *ccw, *ctree, *cev, *ieq;
    const size_t leaves0 = L / 2;
    RC_TRY(m.alloc(&d_cw_terms, E * sizeof(BoTerm)));
    RC_TRY(m.alloc(&d_ev_terms, E * sizeof(BoTerm)));
    RC_TRY(m.alloc(&ccw, L * 16));
    RC_TRY(m.alloc(&ctree, (2 * leaves0 - 1) * 32));
    RC_TRY(m.alloc(&cev, N * 16));
    RC_TRY(m.alloc(&ieq, N * 16));
    GB_CUDA_TRY(cudaMemcpyAsync(d_cw_terms, cw_terms.data(), E * sizeof(BoTerm), cudaMemcpyHostToDevice, s));
    GB_CUDA_TRY(cudaMemcpyAsync(d_ev_terms, ev_terms.data(), E * sizeof(BoTerm), cudaMemcpyHostToDevice, s));
    if (p2_wide(leaves0))
        bo_combine_leaves_kernel<P2_WIDE><<<grid_for(leaves0, P2_WIDE), P2_WIDE, 0, s>>>(d_cw_terms, num_evals, ccw,
                                                                                       ctree, leaves0);
    else
        bo_combine_leaves_kernel<P2_NARROW><<<grid_for(leaves0, P2_NARROW), P2_NARROW, 0, s>>>(d_cw_terms, num_evals,
                                                                                             ccw, ctree, leaves0);
    GB_LAUNCH_CHECK("bo_combine_leaves_kernel");
    bo_combine_evals_kernel<<<grid_for(N, 256), 256, 0, s>>>(d_ev_terms, num_evals, cev, N);
    GB_LAUNCH_CHECK("bo_combine_evals_kernel");
    // 9. combined tree and root
    RC_TRY(merkle_build_from_leaves(ctree, leaves0, rec + 8));
    RC_TRY(read_rec(12));
    for (int k = 0; k < 4; k++) {
        p_croot[k] = canon(stage[8 + k]);
        tr_append_u64(t, "", p_croot[k]);
    }
    // 10. inner phase at r
    std::vector<u64> rr(2 * n);
    for (int i = 0; i < n; i++) {
        rr[2 * i] = r[i].c0;
        rr[2 * i + 1] = r[i].c1;
    }
    u64* d_r = d_pts;  // the points are no longer needed on the device
    GB_CUDA_TRY(cudaMemcpyAsync(d_r, rr.data(), (size_t)n * 16, cudaMemcpyHostToDevice, s));
    RC_TRY(eq_table(d_r, n, true, ieq));
    OpenRounds in{cev, false, ccw, false, ctree, n, lr};
    u64* d_leaf = nullptr;
    RC_TRY(open_rounds(in, tab, ieq, t, num_queries, p_ieval, p_inner, p_roots, p_final, p_cq, m, &d_leaf));
    // 11. individual queries
    if (num_queries > 0) {
        const int depth = n + lr - 1;
        const size_t indiv = 2 + 4 * (size_t)depth;
        std::vector<const u64*> ptrs(2 * E);
        for (size_t i = 0; i < E; i++) {
            ptrs[i] = comms[ev_poly[i]]->d_codeword;
            ptrs[E + i] = comms[ev_poly[i]]->d_tree;
        }
        const u64** d_ptrs;
        u64* d_out;
        RC_TRY(m.alloc(&d_ptrs, 2 * E * sizeof(u64*)));
        RC_TRY(m.alloc(&d_out, (size_t)num_queries * E * indiv * 8));
        GB_CUDA_TRY(cudaMemcpyAsync(d_ptrs, ptrs.data(), 2 * E * sizeof(u64*), cudaMemcpyHostToDevice, s));
        bo_indiv_query_kernel<<<(unsigned)(num_queries * E), 64, 0, s>>>(d_ptrs, d_ptrs + E, d_leaf, num_evals, depth,
                                                                         leaves0, d_out);
        GB_LAUNCH_CHECK("bo_indiv_query_kernel");
        GB_CUDA_TRY(cudaMemcpyAsync(p_iq, d_out, (size_t)num_queries * E * indiv * 8, cudaMemcpyDeviceToHost, s));
    }
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

// ---------------------------------------------------------------- reference ABI
int basefold_bit_reverse_gl_ffi(uint64_t* d, int log_n) {
    if (log_n < 0 || log_n > 40) return GB_EINVAL;
    bit_reverse_inplace_kernel<1><<<grid_for((size_t)1 << log_n, 256), 256, 0, stream()>>>(d, log_n);
    return check_launch("basefold_bit_reverse_gl_ffi");
}
int basefold_bit_reverse_ext2_ffi(uint64_t* d, int log_n) {
    if (log_n < 0 || log_n > 40) return GB_EINVAL;
    bit_reverse_inplace_kernel<2><<<grid_for((size_t)1 << log_n, 256), 256, 0, stream()>>>(d, log_n);
    return check_launch("basefold_bit_reverse_ext2_ffi");
}

int basefold_bhc_interpolate_ffi(const uint64_t* d_evals, uint64_t* d_coeffs, uint64_t* d_bh_evals, int num_vars) {
    if (num_vars < 0 || num_vars > 40) return GB_EINVAL;
    size_t N = (size_t)1 << num_vars;
    RC_TRY(bf_transform<1>(d_evals, d_coeffs, num_vars));
    GB_CUDA_TRY(cudaMemcpyAsync(d_bh_evals, d_evals, N * 8, cudaMemcpyDeviceToDevice, stream()));
    bit_reverse_inplace_kernel<1><<<grid_for(N, 256), 256, 0, stream()>>>(d_bh_evals, num_vars);
    GB_LAUNCH_CHECK("basefold_bhc_interpolate_ffi");
    return sync_stream("basefold_bhc_interpolate_ffi");
}

int basefold_encode_ffi(const uint64_t* d_coeffs, uint64_t* d_codeword, int num_vars, int log_rate) {
    if (num_vars < 0 || log_rate < 0 || num_vars + log_rate > 40) return GB_EINVAL;
    cudaStream_t s = stream();
    size_t N = (size_t)1 << num_vars, L = N << log_rate;
    u64* u = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&u, N * 8, s));
    int rc = bf_transform<2>(d_coeffs, u, num_vars);
    if (!rc) {
        bitrev_replicate_kernel<<<grid_for(L, 256), 256, 0, s>>>(u, d_codeword, num_vars, L);
        rc = check_launch("basefold_encode_ffi");
    }
    cudaFreeAsync(u, s);
    RC_TRY(rc);
    return sync_stream("basefold_encode_ffi");
}

int basefold_fold_gl_ffi(const uint64_t* cw, const uint64_t* tab, uint64_t ch, uint64_t* out, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    bf_fold_kernel<0><<<grid_for(pairs, 256), 256, 0, stream()>>>(cw, tab, ch, 0, out, pairs);
    return check_launch("basefold_fold_gl_ffi");
}
int basefold_fold_mixed_ffi(const uint64_t* cw, const uint64_t* tab, uint64_t c0, uint64_t c1, uint64_t* out, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    bf_fold_kernel<1><<<grid_for(pairs, 256), 256, 0, stream()>>>(cw, tab, c0, c1, out, pairs);
    return check_launch("basefold_fold_mixed_ffi");
}
int basefold_fold_ext2_ffi(const uint64_t* cw, const uint64_t* tab, uint64_t c0, uint64_t c1, uint64_t* out, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    bf_fold_kernel<2><<<grid_for(pairs, 256), 256, 0, stream()>>>(cw, tab, c0, c1, out, pairs);
    return check_launch("basefold_fold_ext2_ffi");
}

int basefold_sumcheck_interp_gl_ffi(uint64_t* d, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    sc_interp_kernel<false><<<grid_for(pairs, 256), 256, 0, stream()>>>(d, pairs);
    return check_launch("basefold_sumcheck_interp_gl_ffi");
}
int basefold_sumcheck_interp_ext2_ffi(uint64_t* d, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    sc_interp_kernel<true><<<grid_for(pairs, 256), 256, 0, stream()>>>(d, pairs);
    return check_launch("basefold_sumcheck_interp_ext2_ffi");
}

int basefold_sumcheck_product_gl_ffi(const uint64_t* eq, const uint64_t* bh, uint64_t* p0, uint64_t* p1, uint64_t* p2,
                                     int pairs, int blocks) {
    if (pairs < 0 || blocks <= 0) return GB_EINVAL;
    sc_product_kernel<false, false><<<blocks, RED_THREADS, 0, stream()>>>(eq, bh, p0, p1, p2, (size_t)pairs);
    return check_launch("basefold_sumcheck_product_gl_ffi");
}
int basefold_sumcheck_product_mixed_ffi(const uint64_t* eq, const uint64_t* bh, uint64_t* p0, uint64_t* p1,
                                        uint64_t* p2, int pairs, int blocks) {
    if (pairs < 0 || blocks <= 0) return GB_EINVAL;
    sc_product_kernel<true, false><<<blocks, RED_THREADS, 0, stream()>>>(eq, bh, p0, p1, p2, (size_t)pairs);
    return check_launch("basefold_sumcheck_product_mixed_ffi");
}
int basefold_sumcheck_product_ext2_ffi(const uint64_t* eq, const uint64_t* bh, uint64_t* p0, uint64_t* p1,
                                       uint64_t* p2, int pairs, int blocks) {
    if (pairs < 0 || blocks <= 0) return GB_EINVAL;
    sc_product_kernel<true, true><<<blocks, RED_THREADS, 0, stream()>>>(eq, bh, p0, p1, p2, (size_t)pairs);
    return check_launch("basefold_sumcheck_product_ext2_ffi");
}

int basefold_sumcheck_eval_gl_ffi(const uint64_t* d, uint64_t ch, uint64_t* out, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    sc_eval_kernel<0><<<grid_for(pairs, 256), 256, 0, stream()>>>(d, ch, 0, out, pairs);
    return check_launch("basefold_sumcheck_eval_gl_ffi");
}
int basefold_sumcheck_eval_mixed_ffi(const uint64_t* d, uint64_t c0, uint64_t c1, uint64_t* out, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    sc_eval_kernel<1><<<grid_for(pairs, 256), 256, 0, stream()>>>(d, c0, c1, out, pairs);
    return check_launch("basefold_sumcheck_eval_mixed_ffi");
}
int basefold_sumcheck_eval_ext2_ffi(const uint64_t* d, uint64_t c0, uint64_t c1, uint64_t* out, int pairs) {
    if (pairs < 0) return GB_EINVAL;
    if (!pairs) return GB_OK;
    sc_eval_kernel<2><<<grid_for(pairs, 256), 256, 0, stream()>>>(d, c0, c1, out, pairs);
    return check_launch("basefold_sumcheck_eval_ext2_ffi");
}

int fused_sumcheck_round_ext2_ffi(const uint64_t* eq_in, const uint64_t* bh_in, uint64_t c0, uint64_t c1,
                                  uint64_t* eq_out, uint64_t* bh_out, uint64_t* p0, uint64_t* p1, uint64_t* p2, int pairs,
                                  int blocks) {
    if (pairs < 0 || blocks <= 0) return GB_EINVAL;
    sc_fused_round_ref_kernel<<<blocks, RED_THREADS, 0, stream()>>>(eq_in, bh_in, c0, c1, eq_out, bh_out, p0, p1, p2,
                                                                    (size_t)pairs);
    return check_launch("fused_sumcheck_round_ext2_ffi");
}

int basefold_dot_product_gl_ffi(const uint64_t* a, const uint64_t* b, uint64_t* partial, int n, int blocks) {
    if (n < 0 || blocks <= 0) return GB_EINVAL;
    dot_product_kernel<false><<<blocks, RED_THREADS, 0, stream()>>>(a, b, partial, (size_t)n);
    return check_launch("basefold_dot_product_gl_ffi");
}
int basefold_dot_product_mixed_ffi(const uint64_t* a, const uint64_t* b, uint64_t* partial, int n, int blocks) {
    if (n < 0 || blocks <= 0) return GB_EINVAL;
    dot_product_kernel<true><<<blocks, RED_THREADS, 0, stream()>>>(a, b, partial, (size_t)n);
    return check_launch("basefold_dot_product_mixed_ffi");
}

// ---------------------------------------------------------------- gb_* drivers
int gb_basefold_table_create(int num_vars, int log_rate, int num_rounds, uint64_t seed, void** handle) {
    if (!handle) return GB_EINVAL;
    BfTable* t = new BfTable();
    int rc = table_create(num_vars, log_rate, num_rounds, seed, t);
    if (rc) {
        if (t->d_entries) cudaFree(t->d_entries);
        delete t;
        return rc;
    }
    *handle = t;
    return GB_OK;
}

int gb_basefold_table_destroy(void* handle) {
    BfTable* t = (BfTable*)handle;
    if (!t) return GB_OK;
    if (t->d_entries) cudaFree(t->d_entries);
    delete t;
    return GB_OK;
}

int gb_basefold_table_info(void* handle, uint64_t** d_entries, uint64_t* h_level_offsets) {
    BfTable* t = (BfTable*)handle;
    if (!t) return GB_EINVAL;
    if (d_entries) *d_entries = t->d_entries;
    if (h_level_offsets)
        for (int i = 0; i < t->num_rounds; i++) h_level_offsets[i] = t->level_offsets[i];
    return GB_OK;
}

int gb_basefold_commit(const uint64_t* d_evals, const uint64_t* h_evals, int num_vars, int log_rate, void** handle,
                       uint64_t root[4]) {
    if (!handle || (!d_evals == !h_evals) || num_vars < 0 || log_rate < 0 || num_vars + log_rate < 1 ||
        num_vars + log_rate > 40)
        return GB_EINVAL;
    cudaStream_t s = stream();
    size_t N = (size_t)1 << num_vars;
    u64* tmp = nullptr;
    const u64* src = d_evals;
    if (h_evals) {
        GB_CUDA_TRY(cudaMallocAsync(&tmp, N * 8, s));
        GB_CUDA_TRY(cudaMemcpyAsync(tmp, h_evals, N * 8, cudaMemcpyHostToDevice, s));
        src = tmp;
    }
    BfCommitment* c = new BfCommitment();
    int rc = commit_device(src, num_vars, log_rate, c);
    if (tmp) cudaFreeAsync(tmp, s);
    if (rc) {
        commitment_free(c);
        delete c;
        return rc;
    }
    if (root)
        for (int k = 0; k < 4; k++) root[k] = c->root[k];
    *handle = c;
    return GB_OK;
}

int gb_basefold_commitment_destroy(void* handle) {
    BfCommitment* c = (BfCommitment*)handle;
    if (!c) return GB_OK;
    commitment_free(c);
    delete c;
    return GB_OK;
}

int gb_basefold_commitment_info(void* handle, uint64_t** d_codeword, uint64_t** d_tree, uint64_t** d_evals,
                                uint64_t root[4]) {
    BfCommitment* c = (BfCommitment*)handle;
    if (!c) return GB_EINVAL;
    if (d_codeword) *d_codeword = c->d_codeword;
    if (d_tree) *d_tree = c->d_tree;
    if (d_evals) *d_evals = c->d_evals;
    if (root)
        for (int k = 0; k < 4; k++) root[k] = c->root[k];
    return GB_OK;
}

size_t gb_basefold_proof_len(int num_vars, int log_rate, int num_queries) {
    return proof_len(num_vars, log_rate, num_queries);
}

int gb_basefold_open_ext2(void* commitment, void* table, const uint64_t* h_point, gb_transcript* t, int num_queries,
                          uint64_t* h_proof) {
    if (!commitment || !table || !h_point || !t || !h_proof) return GB_EINVAL;
    return open_ext2((BfCommitment*)commitment, (BfTable*)table, h_point, t, num_queries, h_proof);
}

size_t gb_basefold_batch_proof_len(int num_vars, int log_rate, int num_queries, int num_evals) {
    if (num_vars < 2 || log_rate < 0 || num_queries < 0 || num_evals < 1) return 0;
    return batch_proof_len(num_vars, log_rate, num_queries, num_evals);
}

int gb_basefold_batch_open_ext2(void* const* commitments, int num_commitments, const uint64_t* h_points,
                                int num_points, const int* eval_poly, const int* eval_point,
                                const uint64_t* h_eval_values, int num_evals, void* table, gb_transcript* t,
                                int num_queries, uint64_t* h_proof) {
    if (!table) return GB_EINVAL;
    return batch_open_ext2(reinterpret_cast<BfCommitment* const*>(commitments), num_commitments, h_points, num_points,
                           eval_poly, eval_point, h_eval_values, num_evals, (BfTable*)table, t, num_queries, h_proof);
}

}  // extern "C"
