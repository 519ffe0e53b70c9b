// Almost-Goldilocks (q = 2^64 - 2^32 - 31) sumcheck, eq tables and the batched same-point
// sumcheck: the reference ABI of almost-goldilocks-cuda-rs (src/ffi.rs:161-196, :228-275,
// implemented by cuda/wrapper.cu:642-707, :811-925 over cuda_almost_goldilocks/
// almost_sumcheck_prover.cuh and almost_eq_lagrange.cuh).
//
// Same grid shapes as the reference (256-thread blocks, grid-stride loops, the caller's block
// count for the messages, at most 256 blocks for the folds), so that every per-block partial
// sum covers the same pairs and equals the reference's value mod q.  Outputs are canonical.
#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "agl.cuh"
#include "common.cuh"

namespace gb {

constexpr int AGL_BLOCK = 256;
constexpr int AGL_MAX_D = 8;

template <int W>
__device__ __forceinline__ void agl_block_sum(u64 (&acc)[W], u64* sh) {
    // warp tree, then one value per warp through shared memory
#pragma unroll
    for (int w = 0; w < W; w++) {
        u64 v = acc[w];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = agl_add(v, __shfl_down_sync(0xffffffffu, v, o));
        acc[w] = v;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int w = 0; w < W; w++) sh[warp * W + w] = acc[w];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < W; w++) {
            u64 v = sh[w];
            for (int k = 1; k < AGL_BLOCK / 32; k++) v = agl_add(v, sh[k * W + w]);
            acc[w] = agl_canon(v);
        }
    }
}

// per-block partial messages: out[block][c] (EXT: [block][c][2]), c = 0..D
template <int D, bool EXT>
__global__ void __launch_bounds__(AGL_BLOCK) agl_round_msg_kernel(const u64* __restrict__ polys, u64* __restrict__ partial,
                                                                  size_t stride, size_t half) {
    constexpr int W = EXT ? 2 * (D + 1) : D + 1;
    __shared__ u64 sh[(AGL_BLOCK / 32) * W];
    u64 acc[W];
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = 0;
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        if constexpr (EXT) {
            ae2 v[D], dl[D];
#pragma unroll
            for (int i = 0; i < D; i++) {
                const u64* p = polys + (size_t)i * 2 * stride + 4 * y;
                v[i] = ae2_make(p[0], p[1]);
                dl[i] = ae2_sub(ae2_make(p[2], p[3]), v[i]);
            }
#pragma unroll
            for (int c = 0; c <= D; c++) {
                ae2 prod = v[0];
#pragma unroll
                for (int i = 1; i < D; i++) prod = ae2_mul(prod, v[i]);
                acc[2 * c] = agl_add(acc[2 * c], prod.c0);
                acc[2 * c + 1] = agl_add(acc[2 * c + 1], prod.c1);
                if (c < D)
#pragma unroll
                    for (int i = 0; i < D; i++) v[i] = ae2_add(v[i], dl[i]);
            }
        } else {
            u64 v[D], dl[D];
#pragma unroll
            for (int i = 0; i < D; i++) {
                const u64* p = polys + (size_t)i * stride + 2 * y;
                v[i] = p[0];
                dl[i] = agl_sub(p[1], p[0]);
            }
#pragma unroll
            for (int c = 0; c <= D; c++) {
                u64 prod = v[0];
#pragma unroll
                for (int i = 1; i < D; i++) prod = agl_mul(prod, v[i]);
                acc[c] = agl_add(acc[c], prod);
                if (c < D)
#pragma unroll
                    for (int i = 0; i < D; i++) v[i] = agl_add(v[i], dl[i]);
            }
        }
    }
    agl_block_sum<W>(acc, sh);
    if (threadIdx.x == 0)
#pragma unroll
        for (int w = 0; w < W; w++) partial[(size_t)blockIdx.x * W + w] = acc[w];
}

template <bool EXT>
__global__ void agl_fold_kernel(const u64* __restrict__ in, u64* __restrict__ out, u64 r0, u64 r1, int d, size_t stride,
                                size_t half) {
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        for (int i = 0; i < d; i++) {
            if constexpr (EXT) {
                const u64* p = in + (size_t)i * 2 * stride + 4 * y;
                ae2 a = ae2_make(p[0], p[1]), b = ae2_make(p[2], p[3]);
                ae2 f = ae2_canon(ae2_add(a, ae2_mul(ae2_make(r0, r1), ae2_sub(b, a))));
                u64* q = out + (size_t)i * 2 * stride + 2 * y;
                q[0] = f.c0;
                q[1] = f.c1;
            } else {
                const u64* p = in + (size_t)i * stride + 2 * y;
                out[(size_t)i * stride + y] = agl_canon(agl_add(p[0], agl_mul(r0, agl_sub(p[1], p[0]))));
            }
        }
    }
}

// batched same-point (eq, f) pairs: leaf l's polys at l * 4 * original_size u64; partials
// [block_x][leaf][c][2] for c = 0, 1, 2
__global__ void __launch_bounds__(AGL_BLOCK) aext2_batched_msg_kernel(const u64* __restrict__ polys, u64* __restrict__ partial,
                                                                      size_t original_size, size_t half, int leaves) {
    __shared__ u64 sh[(AGL_BLOCK / 32) * 6];
    const int leaf = blockIdx.y;
    const u64* lp = polys + (size_t)leaf * 4 * original_size;
    const u64* fp = lp + 2 * original_size;
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        ae2 e0 = ae2_make(lp[4 * y], lp[4 * y + 1]), e1 = ae2_make(lp[4 * y + 2], lp[4 * y + 3]);
        ae2 f0 = ae2_make(fp[4 * y], fp[4 * y + 1]), f1 = ae2_make(fp[4 * y + 2], fp[4 * y + 3]);
        ae2 p0 = ae2_mul(e0, f0), p1 = ae2_mul(e1, f1);
        ae2 e2v = ae2_sub(ae2_add(e1, e1), e0), f2v = ae2_sub(ae2_add(f1, f1), f0);
        ae2 p2 = ae2_mul(e2v, f2v);
        acc[0] = agl_add(acc[0], p0.c0);
        acc[1] = agl_add(acc[1], p0.c1);
        acc[2] = agl_add(acc[2], p1.c0);
        acc[3] = agl_add(acc[3], p1.c1);
        acc[4] = agl_add(acc[4], p2.c0);
        acc[5] = agl_add(acc[5], p2.c1);
    }
    agl_block_sum<6>(acc, sh);
    if (threadIdx.x == 0) {
        u64* o = partial + ((size_t)blockIdx.x * leaves + leaf) * 6;
#pragma unroll
        for (int w = 0; w < 6; w++) o[w] = acc[w];
    }
}

// Round 0 with a binary f (packed bits of leaf l at packed + l * packed_words; the eq slot of
// polys is read, the f slot ignored): c = 0: e0 f0, c = 1: e1 f1, c = 2: (2 e1 - e0)(2 f1 - f0),
// by selective additions (almost_sumcheck_prover.cuh:709-800).  Partials as the batched message.
__global__ void __launch_bounds__(AGL_BLOCK) aext2_round0_binary_msg_kernel(const u64* __restrict__ polys,
                                                                            const u64* __restrict__ packed,
                                                                            u64* __restrict__ partial,
                                                                            size_t original_size, size_t half,
                                                                            int leaves, size_t packed_words) {
    __shared__ u64 sh[(AGL_BLOCK / 32) * 6];
    const int leaf = blockIdx.y;
    const u64* lp = polys + (size_t)leaf * 4 * original_size;
    const u64* bits = packed + (size_t)leaf * packed_words;
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        const ae2 e0 = ae2_make(lp[4 * y], lp[4 * y + 1]), e1 = ae2_make(lp[4 * y + 2], lp[4 * y + 3]);
        const u64 w = bits[(2 * y) >> 6] >> ((2 * y) & 63);
        const int f0 = (int)(w & 1), f1 = (int)((w >> 1) & 1);
        if (f0) {
            acc[0] = agl_add(acc[0], e0.c0);
            acc[1] = agl_add(acc[1], e0.c1);
        }
        if (f1) {
            acc[2] = agl_add(acc[2], e1.c0);
            acc[3] = agl_add(acc[3], e1.c1);
        }
        const int f2 = 2 * f1 - f0;  // in {-1, 0, 1, 2}
        if (f2) {
            ae2 e2v = ae2_sub(ae2_add(e1, e1), e0);
            if (f2 == 2) e2v = ae2_add(e2v, e2v);
            if (f2 < 0) {
                acc[4] = agl_sub(acc[4], e2v.c0);
                acc[5] = agl_sub(acc[5], e2v.c1);
            } else {
                acc[4] = agl_add(acc[4], e2v.c0);
                acc[5] = agl_add(acc[5], e2v.c1);
            }
        }
    }
    agl_block_sum<6>(acc, sh);
    if (threadIdx.x == 0) {
        u64* o = partial + ((size_t)blockIdx.x * leaves + leaf) * 6;
#pragma unroll
        for (int w = 0; w < 6; w++) o[w] = acc[w];
    }
}

// the matching fold: eq' = e0 + r (e1 - e0); f' = f0 + r (f1 - f0) in {0, r, 1 - r, 1}
__global__ void aext2_round0_binary_fold_kernel(const u64* __restrict__ in, const u64* __restrict__ packed,
                                                u64* __restrict__ out, u64 r0, u64 r1, size_t original_size,
                                                size_t half, size_t packed_words) {
    const int leaf = blockIdx.y;
    const u64* il = in + (size_t)leaf * 4 * original_size;
    const u64* bits = packed + (size_t)leaf * packed_words;
    u64* ol = out + (size_t)leaf * 4 * original_size;
    const ae2 r = ae2_make(r0, r1);
    const ae2 omr = ae2_sub(ae2_make(1, 0), r);
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        const ae2 a = ae2_make(il[4 * y], il[4 * y + 1]), b = ae2_make(il[4 * y + 2], il[4 * y + 3]);
        const ae2 e = ae2_canon(ae2_add(a, ae2_mul(r, ae2_sub(b, a))));
        ol[2 * y] = e.c0;
        ol[2 * y + 1] = e.c1;
        const u64 w = bits[(2 * y) >> 6] >> ((2 * y) & 63);
        const int f0 = (int)(w & 1), f1 = (int)((w >> 1) & 1);
        const ae2 f = f0 ? (f1 ? ae2_make(1, 0) : omr) : (f1 ? r : ae2_make(0, 0));
        const ae2 fc = ae2_canon(f);
        ol[2 * original_size + 2 * y] = fc.c0;
        ol[2 * original_size + 2 * y + 1] = fc.c1;
    }
}

// binary (or ternary pos - neg) bits of leaf l lifted to Ext2 at dst + l * leaf_words + off
__global__ void aext2_lift_kernel(const u64* __restrict__ pos, const u64* __restrict__ neg, u64* __restrict__ dst,
                                  size_t original_size, size_t packed_words, size_t leaf_words, size_t off) {
    const int leaf = blockIdx.y;
    const u64* pl = pos + (size_t)leaf * packed_words;
    const u64* nl = neg ? neg + (size_t)leaf * packed_words : nullptr;
    u64* d = dst + (size_t)leaf * leaf_words + off;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < original_size; i += (size_t)gridDim.x * blockDim.x) {
        const u64 p = (pl[i >> 6] >> (i & 63)) & 1, n = nl ? (nl[i >> 6] >> (i & 63)) & 1 : 0;
        d[2 * i] = agl_sub(p, n);  // 0, 1 or q - 1 (pos and neg disjoint)
        d[2 * i + 1] = 0;
    }
}

// per-(block, plane) partial sums of eq[i] over the set bits of each plane (shared eq table)
__global__ void __launch_bounds__(AGL_BLOCK) aext2_selective_add_kernel(const u64* __restrict__ eq,
                                                                        const u64* __restrict__ planes,
                                                                        u64* __restrict__ partial, size_t total,
                                                                        int n_planes, size_t packed_words) {
    __shared__ u64 sh[(AGL_BLOCK / 32) * 2];
    const int plane = blockIdx.y;
    const u64* pb = planes + (size_t)plane * packed_words;
    u64 acc[2] = {0, 0};
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x)
        if ((pb[i >> 6] >> (i & 63)) & 1) {
            acc[0] = agl_add(acc[0], eq[2 * i]);
            acc[1] = agl_add(acc[1], eq[2 * i + 1]);
        }
    agl_block_sum<2>(acc, sh);
    if (threadIdx.x == 0) {
        partial[((size_t)blockIdx.x * n_planes + plane) * 2] = acc[0];
        partial[((size_t)blockIdx.x * n_planes + plane) * 2 + 1] = acc[1];
    }
}

__global__ void aext2_batched_fold_kernel(const u64* __restrict__ in, u64* __restrict__ out, u64 r0, u64 r1,
                                          size_t original_size, size_t half) {
    const int leaf = blockIdx.y;
    const u64* il = in + (size_t)leaf * 4 * original_size;
    u64* ol = out + (size_t)leaf * 4 * original_size;
    const ae2 r = ae2_make(r0, r1);
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const u64* p = il + (size_t)i * 2 * original_size + 4 * y;
            ae2 a = ae2_make(p[0], p[1]), b = ae2_make(p[2], p[3]);
            ae2 f = ae2_canon(ae2_add(a, ae2_mul(r, ae2_sub(b, a))));
            u64* q = ol + (size_t)i * 2 * original_size + 2 * y;
            q[0] = f.c0;
            q[1] = f.c1;
        }
    }
}

// eq(r, x) for every x in {0,1}^n (variable i <-> bit i), in place in `out`: doubling steps
// out[x + h] = out[x] r_i, out[x] = out[x] - out[x] r_i.  One block per table (grid.y = leaf);
// all threads of the block take part in every step.
template <bool EXT>
__global__ void __launch_bounds__(1024) agl_eq_table_kernel(const u64* __restrict__ r_all, int r_stride,
                                                            u64* __restrict__ out_all, int n, size_t leaf_stride) {
    constexpr int W = EXT ? 2 : 1;
    const u64* r = r_all + (size_t)blockIdx.y * r_stride * W;
    u64* out = out_all + (size_t)blockIdx.y * leaf_stride * W;
    if (threadIdx.x == 0) {
        out[0] = 1;
        if (EXT) out[1] = 0;
    }
    __syncthreads();
    for (int i = 0; i < n; i++) {
        const size_t h = (size_t)1 << i;
        for (size_t x = threadIdx.x; x < h; x += blockDim.x) {
            if constexpr (EXT) {
                ae2 a = ae2_make(out[2 * x], out[2 * x + 1]);
                ae2 ar = ae2_mul(a, ae2_make(r[2 * i], r[2 * i + 1]));
                ae2 lo = ae2_canon(ae2_sub(a, ar));
                ar = ae2_canon(ar);
                out[2 * (x + h)] = ar.c0;
                out[2 * (x + h) + 1] = ar.c1;
                out[2 * x] = lo.c0;
                out[2 * x + 1] = lo.c1;
            } else {
                u64 a = out[x], ar = agl_mul(a, r[i]);
                out[x + h] = agl_canon(ar);
                out[x] = agl_canon(agl_sub(a, ar));
            }
        }
        __syncthreads();
    }
}

// Larger tables: eq(r, x) = lo[x mod 2^k] hi[x >> k] from two half tables.
// lo/hi: per-leaf slots of src_stride entries
template <bool EXT>
__global__ void agl_eq_expand_kernel(const u64* __restrict__ lo_all, const u64* __restrict__ hi_all, int k, int n,
                                     size_t src_stride, u64* __restrict__ out_all, size_t leaf_stride) {
    constexpr int W = EXT ? 2 : 1;
    const size_t total = (size_t)1 << n;
    const u64* lo = lo_all + (size_t)blockIdx.y * src_stride * W;
    const u64* hi = hi_all + (size_t)blockIdx.y * src_stride * W;
    u64* out = out_all + (size_t)blockIdx.y * leaf_stride * W;
    const size_t mask = ((size_t)1 << k) - 1;
    for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
        if constexpr (EXT) {
            ae2 v = ae2_canon(ae2_mul(ae2_make(lo[2 * (x & mask)], lo[2 * (x & mask) + 1]),
                                      ae2_make(hi[2 * (x >> k)], hi[2 * (x >> k) + 1])));
            out[2 * x] = v.c0;
            out[2 * x + 1] = v.c1;
        } else {
            out[x] = agl_canon(agl_mul(lo[x & mask], hi[x >> k]));
        }
    }
}

// leaves tables of n variables: r [leaf][n](W), result [leaf][leaf_stride](W) in `res`.  For
// n > 10 the two half tables go to `scratch` (same shape), lo at [0, 2^k) and hi at
// [leaf_stride / 2, ...) of each leaf's slot (2^k, 2^(n-k) <= 2^(n-1) <= leaf_stride / 2).
template <bool EXT>
static int agl_eq_tables(const u64* d_r, int n, int leaves, size_t leaf_stride, u64* res, u64* scratch,
                         cudaStream_t s) {
    constexpr int W = EXT ? 2 : 1;
    if (n <= 10) {
        agl_eq_table_kernel<EXT><<<dim3(1, leaves), 1024, 0, s>>>(d_r, n, res, n, leaf_stride);
        return check_launch("agl_eq_table_kernel");
    }
    const int k = n / 2;
    agl_eq_table_kernel<EXT><<<dim3(1, leaves), 1024, 0, s>>>(d_r, n, scratch, k, leaf_stride);
    GB_LAUNCH_CHECK("agl_eq_table_kernel");
    agl_eq_table_kernel<EXT><<<dim3(1, leaves), 1024, 0, s>>>(d_r + (size_t)k * W, n, scratch + (leaf_stride / 2) * W,
                                                              n - k, leaf_stride);
    GB_LAUNCH_CHECK("agl_eq_table_kernel");
    const size_t total = (size_t)1 << n;
    unsigned gx = (unsigned)((total + 255) / 256 > 4096 ? 4096 : (total + 255) / 256);
    agl_eq_expand_kernel<EXT><<<dim3(gx, leaves), 256, 0, s>>>(scratch, scratch + (leaf_stride / 2) * W, k, n,
                                                               leaf_stride, res, leaf_stride);
    return check_launch("agl_eq_expand_kernel");
}

}  // namespace gb

using namespace gb;

namespace {
template <bool EXT>
struct AglMsg {
    template <int D>
    struct K {
        static int run(const u64* polys, u64* partial, size_t stride, size_t half, int blocks) {
            agl_round_msg_kernel<D, EXT><<<blocks, AGL_BLOCK, 0, stream()>>>(polys, partial, stride, half);
            return check_launch("agl_round_msg_kernel");
        }
    };
};
template <template <int> class F, typename... A>
int agl_dispatch(int d, A... args) {
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
unsigned fold_grid(size_t half) {
    size_t g = (half + AGL_BLOCK - 1) / AGL_BLOCK;
    return (unsigned)(g < 1 ? 1 : g > 256 ? 256 : g);
}
}  // namespace

extern "C" {

int agl_sumcheck_round_message_ffi(const uint64_t* d_polys, uint64_t* d_partial, int d, size_t original_size,
                                   size_t half, int num_blocks) {
    if (num_blocks <= 0 || d < 1 || d > AGL_MAX_D) return GB_EINVAL;
    return agl_dispatch<AglMsg<false>::K>(d, d_polys, d_partial, original_size, half, num_blocks);
}

int aext2_sumcheck_round_message_ffi(const uint64_t* d_polys, uint64_t* d_partial, int d, size_t original_size,
                                     size_t half, int num_blocks) {
    if (num_blocks <= 0 || d < 1 || d > AGL_MAX_D) return GB_EINVAL;
    return agl_dispatch<AglMsg<true>::K>(d, d_polys, d_partial, original_size, half, num_blocks);
}

int agl_sumcheck_fold_ffi(const uint64_t* d_input, uint64_t* d_output, uint64_t challenge, int d,
                          size_t original_size, size_t half) {
    if (d < 1) return GB_EINVAL;
    if (half == 0) return GB_OK;
    agl_fold_kernel<false><<<fold_grid(half), AGL_BLOCK, 0, stream()>>>(d_input, d_output, challenge, 0, d,
                                                                        original_size, half);
    return check_launch("agl_sumcheck_fold_ffi");
}

int aext2_sumcheck_fold_ffi(const uint64_t* d_input, uint64_t* d_output, uint64_t c0, uint64_t c1, int d,
                            size_t original_size, size_t half) {
    if (d < 1) return GB_EINVAL;
    if (half == 0) return GB_OK;
    agl_fold_kernel<true><<<fold_grid(half), AGL_BLOCK, 0, stream()>>>(d_input, d_output, c0, c1, d, original_size,
                                                                       half);
    return check_launch("aext2_sumcheck_fold_ffi");
}

int aext2_sumcheck_batched_round_message_ffi(const uint64_t* d_polys, uint64_t* d_partial, size_t original_size,
                                             size_t half, int num_leaves, int num_blocks_x) {
    if (num_leaves < 0 || num_blocks_x <= 0) return GB_EINVAL;
    if (num_leaves == 0) return GB_OK;
    aext2_batched_msg_kernel<<<dim3(num_blocks_x, num_leaves), AGL_BLOCK, 0, stream()>>>(d_polys, d_partial,
                                                                                         original_size, half,
                                                                                         num_leaves);
    return check_launch("aext2_sumcheck_batched_round_message_ffi");
}

int aext2_sumcheck_batched_fold_ffi(const uint64_t* d_input, uint64_t* d_output, uint64_t c0, uint64_t c1,
                                    size_t original_size, size_t half, int num_leaves) {
    if (num_leaves < 0) return GB_EINVAL;
    if (num_leaves == 0 || half == 0) return GB_OK;
    aext2_batched_fold_kernel<<<dim3(fold_grid(half), num_leaves), AGL_BLOCK, 0, stream()>>>(d_input, d_output, c0,
                                                                                             c1, original_size, half);
    return check_launch("aext2_sumcheck_batched_fold_ffi");
}

int aext2_sumcheck_batched_round0_binary_msg_ffi(const uint64_t* d_polys, const uint64_t* d_packed,
                                                 uint64_t* d_partial, size_t original_size, size_t half,
                                                 int num_leaves, int num_blocks_x, size_t packed_size_u64) {
    if (num_leaves < 0 || num_blocks_x <= 0) return GB_EINVAL;
    if (num_leaves == 0) return GB_OK;
    aext2_round0_binary_msg_kernel<<<dim3(num_blocks_x, num_leaves), AGL_BLOCK, 0, stream()>>>(
        d_polys, d_packed, d_partial, original_size, half, num_leaves, packed_size_u64);
    return check_launch("aext2_sumcheck_batched_round0_binary_msg_ffi");
}

int aext2_sumcheck_batched_round0_binary_fold_ffi(const uint64_t* d_polys, const uint64_t* d_packed,
                                                  uint64_t* d_output, uint64_t c0, uint64_t c1, size_t original_size,
                                                  size_t half, int num_leaves, size_t packed_size_u64) {
    if (num_leaves < 0) return GB_EINVAL;
    if (num_leaves == 0 || half == 0) return GB_OK;
    aext2_round0_binary_fold_kernel<<<dim3(fold_grid(half), num_leaves), AGL_BLOCK, 0, stream()>>>(
        d_polys, d_packed, d_output, c0, c1, original_size, half, packed_size_u64);
    return check_launch("aext2_sumcheck_batched_round0_binary_fold_ffi");
}

int aext2_batched_lift_binary_ffi(const uint64_t* d_packed, uint64_t* d_polys, size_t original_size, int num_leaves,
                                  size_t packed_size_u64) {
    if (num_leaves < 0) return GB_EINVAL;
    if (num_leaves == 0 || original_size == 0) return GB_OK;
    aext2_lift_kernel<<<dim3(fold_grid(original_size), num_leaves), AGL_BLOCK, 0, stream()>>>(
        d_packed, nullptr, d_polys, original_size, packed_size_u64, 4 * original_size, 2 * original_size);
    return check_launch("aext2_batched_lift_binary_ffi");
}

int aext2_batched_lift_ternary_single_ffi(const uint64_t* d_pos, const uint64_t* d_neg, uint64_t* d_polys,
                                          size_t original_size, int num_leaves, size_t packed_size_u64) {
    if (num_leaves < 0 || !d_neg) return GB_EINVAL;
    if (num_leaves == 0 || original_size == 0) return GB_OK;
    aext2_lift_kernel<<<dim3(fold_grid(original_size), num_leaves), AGL_BLOCK, 0, stream()>>>(
        d_pos, d_neg, d_polys, original_size, packed_size_u64, 4 * original_size, 2 * original_size);
    return check_launch("aext2_batched_lift_ternary_single_ffi");
}

int aext2_lift_binary_contig_ffi(const uint64_t* d_packed, uint64_t* d_f, size_t original_size, int num_leaves,
                                 size_t packed_size_u64) {
    if (num_leaves < 0) return GB_EINVAL;
    if (num_leaves == 0 || original_size == 0) return GB_OK;
    aext2_lift_kernel<<<dim3(fold_grid(original_size), num_leaves), AGL_BLOCK, 0, stream()>>>(
        d_packed, nullptr, d_f, original_size, packed_size_u64, 2 * original_size, 0);
    return check_launch("aext2_lift_binary_contig_ffi");
}

int aext2_selective_add_batched_planes_ffi(const uint64_t* d_eq, const uint64_t* d_packed_planes, uint64_t* d_partial,
                                           size_t total, int n_planes, size_t packed_size_u64, int num_blocks_x) {
    if (n_planes < 0 || num_blocks_x <= 0) return GB_EINVAL;
    if (n_planes == 0) return GB_OK;
    aext2_selective_add_kernel<<<dim3(num_blocks_x, n_planes), AGL_BLOCK, 0, stream()>>>(
        d_eq, d_packed_planes, d_partial, total, n_planes, packed_size_u64);
    return check_launch("aext2_selective_add_batched_planes_ffi");
}

// eq tables: like the reference's ping-pong DP, the table ends in d_buf_a when log_n is even
// and in d_buf_b when it is odd (*d_result says which); the other buffer is scratch.
static int agl_eq_entry(bool ext, const uint64_t* d_r, uint64_t* d_buf_a, uint64_t* d_buf_b, int log_n, int leaves,
                        size_t leaf_stride, uint64_t** d_result, cudaStream_t s) {
    if (log_n < 0 || log_n > 40 || !d_r || !d_buf_a || !d_buf_b || !d_result || leaves < 0 ||
        leaf_stride < ((size_t)1 << log_n))
        return GB_EINVAL;
    uint64_t* res = (log_n & 1) ? d_buf_b : d_buf_a;
    uint64_t* scr = (log_n & 1) ? d_buf_a : d_buf_b;
    *d_result = res;
    if (leaves == 0) return GB_OK;
    // an explicit stream (the *_stream / batched entry points) or the thread's launch stream
    cudaStream_t st = s ? s : stream();
    return ext ? agl_eq_tables<true>(d_r, log_n, leaves, leaf_stride, res, scr, st)
               : agl_eq_tables<false>(d_r, log_n, leaves, leaf_stride, res, scr, st);
}

int agl_eq_dp_all_ffi(const uint64_t* d_r, uint64_t* d_buf_a, uint64_t* d_buf_b, int log_n, uint64_t** d_result) {
    return agl_eq_entry(false, d_r, d_buf_a, d_buf_b, log_n, 1, (size_t)1 << log_n, d_result, nullptr);
}

int aext2_eq_dp_all_ffi(const uint64_t* d_r, uint64_t* d_buf_a, uint64_t* d_buf_b, int log_n, uint64_t** d_result) {
    return agl_eq_entry(true, d_r, d_buf_a, d_buf_b, log_n, 1, (size_t)1 << log_n, d_result, nullptr);
}

int aext2_eq_dp_all_stream_ffi(const uint64_t* d_r, uint64_t* d_buf_a, uint64_t* d_buf_b, int log_n,
                               uint64_t** d_result, void* stream_) {
    return agl_eq_entry(true, d_r, d_buf_a, d_buf_b, log_n, 1, (size_t)1 << log_n, d_result, (cudaStream_t)stream_);
}

int aext2_eq_dp_all_batched_ffi(const uint64_t* d_r_all, uint64_t* d_buf_a_all, uint64_t* d_buf_b_all, int log_n,
                                int num_leaves, size_t leaf_stride, uint64_t** d_result, void* stream_) {
    return agl_eq_entry(true, d_r_all, d_buf_a_all, d_buf_b_all, log_n, num_leaves, leaf_stride, d_result,
                        (cudaStream_t)stream_);
}

}  // extern "C"
