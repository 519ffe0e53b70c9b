// The remaining sumcheck provers of almost-goldilocks-cuda-rs/src/sumcheck_prover.rs used by the
// zk-torch-4 fold tree (ffi.rs:141-160, :319-400; almost_sumcheck_prover.cuh:360-700; almost
// wrapper.cu:931-1028, :2652-2980), over q = 2^64 - 2^32 - 31 and Ext2 = F_q[X]/(X^2 - 3):
//
//   shared-eq state: F_u = sum of alpha_leaf (+- bits) over the leaves of unique point u
//     (aext2_build_fu*), the factored eq suffix tables eqsuf_t[y] = prod_{i >= t} eq1(R_i, y_{i-t})
//     (aext2_eq_suffix_dp), per-round partial sums A = sum eqsuf F[2y], B = sum eqsuf F[2y+1]
//     (aext2_sharedeq_factored_msg), the unfactored message (aext2_sharedeq_msg) and the fold of
//     independent polynomials (aext2_fold_single);
//   aext2_wide_to_ternary: the device split of an i16 witness into k signed bit planes, with an
//     error flag for |v| >= 2^k;
//   sparse boolean check (agl_bool_*): entries (idx, val) grouped by term; a round marks the
//     first entry of each pair {2y, 2y+1}, numbers the marked entries by an exclusive scan, sums
//     the degree-3 message w_t v (v - 1) eq over the pairs at 0, 1, 2, 3 and folds each pair to
//     position y of a compacted array.
//
// Launch shapes (256-thread blocks, grid.y = unique / leaf / term, the caller's grid.x for the
// partial sums) follow the reference, so every per-block partial equals the reference's mod q.
// Outputs are canonical.
#include <algorithm>
#include <vector>

#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "agl.cuh"
#include "common.cuh"

namespace gb {

constexpr int AF_BLOCK = 256;

#define AF_RC(x)            \
    do {                    \
        int _r = (x);       \
        if (_r) return _r;  \
    } while (0)

__device__ __forceinline__ ae2 ld_ae2(const u64* p) { return ae2_make(p[0], p[1]); }
__device__ __forceinline__ void st_ae2(u64* p, ae2 v) {
    v = ae2_canon(v);
    p[0] = v.c0;
    p[1] = v.c1;
}

// block-wide sum of W values per thread into thread 0 (warp shuffles, one shared hop)
template <int W>
__device__ __forceinline__ void af_block_sum(u64 (&acc)[W]) {
    __shared__ u64 sh[(AF_BLOCK / 32) * W];
#pragma unroll
    for (int w = 0; w < W; w++)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc[w] = agl_add(acc[w], __shfl_down_sync(0xffffffffu, acc[w], o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int w = 0; w < W; w++) sh[warp * W + w] = acc[w];
    __syncthreads();
    if (threadIdx.x == 0)
#pragma unroll
        for (int w = 0; w < W; w++) {
            u64 v = sh[w];
            for (int k = 1; k < AF_BLOCK / 32; k++) v = agl_add(v, sh[k * W + w]);
            acc[w] = agl_canon(v);
        }
}

// ---------------------------------------------------------------- shared-eq state
// F_u[x] = sum over the leaves s in [off[u], off[u+1]) of alpha_leaf * (pos bit - neg bit)
__global__ void af_build_fu_kernel(const u64* __restrict__ pos, const u64* __restrict__ neg,
                                   const u64* __restrict__ alphas, const int* __restrict__ leaf_sorted,
                                   const int* __restrict__ off, u64* __restrict__ Fu, size_t n, size_t words) {
    const int u = blockIdx.y, lo = off[u], hi = off[u + 1];
    for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
        const size_t wi = x >> 6;
        const u64 bit = 1ull << (x & 63);
        ae2 acc = ae2_make(0, 0);
        for (int s = lo; s < hi; s++) {
            const int leaf = leaf_sorted[s];
            const size_t o = (size_t)leaf * words + wi;
            const ae2 a = ld_ae2(alphas + 2 * (size_t)leaf);
            if (pos[o] & bit) acc = ae2_add(acc, a);
            if (neg && (neg[o] & bit)) acc = ae2_sub(acc, a);
        }
        st_ae2(Fu + (size_t)u * n * 2 + 2 * x, acc);
    }
}

// eqsuf_t from eqsuf_{t+1}: out[2i + b] = eq1(R_t, b) in[i]  (the new variable is the low bit)
__global__ void af_eq_suffix_layer_kernel(const u64* __restrict__ r_all, u64* __restrict__ eqsuf, int t, int log_n,
                                          size_t in_off, size_t out_off, size_t in_size, size_t stride) {
    const int u = blockIdx.y;
    const ae2 r = ld_ae2(r_all + 2 * ((size_t)u * log_n + t));
    u64* base = eqsuf + (size_t)u * stride;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < in_size; i += (size_t)gridDim.x * blockDim.x) {
        const ae2 a = ld_ae2(base + 2 * (in_off + i));
        const ae2 ar = ae2_mul(a, r);
        st_ae2(base + 2 * (out_off + 2 * i), ae2_sub(a, ar));
        st_ae2(base + 2 * (out_off + 2 * i + 1), ar);
    }
}
__global__ void af_eq_suffix_init_kernel(u64* __restrict__ eqsuf, size_t stride) {
    eqsuf[(size_t)blockIdx.x * stride] = 1;
    eqsuf[(size_t)blockIdx.x * stride + 1] = 0;
}

// partials [block][u][A, B] with A = sum_y eqsuf[y] F[2y], B = sum_y eqsuf[y] F[2y + 1]
__global__ void __launch_bounds__(AF_BLOCK) af_sharedeq_factored_kernel(const u64* __restrict__ eqsuf,
                                                                        const u64* __restrict__ fu,
                                                                        u64* __restrict__ partial, size_t eq_off,
                                                                        size_t eq_stride, size_t poly_stride,
                                                                        size_t half, int num_unique) {
    const int u = blockIdx.y;
    const u64* e = eqsuf + (size_t)u * eq_stride + 2 * eq_off;
    const u64* f = fu + (size_t)u * poly_stride;
    u64 acc[4] = {0, 0, 0, 0};
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        const ae2 ev = ld_ae2(e + 2 * y);
        const ae2 a = ae2_mul(ev, ld_ae2(f + 4 * y)), b = ae2_mul(ev, ld_ae2(f + 4 * y + 2));
        acc[0] = agl_add(acc[0], a.c0);
        acc[1] = agl_add(acc[1], a.c1);
        acc[2] = agl_add(acc[2], b.c0);
        acc[3] = agl_add(acc[3], b.c1);
    }
    af_block_sum<4>(acc);
    if (threadIdx.x == 0) {
        u64* o = partial + ((size_t)blockIdx.x * num_unique + u) * 4;
#pragma unroll
        for (int w = 0; w < 4; w++) o[w] = acc[w];
    }
}

// partials [block][leaf][c][2]: c = 0: e0 f0, 1: e1 f1, 2: (2 e1 - e0)(2 f1 - f0), eq of the leaf's unique
__global__ void __launch_bounds__(AF_BLOCK) af_sharedeq_msg_kernel(const u64* __restrict__ eq, const u64* __restrict__ f,
                                                                   const int* __restrict__ leaf_to_unique,
                                                                   u64* __restrict__ partial, size_t n, size_t half,
                                                                   int num_leaves) {
    const int leaf = blockIdx.y;
    const u64* ep = eq + (size_t)leaf_to_unique[leaf] * n * 2;
    const u64* fp = f + (size_t)leaf * n * 2;
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        const ae2 e0 = ld_ae2(ep + 4 * y), e1 = ld_ae2(ep + 4 * y + 2);
        const ae2 f0 = ld_ae2(fp + 4 * y), f1 = ld_ae2(fp + 4 * y + 2);
        const ae2 p0 = ae2_mul(e0, f0), p1 = ae2_mul(e1, f1);
        const ae2 p2 = ae2_mul(ae2_sub(ae2_add(e1, e1), e0), ae2_sub(ae2_add(f1, f1), f0));
        acc[0] = agl_add(acc[0], p0.c0);
        acc[1] = agl_add(acc[1], p0.c1);
        acc[2] = agl_add(acc[2], p1.c0);
        acc[3] = agl_add(acc[3], p1.c1);
        acc[4] = agl_add(acc[4], p2.c0);
        acc[5] = agl_add(acc[5], p2.c1);
    }
    af_block_sum<6>(acc);
    if (threadIdx.x == 0) {
        u64* o = partial + ((size_t)blockIdx.x * num_leaves + leaf) * 6;
#pragma unroll
        for (int w = 0; w < 6; w++) o[w] = acc[w];
    }
}

__global__ void af_fold_single_kernel(const u64* __restrict__ in, u64* __restrict__ out, u64 r0, u64 r1, size_t n,
                                      size_t half) {
    const int p = blockIdx.y;
    const u64* ip = in + (size_t)p * n * 2;
    u64* op = out + (size_t)p * n * 2;
    const ae2 r = ae2_make(r0, r1);
    for (size_t y = blockIdx.x * (size_t)blockDim.x + threadIdx.x; y < half; y += (size_t)gridDim.x * blockDim.x) {
        const ae2 a = ld_ae2(ip + 4 * y), b = ld_ae2(ip + 4 * y + 2);
        st_ae2(op + 2 * y, ae2_add(a, ae2_mul(r, ae2_sub(b, a))));
    }
}

// i16 witness -> k signed bit planes (warp per ring element, two ballots per plane and sign);
// any |v| >= 2^k sets *err
__global__ void af_wide_to_ternary_kernel(const int16_t* __restrict__ z, u64* __restrict__ pos, u64* __restrict__ neg,
                                          int* __restrict__ err, size_t N, int k) {
    const int lane = threadIdx.x & 31;
    const size_t w0 = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5, nw = ((size_t)gridDim.x * blockDim.x) >> 5;
    for (size_t j = w0; j < N; j += nw) {
        const int a = z[j * 64 + lane], b = z[j * 64 + 32 + lane];
        const int aa = a < 0 ? -a : a, bb = b < 0 ? -b : b;
        if (err && ((aa >> k) || (bb >> k))) atomicExch(err, 1);
        u64 mine = 0;
        for (int i = 0; i < k; i++) {
            const unsigned pa = __ballot_sync(0xffffffffu, a > 0 && ((aa >> i) & 1));
            const unsigned pb = __ballot_sync(0xffffffffu, b > 0 && ((bb >> i) & 1));
            const unsigned na = __ballot_sync(0xffffffffu, a < 0 && ((aa >> i) & 1));
            const unsigned nb = __ballot_sync(0xffffffffu, b < 0 && ((bb >> i) & 1));
            if (lane == i) mine = (u64)pa | ((u64)pb << 32);
            if (lane == 16 + i) mine = (u64)na | ((u64)nb << 32);
        }
        if (lane < k) pos[(size_t)lane * N + j] = mine;
        else if (lane >= 16 && lane < 16 + k) neg[(size_t)(lane - 16) * N + j] = mine;
    }
}

// ---------------------------------------------------------------- sparse boolean check
// flags[i] = 1 for the first entry of each pair {2y, 2y + 1} present in its term
__global__ void af_bool_mark_kernel(const uint32_t* __restrict__ idx, const uint32_t* __restrict__ term_off,
                                    uint32_t* __restrict__ flags) {
    const int t = blockIdx.y;
    const size_t s = term_off[t], e = term_off[t + 1];
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < e - s; k += (size_t)gridDim.x * blockDim.x) {
        const size_t i = s + k;
        flags[i] = (k == 0 || !((idx[i] & 1u) && idx[i - 1] == idx[i] - 1u)) ? 1u : 0u;
    }
}

// the pair (v0, v1) of the marked entry i
__device__ __forceinline__ void af_bool_pair(const uint32_t* idx, const u64* val, size_t i, size_t e, uint32_t& rest,
                                             ae2& v0, ae2& v1) {
    const uint32_t pos = idx[i];
    rest = pos >> 1;
    v0 = v1 = ae2_make(0, 0);
    if (!(pos & 1u)) {
        v0 = ld_ae2(val + 2 * i);
        if (i + 1 < e && idx[i + 1] == 2u * rest + 1u) v1 = ld_ae2(val + 2 * (i + 1));
    } else {
        v1 = ld_ae2(val + 2 * i);
    }
}

// partial[(t * grid_x + b) * 8 ..]: the message w_t v (v - 1) eq at 0, 1, 2, 3
__global__ void __launch_bounds__(AF_BLOCK) af_bool_msg_kernel(const uint32_t* __restrict__ idx, const u64* __restrict__ val,
                                                               const uint32_t* __restrict__ flags,
                                                               const uint32_t* __restrict__ term_off,
                                                               const u64* __restrict__ w, const u64* __restrict__ eq,
                                                               u64* __restrict__ partial) {
    const int t = blockIdx.y;
    const size_t s = term_off[t], e = term_off[t + 1];
    const ae2 wt = ld_ae2(w + 2 * t), one = ae2_make(1, 0);
    u64 acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < e - s; k += (size_t)gridDim.x * blockDim.x) {
        const size_t i = s + k;
        if (!flags[i]) continue;
        uint32_t rest;
        ae2 v0, v1;
        af_bool_pair(idx, val, i, e, rest, v0, v1);
        const ae2 q0 = ld_ae2(eq + 4 * (size_t)rest), q1 = ld_ae2(eq + 4 * (size_t)rest + 2);
        const ae2 dv = ae2_sub(v1, v0), dq = ae2_sub(q1, q0);
        ae2 v = v0, q = q0;
#pragma unroll
        for (int c = 0; c < 4; c++) {  // points 0, 1, 2, 3: v = v0 + c dv, q = q0 + c dq
            const ae2 term = ae2_mul(ae2_mul(wt, ae2_mul(v, ae2_sub(v, one))), q);
            acc[2 * c] = agl_add(acc[2 * c], term.c0);
            acc[2 * c + 1] = agl_add(acc[2 * c + 1], term.c1);
            v = ae2_add(v, dv);
            q = ae2_add(q, dq);
        }
    }
    af_block_sum<8>(acc);
    if (threadIdx.x == 0) {
        u64* o = partial + ((size_t)blockIdx.y * gridDim.x + blockIdx.x) * 8;
#pragma unroll
        for (int k = 0; k < 8; k++) o[k] = acc[k];
    }
}

__global__ void af_bool_fold_kernel(const uint32_t* __restrict__ idx, const u64* __restrict__ val,
                                    const uint32_t* __restrict__ flags, const uint32_t* __restrict__ gid,
                                    const uint32_t* __restrict__ term_off, u64 r0, u64 r1,
                                    uint32_t* __restrict__ out_idx, u64* __restrict__ out_val) {
    const int t = blockIdx.y;
    const size_t s = term_off[t], e = term_off[t + 1];
    const ae2 r = ae2_make(r0, r1);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < e - s; k += (size_t)gridDim.x * blockDim.x) {
        const size_t i = s + k;
        if (!flags[i]) continue;
        uint32_t rest;
        ae2 v0, v1;
        af_bool_pair(idx, val, i, e, rest, v0, v1);
        const uint32_t g = gid[i];
        out_idx[g] = rest;
        st_ae2(out_val + 2 * (size_t)g, ae2_add(v0, ae2_mul(r, ae2_sub(v1, v0))));
    }
}

__global__ void af_bool_newoff_kernel(const uint32_t* __restrict__ gid, const uint32_t* __restrict__ term_off,
                                      int n_terms, size_t n, uint32_t total, uint32_t* __restrict__ new_off) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t > n_terms) return;
    const size_t s = term_off[t];
    new_off[t] = (t == n_terms || s >= n) ? total : gid[s];
}

__global__ void af_bool_finish_kernel(const uint32_t* __restrict__ idx, const u64* __restrict__ val,
                                      const uint32_t* __restrict__ term_off, int n_terms, size_t n,
                                      u64* __restrict__ out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_terms) return;
    const size_t s = term_off[t], e = term_off[t + 1];
    u64 c0 = 0, c1 = 0;
    if (s < e && s < n && idx[s] == 0u) {
        c0 = agl_canon(val[2 * s]);
        c1 = agl_canon(val[2 * s + 1]);
    }
    out[2 * t] = c0;
    out[2 * t + 1] = c1;
}

__global__ void af_bool_init_kernel(u64* __restrict__ val, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        val[2 * i] = 1;
        val[2 * i + 1] = 0;
    }
}

// exclusive scan of n u32 values: per-block scans (warp shuffles), the block totals scanned
// recursively in the caller's scratch, then each block's offset added
__global__ void __launch_bounds__(AF_BLOCK) af_scan_block_kernel(const uint32_t* __restrict__ in, uint32_t* __restrict__ out,
                                                                 uint32_t* __restrict__ block_sums, size_t n) {
    __shared__ uint32_t wsum[AF_BLOCK / 32];
    const size_t i = blockIdx.x * (size_t)AF_BLOCK + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t s = lane < AF_BLOCK / 32 ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < AF_BLOCK / 32) wsum[lane] = s;
    }
    __syncthreads();
    const uint32_t incl = x + (warp ? wsum[warp - 1] : 0);
    if (i < n) out[i] = incl - v;
    if (threadIdx.x == AF_BLOCK - 1) block_sums[blockIdx.x] = incl;
}
__global__ void af_scan_add_kernel(uint32_t* __restrict__ out, const uint32_t* __restrict__ offs, size_t n) {
    const size_t i = blockIdx.x * (size_t)AF_BLOCK + threadIdx.x;
    if (i < n) out[i] += offs[blockIdx.x];
}
static int af_exscan(const uint32_t* in, uint32_t* out, size_t n, uint32_t* scratch, size_t scratch_len, cudaStream_t s) {
    const size_t nb = (n + AF_BLOCK - 1) / AF_BLOCK;
    if (nb > scratch_len) return GB_EINVAL;
    af_scan_block_kernel<<<(unsigned)nb, AF_BLOCK, 0, s>>>(in, out, scratch, n);
    GB_LAUNCH_CHECK("af_scan_block_kernel");
    if (nb > 1) {
        uint32_t* rest = scratch + nb;
        if (scratch_len - nb < 2 * nb) return GB_EINVAL;
        AF_RC(af_exscan(scratch, rest, nb, rest + nb, scratch_len - 2 * nb, s));
        af_scan_add_kernel<<<(unsigned)nb, AF_BLOCK, 0, s>>>(out, rest, n);
        GB_LAUNCH_CHECK("af_scan_add_kernel");
    }
    return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

int aext2_build_fu_ffi(const uint64_t* d_packed, const uint64_t* d_alphas, const int* d_leaf_idx_sorted,
                       const int* d_unique_offsets, uint64_t* d_Fu, size_t original_size, int num_unique,
                       size_t packed_size_u64) {
    if (num_unique < 0) return GB_EINVAL;
    if (!num_unique || !original_size) return GB_OK;
    af_build_fu_kernel<<<dim3(grid_for(original_size, AF_BLOCK), num_unique), AF_BLOCK, 0, stream()>>>(
        d_packed, nullptr, d_alphas, d_leaf_idx_sorted, d_unique_offsets, d_Fu, original_size, packed_size_u64);
    return check_launch("aext2_build_fu_ffi");
}

int aext2_build_fu_ternary_ffi(const uint64_t* d_pos, const uint64_t* d_neg, const uint64_t* d_alphas,
                               const int* d_leaf_idx_sorted, const int* d_unique_offsets, uint64_t* d_Fu,
                               size_t original_size, int num_unique, size_t packed_size_u64) {
    if (num_unique < 0 || !d_neg) return GB_EINVAL;
    if (!num_unique || !original_size) return GB_OK;
    af_build_fu_kernel<<<dim3(grid_for(original_size, AF_BLOCK), num_unique), AF_BLOCK, 0, stream()>>>(
        d_pos, d_neg, d_alphas, d_leaf_idx_sorted, d_unique_offsets, d_Fu, original_size, packed_size_u64);
    return check_launch("aext2_build_fu_ternary_ffi");
}

int aext2_wide_to_ternary_ffi(const int16_t* d_wide, uint64_t* d_pos, uint64_t* d_neg, int* d_err, size_t n_ring,
                              int k_chunks) {
    if (k_chunks > 16 || k_chunks < 0) return GB_ECUDA;  // the reference returns -1 above 16 planes
    if (!n_ring) return GB_OK;
    const unsigned g = (unsigned)std::min<size_t>((n_ring + 7) / 8, (size_t)num_sms() * 16);
    af_wide_to_ternary_kernel<<<g, AF_BLOCK, 0, stream()>>>(d_wide, d_pos, d_neg, d_err, n_ring, k_chunks);
    return check_launch("aext2_wide_to_ternary_ffi");
}

int aext2_eq_suffix_dp_ffi(const uint64_t* d_r_all, uint64_t* d_eqsuf, int log_n, int num_unique,
                           size_t eqsuf_stride_u64) {
    if (num_unique < 0 || log_n < 0) return GB_EINVAL;
    if (!num_unique) return GB_OK;
    cudaStream_t s = stream();
    af_eq_suffix_init_kernel<<<num_unique, 1, 0, s>>>(d_eqsuf, eqsuf_stride_u64);
    GB_LAUNCH_CHECK("af_eq_suffix_init_kernel");
    for (int t = log_n - 1; t >= 1; t--) {
        const size_t in_size = (size_t)1 << (log_n - t - 1);
        af_eq_suffix_layer_kernel<<<dim3(grid_for(in_size, AF_BLOCK), num_unique), AF_BLOCK, 0, s>>>(
            d_r_all, d_eqsuf, t, log_n, in_size - 1, ((size_t)1 << (log_n - t)) - 1, in_size, eqsuf_stride_u64);
        GB_LAUNCH_CHECK("af_eq_suffix_layer_kernel");
    }
    return GB_OK;
}

int aext2_sharedeq_factored_msg_ffi(const uint64_t* d_eqsuf, const uint64_t* d_fu, uint64_t* d_partial,
                                    size_t eqsuf_off_elems, size_t eqsuf_stride_u64, size_t poly_stride_u64,
                                    size_t half, int num_unique, int num_blocks_x) {
    if (num_unique < 0 || num_blocks_x <= 0) return GB_EINVAL;
    if (!num_unique) return GB_OK;
    af_sharedeq_factored_kernel<<<dim3(num_blocks_x, num_unique), AF_BLOCK, 0, stream()>>>(
        d_eqsuf, d_fu, d_partial, eqsuf_off_elems, eqsuf_stride_u64, poly_stride_u64, half, num_unique);
    return check_launch("aext2_sharedeq_factored_msg_ffi");
}

int aext2_sharedeq_msg_ffi(const uint64_t* d_eq, const uint64_t* d_f, const int* d_leaf_to_unique,
                           uint64_t* d_partial, size_t original_size, size_t half, int num_leaves, int num_blocks_x) {
    if (num_leaves < 0 || num_blocks_x <= 0) return GB_EINVAL;
    if (!num_leaves) return GB_OK;
    af_sharedeq_msg_kernel<<<dim3(num_blocks_x, num_leaves), AF_BLOCK, 0, stream()>>>(
        d_eq, d_f, d_leaf_to_unique, d_partial, original_size, half, num_leaves);
    return check_launch("aext2_sharedeq_msg_ffi");
}

int aext2_fold_single_ffi(const uint64_t* d_in, uint64_t* d_out, uint64_t c0, uint64_t c1, size_t original_size,
                          size_t half, int count) {
    if (count < 0) return GB_EINVAL;
    if (!count || !half) return GB_OK;
    af_fold_single_kernel<<<dim3(grid_for(half, AF_BLOCK), count), AF_BLOCK, 0, stream()>>>(d_in, d_out, c0, c1,
                                                                                             original_size, half);
    return check_launch("aext2_fold_single_ffi");
}

int agl_bool_init_val_ffi(uint64_t* d_val, size_t n) {
    if (!n) return GB_OK;
    cudaStream_t s = stream();
    af_bool_init_kernel<<<grid_for(n, AF_BLOCK), AF_BLOCK, 0, s>>>(d_val, n);
    GB_LAUNCH_CHECK("af_bool_init_kernel");
    return sync_stream("agl_bool_init_val_ffi");
}

int agl_bool_finish_ffi(const uint32_t* d_idx, const uint64_t* d_val, const uint32_t* d_term_off, int n_terms, size_t n,
                        uint64_t* d_out) {
    if (n_terms <= 0) return GB_OK;
    cudaStream_t s = stream();
    af_bool_finish_kernel<<<(n_terms + 255) / 256, 256, 0, s>>>(d_idx, d_val, d_term_off, n_terms, n, d_out);
    GB_LAUNCH_CHECK("af_bool_finish_kernel");
    return sync_stream("agl_bool_finish_ffi");
}

int agl_bool_round_msg_ffi(const uint32_t* d_idx, const uint64_t* d_val, const uint32_t* d_term_off, const uint64_t* d_w,
                           const uint64_t* d_eq, int n_terms, size_t n, uint32_t* d_flags, uint32_t* d_gid,
                           uint64_t* d_partial, int grid_x, uint32_t* d_scan_scratch, size_t scan_scratch_len,
                           uint64_t* h_msg, uint32_t* h_total) {
    if (!h_msg || !h_total) return GB_EINVAL;
    if (n == 0) {
        for (int k = 0; k < 8; k++) h_msg[k] = 0;
        *h_total = 0;
        return GB_OK;
    }
    if (n_terms <= 0 || grid_x <= 0) return GB_EINVAL;
    cudaStream_t s = stream();
    const dim3 g(grid_x, n_terms);
    af_bool_mark_kernel<<<g, AF_BLOCK, 0, s>>>(d_idx, d_term_off, d_flags);
    GB_LAUNCH_CHECK("af_bool_mark_kernel");
    AF_RC(af_exscan(d_flags, d_gid, n, d_scan_scratch, scan_scratch_len, s));
    af_bool_msg_kernel<<<g, AF_BLOCK, 0, s>>>(d_idx, d_val, d_flags, d_term_off, d_w, d_eq, d_partial);
    GB_LAUNCH_CHECK("af_bool_msg_kernel");
    const size_t mb = (size_t)grid_x * n_terms;
    std::vector<u64> h(mb * 8);
    uint32_t last[2];
    GB_CUDA_TRY(cudaMemcpyAsync(&last[0], d_gid + (n - 1), 4, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaMemcpyAsync(&last[1], d_flags + (n - 1), 4, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaMemcpyAsync(h.data(), d_partial, mb * 64, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    *h_total = last[0] + last[1];
    unsigned __int128 acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (size_t b = 0; b < mb; b++)
        for (int k = 0; k < 8; k++) acc[k] += h[b * 8 + k];
    for (int k = 0; k < 8; k++) h_msg[k] = (u64)(acc[k] % AGL_Q);
    return GB_OK;
}

int agl_bool_fold_ffi(const uint32_t* d_idx, const uint64_t* d_val, const uint32_t* d_flags, const uint32_t* d_gid,
                      const uint32_t* d_term_off, int n_terms, size_t n, uint64_t r0, uint64_t r1, uint32_t total,
                      int grid_x, uint32_t* d_out_idx, uint64_t* d_out_val, uint32_t* d_new_off) {
    if (n == 0) return GB_OK;
    if (n_terms <= 0 || grid_x <= 0) return GB_EINVAL;
    cudaStream_t s = stream();
    af_bool_fold_kernel<<<dim3(grid_x, n_terms), AF_BLOCK, 0, s>>>(d_idx, d_val, d_flags, d_gid, d_term_off, r0, r1,
                                                                   d_out_idx, d_out_val);
    GB_LAUNCH_CHECK("af_bool_fold_kernel");
    af_bool_newoff_kernel<<<(n_terms + 1 + 255) / 256, 256, 0, s>>>(d_gid, d_term_off, n_terms, n, total, d_new_off);
    GB_LAUNCH_CHECK("af_bool_newoff_kernel");
    return sync_stream("agl_bool_fold_ffi");
}

}  // extern "C"
