// eq(r, x) = prod_i (r_i x_i + (1 - r_i)(1 - x_i)) over {0,1}^n, variable i <-> bit i
// of x (zk-torch-3/src/poly/mod.rs:106-161; cuda/eq_lagrange.cuh:22-158).
//
// Two small tables -- eq over the low k variables and eq over the high n-k -- are
// built by one CTA (a doubling loop in global memory, at most 2^12 entries each),
// then every output entry is one product lo[x & mask] * hi[x >> k].  The 2^n
// table is therefore written once instead of once per variable as in a
// layer-by-layer expansion.
#include "../../include/goldilocks_cuda_wrapper.h"
#include "basefold.cuh"

namespace gb {

// eq over variables [v0, v1) into out (2^(v1-v0) entries), one CTA.
template <bool EXT>
__global__ void eq_small_table_kernel(const u64* __restrict__ r, int v0, int v1, u64* __restrict__ out) {
    if (threadIdx.x == 0) {
        out[0] = 1;
        if (EXT) out[1] = 0;
    }
    __syncthreads();
    for (int v = v0; v < v1; v++) {
        size_t half = (size_t)1 << (v - v0);
        for (size_t j = threadIdx.x; j < half; j += blockDim.x) {
            if (EXT) {
                e2 a = e2_make(out[2 * j], out[2 * j + 1]);
                e2 ar = e2_mul(a, e2_make(r[2 * v], r[2 * v + 1]));
                e2 lo_v = e2_sub(a, ar);
                out[2 * (j + half)] = ar.c0;
                out[2 * (j + half) + 1] = ar.c1;
                out[2 * j] = lo_v.c0;
                out[2 * j + 1] = lo_v.c1;
            } else {
                u64 a = out[j];
                u64 ar = gl_mul(a, r[v]);
                out[j + half] = ar;
                out[j] = gl_sub(a, ar);
            }
        }
        __syncthreads();
    }
}

template <bool EXT>
__global__ void eq_expand_kernel(const u64* __restrict__ lo, const u64* __restrict__ hi, int k, size_t total,
                                 u64* __restrict__ out) {
    size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (x >= total) return;
    size_t xl = x & (((size_t)1 << k) - 1), xh = x >> k;
    if (EXT) {
        e2 v = e2_mul(e2_ld(lo + 2 * xl), e2_ld(hi + 2 * xh));
        e2_st(out + 2 * x, v);
    } else {
        out[x] = gl_mul(__ldg(lo + xl), __ldg(hi + xh));
    }
}

int eq_table(const u64* d_r, int n, bool ext, u64* d_out) {
    cudaStream_t s = stream();
    const int w = ext ? 2 : 1;
    if (n <= 12) {
        // small: the doubling loop directly in the output buffer (2^n entries)
        if (ext) eq_small_table_kernel<true><<<1, 256, 0, s>>>(d_r, 0, n, d_out);
        else eq_small_table_kernel<false><<<1, 256, 0, s>>>(d_r, 0, n, d_out);
        return check_launch("eq_small_table_kernel");
    }
    int k = n / 2;
    u64* tabs = nullptr;
    size_t lo_words = (size_t)w << k, hi_words = (size_t)w << (n - k);
    GB_CUDA_TRY(cudaMallocAsync(&tabs, (lo_words + hi_words) * 8, s));
    if (ext) {
        eq_small_table_kernel<true><<<1, 512, 0, s>>>(d_r, 0, k, tabs);
        eq_small_table_kernel<true><<<1, 512, 0, s>>>(d_r, k, n, tabs + lo_words);
    } else {
        eq_small_table_kernel<false><<<1, 512, 0, s>>>(d_r, 0, k, tabs);
        eq_small_table_kernel<false><<<1, 512, 0, s>>>(d_r, k, n, tabs + lo_words);
    }
    GB_LAUNCH_CHECK("eq_small_table_kernel");
    size_t total = (size_t)1 << n;
    if (ext) eq_expand_kernel<true><<<grid_for(total, 256), 256, 0, s>>>(tabs, tabs + lo_words, k, total, d_out);
    else eq_expand_kernel<false><<<grid_for(total, 256), 256, 0, s>>>(tabs, tabs + lo_words, k, total, d_out);
    GB_LAUNCH_CHECK("eq_expand_kernel");
    GB_CUDA_TRY(cudaFreeAsync(tabs, s));
    return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" {

// The reference ping-pongs one layer per variable starting in d_buf_a, so its result
// sits in d_buf_a for even log_n and in d_buf_b for odd log_n; the same buffer is
// chosen here so callers that look at *d_result or at the buffer see the same thing.
int eq_dp_all_ffi(const uint64_t* d_r, uint64_t* d_buf_a, uint64_t* d_buf_b, int log_n, uint64_t** d_result) {
    if (log_n < 0 || log_n > 40) return GB_EINVAL;
    uint64_t* out = (log_n & 1) ? d_buf_b : d_buf_a;
    int rc = eq_table(d_r, log_n, false, out);
    if (rc) return rc;
    if (d_result) *d_result = out;
    return GB_OK;
}

int ext2_eq_dp_all_ffi(const uint64_t* d_r, uint64_t* d_buf_a, uint64_t* d_buf_b, int log_n, uint64_t** d_result) {
    if (log_n < 0 || log_n > 40) return GB_EINVAL;
    uint64_t* out = (log_n & 1) ? d_buf_b : d_buf_a;
    int rc = eq_table(d_r, log_n, true, out);
    if (rc) return rc;
    if (d_result) *d_result = out;
    return GB_OK;
}

}  // extern "C"
