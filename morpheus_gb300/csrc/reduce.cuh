// Block- and grid-level reductions of W field elements per thread.
//
// Each block reduces with warp shuffles and one shared-memory hop; the grid
// finishes in the last block to arrive (a ticket counter in global memory,
// reset by that block), so a whole round message is produced by one launch.
#pragma once
#include "gl.cuh"

namespace gb {

constexpr int RED_THREADS = 256;
constexpr int RED_WARPS = RED_THREADS / 32;

// Reduce acc[W] over the block.  Result valid in thread 0 (returned in acc).
template <int W>
__device__ __forceinline__ void block_reduce(u64 (&acc)[W]) {
    __shared__ u64 sm[RED_WARPS][W];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = gl_warp_sum(acc[w]);
    if (lane == 0) {
#pragma unroll
        for (int w = 0; w < W; w++) sm[warp][w] = acc[w];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int w = 0; w < W; w++) {
            u64 v = (lane < (int)(blockDim.x >> 5)) ? sm[lane][w] : 0;
            acc[w] = gl_warp_sum(v);
        }
    }
    __syncthreads();
}

// Per-block partials to partials[blockIdx.x * W + w]; the last block sums all of
// them and writes the canonical total to out[w], then re-arms the counter.
// bid / nblocks: this block's index among the nblocks blocks that share the reduction.
template <int W>
__device__ __forceinline__ void grid_reduce_finish_n(u64 (&acc)[W], u64* __restrict__ partials, u64* __restrict__ out,
                                                     unsigned* __restrict__ counter, unsigned bid, unsigned nblocks) {
    __shared__ bool s_last;
    block_reduce<W>(acc);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < W; w++) partials[(size_t)bid * W + w] = acc[w];
        __threadfence();
        unsigned t = atomicAdd(counter, 1u);
        s_last = (t == nblocks - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    u64 tot[W];
#pragma unroll
    for (int w = 0; w < W; w++) tot[w] = 0;
    for (unsigned b = threadIdx.x; b < nblocks; b += blockDim.x) {
#pragma unroll
        for (int w = 0; w < W; w++) tot[w] = gl_add(tot[w], __ldcg(reinterpret_cast<const unsigned long long*>(partials) + (size_t)b * W + w));
    }
    block_reduce<W>(tot);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < W; w++) out[w] = gl_canon(tot[w]);
        *counter = 0;
    }
}
template <int W>
__device__ __forceinline__ void grid_reduce_finish(u64 (&acc)[W], u64* __restrict__ partials, u64* __restrict__ out,
                                                   unsigned* __restrict__ counter) {
    grid_reduce_finish_n<W>(acc, partials, out, counter, blockIdx.x, gridDim.x);
}

// Per-block partials only (the reference ABI leaves the final sum to the caller).
template <int W>
__device__ __forceinline__ void block_partials(u64 (&acc)[W], u64* __restrict__ partials) {
    block_reduce<W>(acc);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 0; w < W; w++) partials[(size_t)blockIdx.x * W + w] = acc[w];
    }
}

}  // namespace gb
