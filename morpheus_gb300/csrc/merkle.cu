// Poseidon2 Merkle-tree kernels and the reference Merkle / Poseidon2 entry points
// (goldilocks-cuda-rs/src/ffi.rs:287-300, :549-560; wrapper.cu:864-962, :1604-1714).
//
// One permutation per thread, state in registers.  Large layers get one launch
// each (every warp fully busy); once a layer is small enough its remaining
// levels are finished by a single CTA in one launch, since those levels are a
// latency chain, not a throughput problem.  Nothing here synchronises with the
// host except the reference entry points, which the reference documents as
// synchronising.
#include "../../include/goldilocks_cuda_wrapper.h"
#include "merkle.cuh"

namespace gb {

constexpr int MK_THREADS = 128;
constexpr size_t MK_TOP_NODES = 2048;  // layers at or below this size finish in one CTA

__global__ void __launch_bounds__(MK_THREADS) merkle_level_kernel(const u64* __restrict__ in, u64* __restrict__ out,
                                                                  size_t nodes) {
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= nodes) return;
    u64 s[8];
    ld_digest(in + 8 * j, s);
    ld_digest(in + 8 * j + 4, s + 4);
    p2_permute(s);
    st_digest(out + 4 * j, s);
}

__global__ void __launch_bounds__(MK_THREADS) merkle_level_scalar_kernel(const u64* __restrict__ in,
                                                                         u64* __restrict__ out, size_t nodes) {
    size_t j = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (j >= nodes) return;
    u64 s[8];
#pragma unroll
    for (int k = 0; k < 8; k++) s[k] = in[8 * j + k];
    p2_permute(s);
#pragma unroll
    for (int k = 0; k < 4; k++) out[4 * j + k] = s[k];
}

// Finish all layers from a layer of `nodes` digests at `layer` up to the root.
__global__ void __launch_bounds__(512) merkle_top_kernel(u64* __restrict__ layer, size_t nodes) {
    while (nodes > 1) {
        u64* out = layer + 4 * nodes;
        size_t half = nodes >> 1;
        for (size_t j = threadIdx.x; j < half; j += blockDim.x) {
            u64 s[8];
#pragma unroll
            for (int k = 0; k < 8; k++) s[k] = layer[8 * j + k];
            p2_permute(s);
#pragma unroll
            for (int k = 0; k < 4; k++) out[4 * j + k] = s[k];
        }
        __syncthreads();
        layer = out;
        nodes = half;
    }
}

__global__ void __launch_bounds__(MK_THREADS) hash_leaves_gl_kernel(const u64* __restrict__ cw, u64* __restrict__ tree,
                                                                    size_t leaves) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= leaves) return;
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(cw) + i);
    u64 s[8] = {v.x, v.y, 0, 0, 0, 0, 0, 0};
    p2_permute(s);
    st_digest(tree + 4 * i, s);
}

__global__ void __launch_bounds__(MK_THREADS) hash_leaves_ext2_kernel(const u64* __restrict__ cw, u64* __restrict__ tree,
                                                                      size_t leaves) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= leaves) return;
    u64 s[8];
    ld_digest(cw + 4 * i, s);
    s[4] = s[5] = s[6] = s[7] = 0;
    p2_permute(s);
    st_digest(tree + 4 * i, s);
}

// Copy the first `count` digests of a layer to the following (copies-1) slots.
__global__ void replicate_kernel(u64* __restrict__ layer, size_t count, int copies) {
    size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t words = count * 4;
    if (k >= words * (size_t)(copies - 1)) return;
    layer[words + k] = layer[k % words];
}

int merkle_build_from_leaves(u64* tree, size_t leaves) {
    cudaStream_t s = stream();
    u64* layer = tree;
    size_t nodes = leaves;
    while (nodes > MK_TOP_NODES) {
        size_t half = nodes >> 1;
        merkle_level_kernel<<<grid_for(half, MK_THREADS), MK_THREADS, 0, s>>>(layer, layer + 4 * nodes, half);
        GB_LAUNCH_CHECK("merkle_level_kernel");
        layer += 4 * nodes;
        nodes = half;
    }
    if (nodes > 1) {
        merkle_top_kernel<<<1, 512, 0, s>>>(layer, nodes);
        GB_LAUNCH_CHECK("merkle_top_kernel");
    }
    return GB_OK;
}

int merkle_hash_leaves_gl(const u64* cw, u64* tree, size_t leaves) {
    hash_leaves_gl_kernel<<<grid_for(leaves, MK_THREADS), MK_THREADS, 0, stream()>>>(cw, tree, leaves);
    return check_launch("hash_leaves_gl_kernel");
}

int merkle_hash_leaves_ext2(const u64* cw, u64* tree, size_t leaves) {
    hash_leaves_ext2_kernel<<<grid_for(leaves, MK_THREADS), MK_THREADS, 0, stream()>>>(cw, tree, leaves);
    return check_launch("hash_leaves_ext2_kernel");
}

int merkle_tree_gl_replicated(const u64* cw, u64* tree, size_t leaves, int copies_log) {
    size_t copies = (size_t)1 << copies_log;
    size_t sub = leaves / copies;  // leaves of one copy's subtree
    if (copies_log == 0 || sub < 1 || leaves % copies) {
        int rc = merkle_hash_leaves_gl(cw, tree, leaves);
        return rc ? rc : merkle_build_from_leaves(tree, leaves);
    }
    cudaStream_t s = stream();
    // one copy's subtree: its nodes are the leading entries of every layer
    int rc = merkle_hash_leaves_gl(cw, tree, sub);
    if (rc) return rc;
    size_t off = 0, layer_nodes = leaves, n = sub;
    for (;;) {
        u64* layer = tree + off;
        if (copies > 1) {
            size_t work = n * 4 * (copies - 1);
            replicate_kernel<<<grid_for(work, 256), 256, 0, s>>>(layer, n, (int)copies);
            GB_LAUNCH_CHECK("replicate_kernel");
        }
        if (n == 1) break;
        size_t half = n >> 1;
        merkle_level_kernel<<<grid_for(half, MK_THREADS), MK_THREADS, 0, s>>>(layer, layer + 4 * layer_nodes, half);
        GB_LAUNCH_CHECK("merkle_level_kernel");
        off += 4 * layer_nodes;
        layer_nodes >>= 1;
        n = half;
    }
    // the layer holding the copy roots is complete; finish the top copies_log levels
    return merkle_build_from_leaves(tree + off, layer_nodes);
}

__global__ void permute_batch_kernel(const u64* __restrict__ in, u64* __restrict__ out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u64 s[8];
#pragma unroll
    for (int k = 0; k < 8; k++) s[k] = in[8 * (size_t)i + k];
    p2_permute(s);
#pragma unroll
    for (int k = 0; k < 8; k++) out[8 * (size_t)i + k] = s[k];
}

__global__ void compress_batch_kernel(const u64* __restrict__ l, const u64* __restrict__ r, u64* __restrict__ out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u64 s[8];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        s[k] = l[4 * (size_t)i + k];
        s[4 + k] = r[4 * (size_t)i + k];
    }
    p2_permute(s);
#pragma unroll
    for (int k = 0; k < 4; k++) out[4 * (size_t)i + k] = s[k];
}

}  // namespace gb

using namespace gb;

extern "C" {

int poseidon2_hash_batch_ffi(const uint64_t* d_input, uint64_t* d_output, int n) {
    if (n < 0) return GB_EINVAL;
    if (n == 0) return GB_OK;
    permute_batch_kernel<<<grid_for(n, MK_THREADS), MK_THREADS, 0, stream()>>>(d_input, d_output, n);
    return check_launch("poseidon2_hash_batch_ffi");
}

int poseidon2_compress_batch_ffi(const uint64_t* d_left, const uint64_t* d_right, uint64_t* d_output, int n) {
    if (n < 0) return GB_EINVAL;
    if (n == 0) return GB_OK;
    compress_batch_kernel<<<grid_for(n, MK_THREADS), MK_THREADS, 0, stream()>>>(d_left, d_right, d_output, n);
    return check_launch("poseidon2_compress_batch_ffi");
}

int poseidon2_merkle_layer_ffi(const uint64_t* d_input, uint64_t* d_output, int n) {
    if (n < 0) return GB_EINVAL;
    if (n == 0) return GB_OK;
    if (((uintptr_t)d_input & 15) || ((uintptr_t)d_output & 15)) {
        // a layer sliced at an odd word offset: element-wise loads
        merkle_level_scalar_kernel<<<grid_for(n, MK_THREADS), MK_THREADS, 0, stream()>>>(d_input, d_output, (size_t)n);
        return check_launch("poseidon2_merkle_layer_ffi");
    }
    merkle_level_kernel<<<grid_for(n, MK_THREADS), MK_THREADS, 0, stream()>>>(d_input, d_output, (size_t)n);
    return check_launch("poseidon2_merkle_layer_ffi");
}

int poseidon2_merkle_tree_gl_ffi(const uint64_t* d_codeword, uint64_t* d_tree, int num_leaves) {
    if (num_leaves <= 0 || (num_leaves & (num_leaves - 1))) return GB_EINVAL;
    int rc = merkle_hash_leaves_gl(d_codeword, d_tree, (size_t)num_leaves);
    if (!rc) rc = merkle_build_from_leaves(d_tree, (size_t)num_leaves);
    return rc ? rc : sync_stream("poseidon2_merkle_tree_gl_ffi");
}

int poseidon2_merkle_tree_ext2_ffi(const uint64_t* d_codeword, uint64_t* d_tree, int num_leaves) {
    if (num_leaves <= 0 || (num_leaves & (num_leaves - 1))) return GB_EINVAL;
    int rc = merkle_hash_leaves_ext2(d_codeword, d_tree, (size_t)num_leaves);
    if (!rc) rc = merkle_build_from_leaves(d_tree, (size_t)num_leaves);
    return rc ? rc : sync_stream("poseidon2_merkle_tree_ext2_ffi");
}

}  // extern "C"
