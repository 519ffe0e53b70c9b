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
constexpr int MK_COOP_THREADS = 256;

template <int T>
__global__ void P2_BOUNDS(T) merkle_level_kernel(const u64* __restrict__ in, u64* __restrict__ out, size_t nodes) {
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

// One parent per lane pair (p2_permute_pair): lane h loads child 2j + h.  Pairs past the end
// compute parent 0 and store nothing: their warp still takes part in the exchanges.
template <int T>
__global__ void P2_PAIR_BOUNDS(T) merkle_level_pair_kernel(const u64* __restrict__ in, u64* __restrict__ out,
                                                           size_t nodes) {
    const size_t j = (blockIdx.x * (size_t)T + threadIdx.x) >> 1;
    const int h = threadIdx.x & 1;
    const bool live = j < nodes;
    u64 s[4];
    ld_digest(in + 8 * (live ? j : 0) + 4 * h, s);
    p2_permute_pair(s, h);
    if (live && h == 0) st_digest(out + 4 * j, s);
}

// One parent per 8-lane group.  Groups past the end compute node 0 and store nothing:
// their warp still has to take part in the shuffles.
__global__ void __launch_bounds__(MK_COOP_THREADS) merkle_level_coop_kernel(const u64* __restrict__ in,
                                                                          u64* __restrict__ out, size_t nodes) {
    pdl_enter();
    size_t g = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 3;
    int l = threadIdx.x & 7;
    bool live = g < nodes;
    size_t gg = live ? g : 0;
    P2Lane c = p2_lane_consts(l);
    u64 x = p2_permute_coop(in[8 * gg + l], l, c);
    if (live && l < 4) out[4 * g + l] = x;
}

// Finish all layers from a small layer up to the root in one CTA: 8-lane groups take the
// parents of a layer in turns (every warp runs the same number of turns, since the
// permutation's shuffles need all 32 lanes), then the CTA moves up a layer.  The root is also
// written to root_out when given.
__global__ void __launch_bounds__(1024) merkle_top_coop_kernel(u64* __restrict__ layer, size_t nodes,
                                                               u64* __restrict__ root_out) {
    pdl_enter();
    const int groups = blockDim.x >> 3, grp = threadIdx.x >> 3, l = threadIdx.x & 7;
    P2Lane c = p2_lane_consts(l);
    while (nodes > 1) {
        size_t half = nodes >> 1;
        u64* out = layer + 4 * nodes;
        for (size_t base = 0; base < half; base += groups) {
            size_t p = base + grp;
            bool live = p < half;
            u64 x = p2_permute_coop(layer[8 * (live ? p : 0) + l], l, c);
            if (live && l < 4) out[4 * p + l] = x;
        }
        __syncthreads();
        layer = out;
        nodes = half;
    }
    if (root_out && threadIdx.x < 4) root_out[threadIdx.x] = layer[threadIdx.x];
}

// Copies of the first copy's subtree: on layer k (2^(levels-k) * copies nodes, offsets as in
// the full tree) the first sub >> k digests are repeated copies - 1 times.  One thread per
// copied word, all layers in one launch.
__global__ void replicate_layers_kernel(u64* __restrict__ tree, size_t leaves, size_t sub, int copies, size_t total) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= total) return;
    size_t off = 0, nodes = leaves, n = sub;
    for (;;) {
        size_t words = 4 * n * (size_t)(copies - 1);
        if (t < words) {
            u64* layer = tree + off;
            layer[4 * n + t] = layer[t % (4 * n)];
            return;
        }
        t -= words;
        off += 4 * nodes;
        nodes >>= 1;
        n >>= 1;
        if (n == 0) return;
    }
}

// Leaf hashes in the pair form: lane 0 of a pair holds the leaf's `width` (2 or 4) elements,
// lane 1 the zero half of the state.
template <int T>
__global__ void P2_PAIR_BOUNDS(T) hash_leaves_pair_kernel(const u64* __restrict__ cw, u64* __restrict__ tree,
                                                          size_t leaves, int width) {
    const size_t i = (blockIdx.x * (size_t)T + threadIdx.x) >> 1;
    const int h = threadIdx.x & 1;
    const bool live = i < leaves;
    u64 s[4] = {0, 0, 0, 0};
    if (h == 0) {
        const ulonglong2* p = reinterpret_cast<const ulonglong2*>(cw + (size_t)width * (live ? i : 0));
        ulonglong2 v = __ldg(p);
        s[0] = v.x;
        s[1] = v.y;
        if (width == 4) {
            v = __ldg(p + 1);
            s[2] = v.x;
            s[3] = v.y;
        }
    }
    p2_permute_pair(s, h);
    if (live && h == 0) st_digest(tree + 4 * i, s);
}

__global__ void __launch_bounds__(MK_COOP_THREADS) hash_leaves_coop_kernel(const u64* __restrict__ cw,
                                                                         u64* __restrict__ tree, size_t leaves,
                                                                         int width) {
    pdl_enter();
    size_t g = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 3;
    int l = threadIdx.x & 7;
    bool live = g < leaves;
    size_t gg = live ? g : 0;
    P2Lane c = p2_lane_consts(l);
    u64 x = l < width ? cw[(size_t)width * gg + l] : 0;
    x = p2_permute_coop(x, l, c);
    if (live && l < 4) tree[4 * g + l] = x;
}

template <int T>
__global__ void P2_BOUNDS(T) hash_leaves_gl_kernel(const u64* __restrict__ cw, u64* __restrict__ tree, size_t leaves) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= leaves) return;
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(cw) + i);
    u64 s[8] = {v.x, v.y, 0, 0, 0, 0, 0, 0};
    p2_permute<2>(s);
    st_digest(tree + 4 * i, s);
}

template <int T>
__global__ void P2_BOUNDS(T) hash_leaves_ext2_kernel(const u64* __restrict__ cw, u64* __restrict__ tree, size_t leaves) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= leaves) return;
    u64 s[8];
    ld_digest(cw + 4 * i, s);
    s[4] = s[5] = s[6] = s[7] = 0;
    p2_permute<4>(s);
    st_digest(tree + 4 * i, s);
}

// Copy the first `count` digests of a layer to the following (copies-1) slots.
__global__ void replicate_kernel(u64* __restrict__ layer, size_t count, int copies) {
    size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t words = count * 4;
    if (k >= words * (size_t)(copies - 1)) return;
    layer[words + k] = layer[k % words];
}

static thread_local size_t t_coop_below = MK_COOP_BELOW_DEFAULT;
size_t mk_coop_below() { return t_coop_below; }

// one layer: `half` parents from the 2*half digests at `in`
static int merkle_level(const u64* in, u64* out, size_t half) {
    cudaStream_t s = stream();
    const P2Form f = p2_form(half);
    if (f == P2_ONE) {
        merkle_level_kernel<P2_WIDE><<<grid_for(half, P2_WIDE), P2_WIDE, 0, s>>>(in, out, half);
        return check_launch("merkle_level_kernel");
    }
    if (f == P2_PAIR) {
        if (p2_pair_threads(half) == 256)
            merkle_level_pair_kernel<256><<<grid_for(2 * half, 256), 256, 0, s>>>(in, out, half);
        else
            merkle_level_pair_kernel<128><<<grid_for(2 * half, 128), 128, 0, s>>>(in, out, half);
        return check_launch("merkle_level_pair_kernel");
    }
    int threads = coop_threads(half);
    GB_CUDA_TRY(launch_pdl(merkle_level_coop_kernel, grid_for(half * 8, threads), threads, s, in, out, half));
    return check_launch("merkle_level_coop_kernel");
}

static thread_local size_t t_top_nodes = MK_TOP_NODES;

int merkle_build_from_leaves(u64* tree, size_t leaves, u64* root_out) {
    u64* layer = tree;
    size_t nodes = leaves;
    const size_t top = t_top_nodes;
    while (nodes > top) {
        size_t half = nodes >> 1;
        int rc = merkle_level(layer, layer + 4 * nodes, half);
        if (rc) return rc;
        layer += 4 * nodes;
        nodes = half;
    }
    if (nodes > 1) {
        size_t half = nodes >> 1;
        int threads = (int)(8 * (half < 128 ? half : 128));
        threads = threads < 64 ? 64 : (threads + 31) / 32 * 32;
        GB_CUDA_TRY(launch_pdl(merkle_top_coop_kernel, 1, threads, stream(), layer, nodes, root_out));
        GB_LAUNCH_CHECK("merkle_top_coop_kernel");
    } else if (root_out) {
        GB_CUDA_TRY(cudaMemcpyAsync(root_out, layer, 32, cudaMemcpyDefault, stream()));  // root_out may be mapped host memory
    }
    return GB_OK;
}

int merkle_hash_leaves_gl(const u64* cw, u64* tree, size_t leaves) {
    const P2Form f = p2_form(leaves);
    if (f == P2_COOP) {
        int t = coop_threads(leaves);
        GB_CUDA_TRY(launch_pdl(hash_leaves_coop_kernel, grid_for(leaves * 8, t), t, stream(), cw, tree, leaves, 2));
        return check_launch("hash_leaves_coop_kernel");
    }
    if (f == P2_PAIR) {
        if (p2_pair_threads(leaves) == 256)
            hash_leaves_pair_kernel<256><<<grid_for(2 * leaves, 256), 256, 0, stream()>>>(cw, tree, leaves, 2);
        else
            hash_leaves_pair_kernel<128><<<grid_for(2 * leaves, 128), 128, 0, stream()>>>(cw, tree, leaves, 2);
        return check_launch("hash_leaves_pair_kernel");
    }
    hash_leaves_gl_kernel<P2_WIDE><<<grid_for(leaves, P2_WIDE), P2_WIDE, 0, stream()>>>(cw, tree, leaves);
    return check_launch("hash_leaves_gl_kernel");
}

int merkle_hash_leaves_ext2(const u64* cw, u64* tree, size_t leaves) {
    const P2Form f = p2_form(leaves);
    if (f == P2_COOP) {
        int t = coop_threads(leaves);
        GB_CUDA_TRY(launch_pdl(hash_leaves_coop_kernel, grid_for(leaves * 8, t), t, stream(), cw, tree, leaves, 4));
        return check_launch("hash_leaves_coop_kernel");
    }
    if (f == P2_PAIR) {
        if (p2_pair_threads(leaves) == 256)
            hash_leaves_pair_kernel<256><<<grid_for(2 * leaves, 256), 256, 0, stream()>>>(cw, tree, leaves, 4);
        else
            hash_leaves_pair_kernel<128><<<grid_for(2 * leaves, 128), 128, 0, stream()>>>(cw, tree, leaves, 4);
        return check_launch("hash_leaves_pair_kernel");
    }
    hash_leaves_ext2_kernel<P2_WIDE><<<grid_for(leaves, P2_WIDE), P2_WIDE, 0, stream()>>>(cw, tree, leaves);
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
    // one copy's subtree: its nodes are the leading entries of every layer; the copies are
    // filled afterwards, all layers in one launch
    int rc = merkle_hash_leaves_gl(cw, tree, sub);
    if (rc) return rc;
    size_t off = 0, layer_nodes = leaves, n = sub, total = 0;
    for (;;) {
        total += 4 * n * (copies - 1);
        if (n == 1) break;
        size_t half = n >> 1;
        rc = merkle_level(tree + off, tree + off + 4 * layer_nodes, half);
        if (rc) return rc;
        off += 4 * layer_nodes;
        layer_nodes >>= 1;
        n = half;
    }
    replicate_layers_kernel<<<grid_for(total, 256), 256, 0, s>>>(tree, leaves, sub, (int)copies, total);
    GB_LAUNCH_CHECK("replicate_layers_kernel");
    // the layer holding the copy roots is complete; finish the top copies_log levels
    return merkle_build_from_leaves(tree + off, layer_nodes);
}

template <int T>
__global__ void P2_BOUNDS(T) permute_batch_kernel(const u64* __restrict__ in, u64* __restrict__ out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u64 s[8];
#pragma unroll
    for (int k = 0; k < 8; k++) s[k] = in[8 * (size_t)i + k];
    p2_permute(s);
#pragma unroll
    for (int k = 0; k < 8; k++) out[8 * (size_t)i + k] = s[k];
}

template <int T>
__global__ void P2_BOUNDS(T) compress_batch_kernel(const u64* __restrict__ l, const u64* __restrict__ r,
                                                   u64* __restrict__ out, int n) {
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

size_t gb_set_coop_threshold(size_t parents) {
    size_t old = t_coop_below;
    t_coop_below = parents;
    return old;
}
size_t gb_get_coop_threshold(void) { return t_coop_below; }

size_t gb_set_merkle_top_nodes(size_t nodes) {
    size_t old = t_top_nodes;
    t_top_nodes = nodes < 2 ? 2 : nodes > 2048 ? 2048 : nodes;
    return old;
}
size_t gb_get_merkle_top_nodes(void) { return t_top_nodes; }

int poseidon2_hash_batch_ffi(const uint64_t* d_input, uint64_t* d_output, int n) {
    if (n < 0) return GB_EINVAL;
    if (n == 0) return GB_OK;
    if (p2_wide((size_t)n))
        permute_batch_kernel<P2_WIDE><<<grid_for(n, P2_WIDE), P2_WIDE, 0, stream()>>>(d_input, d_output, n);
    else
        permute_batch_kernel<P2_NARROW><<<grid_for(n, P2_NARROW), P2_NARROW, 0, stream()>>>(d_input, d_output, n);
    return check_launch("poseidon2_hash_batch_ffi");
}

int poseidon2_compress_batch_ffi(const uint64_t* d_left, const uint64_t* d_right, uint64_t* d_output, int n) {
    if (n < 0) return GB_EINVAL;
    if (n == 0) return GB_OK;
    if (p2_wide((size_t)n))
        compress_batch_kernel<P2_WIDE><<<grid_for(n, P2_WIDE), P2_WIDE, 0, stream()>>>(d_left, d_right, d_output, n);
    else
        compress_batch_kernel<P2_NARROW><<<grid_for(n, P2_NARROW), P2_NARROW, 0, stream()>>>(d_left, d_right, d_output,
                                                                                            n);
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
    return merkle_level(d_input, d_output, (size_t)n);
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
