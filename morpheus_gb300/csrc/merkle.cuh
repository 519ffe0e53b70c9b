// Poseidon2 Merkle trees on the device.
//
// Layout (goldilocks-cuda-rs/src/merkle.rs:1-10): one buffer of (2L - 1) digests of
// 4 u64, layers packed leaves first, root last.  Leaves hash pairs of codeword
// elements: P2(a, b, 0^6)[0..4] for base-field codewords, P2(a.c0, a.c1, b.c0,
// b.c1, 0^4)[0..4] for Ext2 codewords (goldilocks-cuda-rs/cuda/wrapper.cu:1604-1650);
// parents are P2(left || right)[0..4].
#pragma once
#include "common.cuh"
#include "poseidon2.cuh"

namespace gb {

// Number of u64 words before layer `level` of a tree with `leaves` leaves.
__host__ __device__ inline size_t tree_layer_offset(size_t leaves, int level) {
    size_t off = 0, sz = leaves;
    for (int l = 0; l < level; l++) {
        off += sz;
        sz >>= 1;
    }
    return off * 4;
}

__host__ __device__ inline int tree_depth(size_t leaves) {
    int d = 0;
    while (((size_t)1 << d) < leaves) d++;
    return d;
}

__device__ __forceinline__ void st_digest(u64* p, const u64* s) {
    ulonglong2 a, b;
    a.x = s[0];
    a.y = s[1];
    b.x = s[2];
    b.y = s[3];
    reinterpret_cast<ulonglong2*>(p)[0] = a;
    reinterpret_cast<ulonglong2*>(p)[1] = b;
}
__device__ __forceinline__ void ld_digest(const u64* p, u64* s) {
    ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2*>(p));
    ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2*>(p) + 1);
    s[0] = a.x;
    s[1] = a.y;
    s[2] = b.x;
    s[3] = b.y;
}

// Work below this many permutations per launch is latency-bound: one thread's
// permutation is a long serial chain, so those launches use 8 lanes per state (at about
// half the throughput of one state per thread).  The threshold belongs to the calling
// thread (gb_set_coop_threshold); many concurrent proofs favour a lower one.
constexpr size_t MK_COOP_BELOW_DEFAULT = 16384;
size_t mk_coop_below();
// Once a layer has at most this many nodes, the layers above it are finished by one CTA
// (default; the calling thread can raise it with gb_set_merkle_top_nodes: fewer launches,
// a longer chain inside the one CTA).
constexpr size_t MK_TOP_NODES = 16;

// Launch shape of the one-permutation-per-thread kernels: 512-thread CTAs, four per SM (at most
// 32 registers; 8-16 bytes spill), measured 1.917 G permutations/s on a 2^21-parent layer against
// 1.891 G with three per SM (40 registers), and 1.52-1.59 G with 128-thread CTAs of the same code.
// The likely cause of the CTA-size effect is instruction-cache locality: the unrolled permutation
// is about 15 k instructions, and the warps of one CTA run through it together.  Launches below
// P2_WIDE_FROM permutations keep 128-thread CTAs, so that a launch of less than a wave still
// spreads over every SM.  The segmented kernels of the batched engine (P2_SEG_BOUNDS) keep three
// CTAs per SM: at 32 registers their segment bookkeeping spills (28 bytes, 784 in one of them),
// and the batch measured 993-997 against 1009-1013 proofs/s.
constexpr int P2_WIDE = 512, P2_NARROW = 128;
constexpr size_t P2_WIDE_FROM = (size_t)1 << 16;
#define P2_BOUNDS(T) __launch_bounds__(T, (T) == 512 ? 4 : 10)
#define P2_SEG_BOUNDS(T) __launch_bounds__(T, (T) == 512 ? 3 : 10)
inline bool p2_wide(size_t items) { return items >= P2_WIDE_FROM; }

// Form of a single-tree launch of `items` permutations, by the per-launch times measured on
// GB300 (a 2^21-leaf tree's chain of levels down to 16 nodes: 1.32 ms against 1.50 ms with
// the one-thread form from the cooperative threshold up): the 8-lane cooperative form below
// mk_coop_below(), the pair form (p2_permute_pair) below P2_ONE_FROM, and one permutation per
// thread in 512-thread CTAs from there.
constexpr size_t P2_ONE_FROM = (size_t)1 << 16;
enum P2Form { P2_COOP, P2_PAIR, P2_ONE };
inline P2Form p2_form(size_t items) {
    return items < mk_coop_below() ? P2_COOP : items < P2_ONE_FROM ? P2_PAIR : P2_ONE;
}
// pair-form CTA size (2 threads per permutation) and its bounds (up to 64 registers)
inline int p2_pair_threads(size_t items) { return items >= ((size_t)1 << 15) ? 256 : 128; }
#define P2_PAIR_BOUNDS(T) __launch_bounds__(T, (T) == 256 ? 4 : 8)

// Programmatic dependent launch for the latency-bound cooperative kernels: launched with
// launch_pdl, such a kernel may be scheduled while the kernel before it on the stream drains;
// pdl_enter (its first statement) lets the next such kernel be scheduled in turn and waits for
// the previous kernel's completion and memory before anything is read.  Without the launch
// attribute both instructions return at once.  Only these small, single-wave kernels use it:
// an early-scheduled kernel holds SM slots while it waits.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}
template <typename... Params, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(Params...), unsigned grid, int block, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// CTA size for a cooperative launch over `groups` 8-lane groups: small launches use
// 64-thread CTAs so that the work spreads over as many SMs as there are CTAs.
inline int coop_threads(size_t groups) { return groups * 8 >= (size_t)num_sms() * 256 ? 256 : 64; }

// Host-side tree builders (merkle.cu).  merkle_build_from_leaves expects the leaf
// digests in layer 0.  All launches on gb::stream(); no synchronisation.
// root_out (device, 4 words) also receives the root when given.
int merkle_build_from_leaves(u64* tree, size_t leaves, u64* root_out = nullptr);
int merkle_hash_leaves_gl(const u64* cw, u64* tree, size_t leaves);
int merkle_hash_leaves_ext2(const u64* cw, u64* tree, size_t leaves);
// Tree over a base-field codeword made of 2^copies identical blocks: hashes one
// block's subtree, replicates it, and finishes the top `copies` levels.
int merkle_tree_gl_replicated(const u64* cw, u64* tree, size_t leaves, int copies_log);

}  // namespace gb
