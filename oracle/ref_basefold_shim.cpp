// The reference's own Basefold commit kernels run on the host, for pinning the oracle and the
// CUDA library to code the reference executes.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/ from the reference's
// sources where they lie (cuda/basefold.cuh with its includes, and the kernels that
// goldilocks-cuda-rs/cuda/wrapper.cu defines, extracted from that file at build time).  The
// kernel bodies are the reference's; ref_sim.hpp runs their grids on host threads.  The launch
// sequences below restate the host side of the reference's FFI functions, which cannot be
// compiled as host C++ because of the <<<>>> launch syntax; each cites the lines it follows.
#include <cstring>

#include "ref_sim.hpp"

#define __syncthreads() sim::syncthreads()
#include "basefold.cuh"
#include "wrapper_kernels.inc"

SIM_DEFINE_BUILTINS

namespace {
constexpr int BS = BLOCK_SIZE;
inline unsigned blocks_for(size_t n) { return (unsigned)((n + BS - 1) / BS); }
inline GoldilocksField* gf(uint64_t* p) { return reinterpret_cast<GoldilocksField*>(p); }
inline const GoldilocksField* gf(const uint64_t* p) { return reinterpret_cast<const GoldilocksField*>(p); }

// build_merkle_tree_inplace (wrapper.cu:1653-1672): one layer launch per level, leaves first
void merkle_layers(uint64_t* tree, int num_leaves) {
    int layer_offset = 0, layer_size = num_leaves;
    while (layer_size > 1) {
        int num_pairs = layer_size / 2;
        const uint64_t* in = tree + (size_t)layer_offset * 4;
        uint64_t* out = tree + (size_t)(layer_offset + layer_size) * 4;
        sim::launch(blocks_for(num_pairs), BS, [&] { poseidon2_merkle_layer_kernel_ffi(in, out, num_pairs); });
        layer_offset += layer_size;
        layer_size = num_pairs;
    }
}
}  // namespace

extern "C" {

// poseidon2_init (cuda/poseidon2.cuh): the __constant__ round constants from their host copies
void ref_bf_init(void) {
    std::memcpy((void*)d_RC_EXT_8, h_RC_EXT_8, sizeof(h_RC_EXT_8));
    std::memcpy((void*)d_RC_INT, h_RC_INT, sizeof(h_RC_INT));
    std::memcpy((void*)d_DIAG_8, h_DIAG_8, sizeof(h_DIAG_8));
}

// basefold_bhc_interpolate_ffi (wrapper.cu:1242-1274): evals -> coeffs (Type2) and bh_evals
// (Type1, the bit-reversed copy)
void ref_bhc_interpolate(const uint64_t* evals, uint64_t* coeffs, uint64_t* bh_evals, int num_vars) {
    size_t n = (size_t)1 << num_vars;
    unsigned grid = blocks_for(n / 2);
    sim::launch(grid, BS, [&] { bhc_interp_first_pass_kernel(gf(evals), gf(coeffs), gf(bh_evals), n); });
    for (int k = 1; k < num_vars; k++) {
        size_t half_chunk = (size_t)1 << k;
        sim::launch(grid, BS, [&] { bhc_interp_layer_kernel(gf(coeffs), half_chunk, n); });
    }
    sim::launch(blocks_for(n), BS, [&] { bit_reverse_permute_gl_kernel(gf(bh_evals), num_vars); });
}

// basefold_encode_ffi (wrapper.cu:1277-1313): repetition code, num_vars butterfly layers, then
// bit reversal of the 2^(num_vars + log_rate) codeword
void ref_basefold_encode(const uint64_t* coeffs, uint64_t* codeword, int num_vars, int log_rate) {
    size_t k = (size_t)1 << num_vars;
    int rate = 1 << log_rate;
    size_t n_output = k * rate;
    sim::launch(blocks_for(n_output), BS, [&] { repetition_encode_kernel(gf(coeffs), gf(codeword), rate, n_output); });
    for (int i = 0; i < num_vars; i++) {
        size_t half_chunk = (size_t)1 << (i + log_rate);
        sim::launch(blocks_for(n_output / 2), BS, [&] { foldable_domain_layer_kernel(gf(codeword), half_chunk, n_output); });
    }
    sim::launch(blocks_for(n_output), BS, [&] { bit_reverse_permute_gl_kernel(gf(codeword), num_vars + log_rate); });
}

// poseidon2_merkle_tree_gl_ffi (wrapper.cu:1677-1692): leaf digests of codeword pairs, then the tree
void ref_merkle_tree_gl(const uint64_t* codeword, uint64_t* tree, int num_leaves) {
    sim::launch(blocks_for(num_leaves), BS, [&] { hash_gl_leaves_kernel(codeword, tree, num_leaves); });
    merkle_layers(tree, num_leaves);
}

// poseidon2_merkle_tree_ext2_ffi (wrapper.cu:1697-1710)
void ref_merkle_tree_ext2(const uint64_t* codeword, uint64_t* tree, int num_leaves) {
    sim::launch(blocks_for(num_leaves), BS, [&] { hash_ext2_leaves_kernel(codeword, tree, num_leaves); });
    merkle_layers(tree, num_leaves);
}

// The Rust commit's sequence (BasefoldCommitment::commit_device, goldilocks-cuda-rs/src/basefold.rs:
// 380-410): interpolate, encode, tree over the codeword's pairs; root = the tree's last node.
void ref_basefold_commit(const uint64_t* evals, int num_vars, int log_rate, uint64_t* codeword, uint64_t* bh_evals,
                         uint64_t* tree, uint64_t root[4]) {
    size_t n = (size_t)1 << num_vars;
    uint64_t* coeffs = new uint64_t[n];
    ref_bhc_interpolate(evals, coeffs, bh_evals, num_vars);
    ref_basefold_encode(coeffs, codeword, num_vars, log_rate);
    delete[] coeffs;
    int leaves = (int)(((size_t)1 << (num_vars + log_rate)) / 2);
    ref_merkle_tree_gl(codeword, tree, leaves);
    std::memcpy(root, tree + (size_t)(2 * leaves - 2) * 4, 32);
}

}  // extern "C"
