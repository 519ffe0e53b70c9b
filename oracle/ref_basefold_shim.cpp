// The reference's own Basefold commit kernels run on the host, for pinning the oracle and the
// CUDA library to code the reference executes.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/ from the reference's
// sources where they lie (cuda/basefold.cuh with its includes, and the kernels that
// goldilocks-cuda-rs/cuda/wrapper.cu defines, extracted from that file at build time).  The
// kernel bodies are the reference's; ref_sim.hpp runs their grids on host threads.  The launch
// sequences below restate the host side of the reference's FFI functions, which cannot be
// compiled as host C++ because of the <<<>>> launch syntax; each cites the lines it follows.
#include <algorithm>
#include <cstring>
#include <vector>

#include "ref_sim.hpp"

#define __syncthreads() sim::syncthreads()
#include "basefold.cuh"
#include "sumcheck_prover.cuh"
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
inline GoldilocksExt2* ge(uint64_t* p) { return reinterpret_cast<GoldilocksExt2*>(p); }
inline const GoldilocksExt2* ge(const uint64_t* p) { return reinterpret_cast<const GoldilocksExt2*>(p); }
constexpr uint64_t P = 0xFFFFFFFF00000001ULL;

// gl_add_host (goldilocks-cuda-rs/src/basefold.rs:3144-3155): the host sum of per-block partials
uint64_t gl_add_host(uint64_t a, uint64_t b) {
    a %= P;
    b %= P;
    uint64_t sum = a + b;
    return (sum < a || sum >= P) ? sum - P : sum;
}
void reduce_ext2(const std::vector<uint64_t>& v, int num_blocks, uint64_t out[2]) {
    uint64_t c0 = 0, c1 = 0;
    for (int i = 0; i < num_blocks; i++) {
        c0 = gl_add_host(c0, v[2 * i]);
        c1 = gl_add_host(c1, v[2 * i + 1]);
    }
    out[0] = c0;
    out[1] = c1;
}
int product_blocks(size_t pair_count) {
    size_t b = (pair_count + BS - 1) / BS;
    return (int)(b < 256 ? b : 256);
}
}  // namespace

// The Fiat-Shamir transcript of the opening (BasefoldTranscript, zk-torch-3/src/transcript.rs:
// 331-350), supplied by the caller: the reference's is Rust.
struct RefTranscript {
    void* ctx;
    void (*observe_ext2)(void* ctx, const uint64_t v[2]);
    void (*observe_hash)(void* ctx, const uint64_t h[4]);
    uint64_t (*sample)(void* ctx);
    void (*sample_ext2)(void* ctx, uint64_t out[2]);
};

namespace {
// ext2_eq_dp_all (cuda/eq_lagrange.cuh:129-158): result in the buffer the last layer wrote
uint64_t* eq_dp_all_ext2(const uint64_t* r, uint64_t* buf_a, uint64_t* buf_b, int log_n) {
    size_t n = (size_t)1 << log_n;
    sim::launch(blocks_for(n), BS, [&] { ext2_eq_init_one_kernel(ge(buf_a), n); });
    size_t half_n = 1;
    for (int i = 0; i < log_n; i++) {
        sim::launch(blocks_for(half_n), BS, [&] { ext2_eq_dp_layer_kernel(ge(buf_a), ge(buf_b), ge(r), i, half_n); });
        std::swap(buf_a, buf_b);
        half_n <<= 1;
    }
    return buf_a;
}

// sumcheck_product_and_reduce_{mixed,ext2}[_reuse] (basefold.rs:2798-2897): per-block partials,
// summed on the host
template <bool MIXED>
void product_and_reduce(const uint64_t* eq, const uint64_t* bh, size_t pair_count, uint64_t oracle[6]) {
    int nb = product_blocks(pair_count);
    std::vector<uint64_t> p0(2 * nb), p1(2 * nb), p2(2 * nb);
    sim::launch_sync(nb, BS, [&] {
        if (MIXED)
            sumcheck_product_mixed_kernel(ge(eq), gf(bh), ge(p0.data()), ge(p1.data()), ge(p2.data()), pair_count);
        else
            sumcheck_product_ext2_kernel(ge(eq), ge(bh), ge(p0.data()), ge(p1.data()), ge(p2.data()), pair_count);
    });
    reduce_ext2(p0, nb, oracle);
    reduce_ext2(p1, nb, oracle + 2);
    reduce_ext2(p2, nb, oracle + 4);
}

void observe_oracle(RefTranscript* t, const uint64_t o[6]) {
    for (int c = 0; c < 3; c++) t->observe_ext2(t->ctx, o + 2 * c);
}

void tree_path(const uint64_t* tree, size_t num_leaves, size_t leaf, uint64_t* out) {
    size_t off = 0, sz = num_leaves, idx = leaf, k = 0;
    while (sz > 1) {
        std::memcpy(out + 4 * k, tree + (off + (idx ^ 1)) * 4, 32);
        k++;
        off += sz;
        sz /= 2;
        idx >>= 1;
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

// The transcript of GpuLinearSumcheckProver::prove (zk-torch-3/src/sumcheck/gpu_prover.rs:36-90),
// supplied by the caller: append_ext2("round_message", v) and challenge_ext2("challenge").
struct RefSumcheckTranscript {
    void* ctx;
    void (*append_message)(void* ctx, const uint64_t v[2]);
    void (*challenge)(void* ctx, uint64_t out[2]);
};

// GpuLinearSumcheckProver::prove on GpuSumcheckStateExt2 (goldilocks-cuda-rs/src/sumcheck_prover.rs:
// 215-410): base-field inputs lifted to Ext2, then per round sumcheck_round_message_ext2_ffi
// (wrapper.cu:1751-1766; block partials summed on the host), the transcript, and
// sumcheck_fold_ext2_ffi (wrapper.cu:1768-1785) into the other buffer.  polys: [d][2^num_vars] base
// values; msgs [num_vars][d+1][2], challenges [num_vars][2], finals [d][2], final_eval [2].
int ref_sumcheck_prove_ext2(const uint64_t* polys, int num_vars, int d, RefSumcheckTranscript* tr, uint64_t* msgs,
                            uint64_t* challenges, uint64_t* finals, uint64_t final_eval[2]) {
    if (d < 1 || d > MAX_DEGREE || num_vars < 0) return -1;
    const size_t original_size = (size_t)1 << num_vars;
    const size_t stride = 2 * original_size;
    std::vector<uint64_t> a((size_t)d * stride, 0), b((size_t)d * stride, 0);
    for (int i = 0; i < d; i++)
        for (size_t k = 0; k < original_size; k++) a[i * stride + 2 * k] = polys[i * original_size + k];
    uint64_t* cur = a.data();
    uint64_t* nxt = b.data();
    const int dp1 = d + 1;
    for (int round = 0; round < num_vars; round++) {
        size_t half = (original_size >> round) / 2;
        int nb = (int)std::min<size_t>((half + SUMCHECK_BLOCK_SIZE - 1) / SUMCHECK_BLOCK_SIZE, 256);
        std::vector<uint64_t> part((size_t)nb * dp1 * 2);
        sim::launch_sync(nb, SUMCHECK_BLOCK_SIZE, [&] {
            sumcheck_round_message_ext2_kernel(cur, part.data(), d, original_size, half);
        });
        uint64_t* m = msgs + (size_t)round * dp1 * 2;
        for (int c = 0; c < dp1; c++) {
            GoldilocksExt2 acc;
            for (int blk = 0; blk < nb; blk++) {
                size_t off = ((size_t)blk * dp1 + c) * 2;
                acc = ext2_add(acc, GoldilocksExt2(part[off], part[off + 1]));
            }
            m[2 * c] = canonicalize(acc.c[0].value);
            m[2 * c + 1] = canonicalize(acc.c[1].value);
            tr->append_message(tr->ctx, m + 2 * c);
        }
        uint64_t* ch = challenges + 2 * round;
        tr->challenge(tr->ctx, ch);
        unsigned grid = (unsigned)((half + SUMCHECK_BLOCK_SIZE - 1) / SUMCHECK_BLOCK_SIZE);
        sim::launch(grid, SUMCHECK_BLOCK_SIZE, [&] {
            sumcheck_fold_ext2_kernel(cur, nxt, ch[0], ch[1], d, original_size, half);
        });
        std::swap(cur, nxt);
    }
    GoldilocksExt2 fe(GoldilocksField(1));
    for (int i = 0; i < d; i++) {
        GoldilocksExt2 v(cur[i * stride], cur[i * stride + 1]);
        finals[2 * i] = canonicalize(v.c[0].value);
        finals[2 * i + 1] = canonicalize(v.c[1].value);
        fe = ext2_mul(fe, v);
    }
    final_eval[0] = canonicalize(fe.c[0].value);
    final_eval[1] = canonicalize(fe.c[1].value);
    return 0;
}

// BasefoldCommitment::open_ext2 (goldilocks-cuda-rs/src/basefold.rs:578-870) over the reference's
// kernels, writing the proof in the flat layout of the oracle (eval, oracles, folded roots, final
// codeword, then per query: index, round values, Merkle paths).  codeword / bh_evals / tree are
// the commitment's (bh_evals in the bit-reversed order the commitment keeps); table_entries are
// (point, weight) pairs at level_offsets.  Returns 0, or -1 for num_vars < 2.
int ref_basefold_open_ext2(const uint64_t* codeword, const uint64_t* bh_evals, const uint64_t* tree0,
                           const uint64_t root[4], int num_vars, int log_rate, const uint64_t* point,
                           const uint64_t* table_entries, const uint64_t* level_offsets, RefTranscript* tr,
                           int num_queries, uint64_t* proof) {
    if (num_vars < 2) return -1;
    const int num_rounds = num_vars;
    const size_t n = (size_t)1 << num_vars;
    const size_t L = (size_t)1 << (num_vars + log_rate);
    auto level = [&](int r) { return reinterpret_cast<const FoldingEntry*>(table_entries + 2 * level_offsets[r]); };
    uint64_t* pp = proof;
    uint64_t* eval_out = pp;
    pp += 2;
    uint64_t* oracles = pp;
    pp += (size_t)num_vars * 6;
    uint64_t* roots = pp;
    pp += (size_t)(num_vars - 1) * 4;
    uint64_t* final_cw = pp;
    pp += (size_t)2 << log_rate;
    uint64_t* queries = pp;

    tr->observe_hash(tr->ctx, root);
    for (int i = 0; i < num_vars; i++) tr->observe_ext2(tr->ctx, point + 2 * i);

    // 1-3: eq table, Type2 copy of bh_evals, eval = <bh, eq> (dot_product_mixed + host reduce)
    std::vector<uint64_t> eq_a(2 * n), eq_b(2 * n), bh_a(2 * n), bh_b(2 * n);
    uint64_t* eq_init = eq_dp_all_ext2(point, eq_a.data(), eq_b.data(), num_vars);
    if (eq_init != eq_a.data()) std::memcpy(eq_a.data(), eq_init, 16 * n);
    std::vector<uint64_t> bh_fp(bh_evals, bh_evals + n);
    sim::launch(blocks_for(n), BS, [&] { bit_reverse_permute_gl_kernel(gf(bh_fp.data()), num_vars); });
    {
        int dp_blocks = product_blocks(n);
        std::vector<uint64_t> part(2 * dp_blocks);
        sim::launch_sync(dp_blocks, BS, [&] {
            ext2_dot_product_mixed_kernel(gf(bh_fp.data()), ge(eq_a.data()), ge(part.data()), (int)n);
        });
        reduce_ext2(part, dp_blocks, eval_out);
    }

    // 4: first round, mixed (bh in F_p, eq in F_p^2)
    size_t pair_count = n / 2;
    sim::launch(blocks_for(pair_count), BS, [&] { sumcheck_interp_kernel(gf(bh_fp.data()), pair_count); });
    sim::launch(blocks_for(pair_count), BS, [&] { sumcheck_interp_ext2_kernel(ge(eq_a.data()), pair_count); });
    product_and_reduce<true>(eq_a.data(), bh_fp.data(), pair_count, oracles);
    observe_oracle(tr, oracles);

    // 5: round 0 challenge; bh moves to F_p^2 (bh_a), eq is evaluated into eq_b
    uint64_t ch[2];
    tr->sample_ext2(tr->ctx, ch);
    GoldilocksExt2 ch0(ch[0], ch[1]);
    sim::launch(blocks_for(pair_count), BS, [&] { sumcheck_eval_mixed_kernel(gf(bh_fp.data()), ch0, ge(bh_a.data()), pair_count); });
    sim::launch(blocks_for(pair_count), BS, [&] { sumcheck_eval_ext2_kernel(ge(eq_a.data()), ch0, ge(eq_b.data()), pair_count); });
    pair_count /= 2;
    bool eq_is_a = false, bh_is_a = true;
    sim::launch(blocks_for(pair_count), BS, [&] { sumcheck_interp_ext2_kernel(ge(eq_b.data()), pair_count); });
    sim::launch(blocks_for(pair_count), BS, [&] { sumcheck_interp_ext2_kernel(ge(bh_a.data()), pair_count); });
    product_and_reduce<false>(eq_b.data(), bh_a.data(), pair_count, oracles + 6);
    observe_oracle(tr, oracles + 6);

    // codeword fold of round 0 (mixed) and its tree
    size_t cw_pair_count = L / 2;
    std::vector<std::vector<uint64_t>> folds(num_rounds), trees(num_rounds - 1);
    {
        size_t sz = cw_pair_count;
        for (int r = 0; r < num_rounds; r++, sz /= 2) folds[r].resize(2 * sz);
    }
    auto build_tree = [&](int r, size_t cw_len_ext2) {
        size_t leaves = cw_len_ext2 / 2;
        trees[r].resize((2 * leaves - 1) * 4);
        ref_merkle_tree_ext2(folds[r].data(), trees[r].data(), (int)leaves);
        std::memcpy(roots + 4 * r, trees[r].data() + (2 * leaves - 2) * 4, 32);
        tr->observe_hash(tr->ctx, roots + 4 * r);
    };
    sim::launch(blocks_for(cw_pair_count), BS, [&] {
        basefold_fold_mixed_kernel(gf(codeword), level(0), ch0, ge(folds[0].data()), cw_pair_count);
    });
    build_tree(0, cw_pair_count);
    cw_pair_count /= 2;

    // 6: remaining rounds, fused eval + interp + product
    for (int round = 1; round < num_rounds - 1; round++) {
        tr->sample_ext2(tr->ctx, ch);
        GoldilocksExt2 c(ch[0], ch[1]);
        size_t product_pairs = pair_count / 2;
        int nb = product_blocks(product_pairs);
        std::vector<uint64_t> p0(2 * nb), p1(2 * nb), p2(2 * nb);
        const uint64_t* eq_in = eq_is_a ? eq_a.data() : eq_b.data();
        const uint64_t* bh_in = bh_is_a ? bh_a.data() : bh_b.data();
        uint64_t* eq_out = eq_is_a ? eq_b.data() : eq_a.data();
        uint64_t* bh_out = bh_is_a ? bh_b.data() : bh_a.data();
        sim::launch_sync(nb, BS, [&] {
            fused_sumcheck_round_ext2_kernel(ge(eq_in), ge(bh_in), c, ge(eq_out), ge(bh_out), ge(p0.data()),
                                             ge(p1.data()), ge(p2.data()), product_pairs);
        });
        eq_is_a = !eq_is_a;
        bh_is_a = !bh_is_a;
        pair_count /= 2;
        uint64_t* o = oracles + 6 * (round + 1);
        reduce_ext2(p0, nb, o);
        reduce_ext2(p1, nb, o + 2);
        reduce_ext2(p2, nb, o + 4);
        observe_oracle(tr, o);
        sim::launch(blocks_for(cw_pair_count), BS, [&] {
            basefold_fold_ext2_kernel(ge(folds[round - 1].data()), level(round), c, ge(folds[round].data()),
                                      cw_pair_count);
        });
        build_tree(round, cw_pair_count);
        cw_pair_count /= 2;
    }

    // last fold: the final codeword
    tr->sample_ext2(tr->ctx, ch);
    {
        GoldilocksExt2 c(ch[0], ch[1]);
        int last = num_rounds - 1;
        sim::launch(blocks_for(cw_pair_count), BS, [&] {
            basefold_fold_ext2_kernel(ge(folds[last - 1].data()), level(last), c, ge(folds[last].data()),
                                      cw_pair_count);
        });
        std::memcpy(final_cw, folds[last].data(), 16 * cw_pair_count);
    }

    // queries (extract_ext2_queries, basefold.rs:2310-2406): every index sampled first
    std::vector<size_t> leaf(num_queries);
    for (int q = 0; q < num_queries; q++) leaf[q] = (size_t)(tr->sample(tr->ctx) % (uint64_t)(L / 2));
    for (int q = 0; q < num_queries; q++) {
        *queries++ = leaf[q];
        uint64_t* vals = queries;
        queries += (size_t)num_vars * 4;
        vals[0] = codeword[2 * leaf[q]];
        vals[1] = 0;
        vals[2] = codeword[2 * leaf[q] + 1];
        vals[3] = 0;
        size_t idx = leaf[q] / 2;
        for (int i = 0; i + 1 < num_rounds; i++) {
            std::memcpy(vals + 4 * (i + 1), folds[i].data() + idx * 4, 32);
            idx /= 2;
        }
        tree_path(tree0, L / 2, leaf[q], queries);
        queries += (size_t)(num_vars + log_rate - 1) * 4;
        idx = leaf[q] / 2;
        for (int i = 0; i + 1 < num_rounds; i++) {
            tree_path(trees[i].data(), (L >> (i + 1)) / 2, idx, queries);
            queries += (size_t)(num_vars + log_rate - 2 - i) * 4;
            idx /= 2;
        }
    }
    return 0;
}

}  // extern "C"
