/*
 * goldilocks_cuda_wrapper.h -- C ABI of the GB300-native Goldilocks prover library.
 *
 * Part 1 is a drop-in for the extern "C" surface that goldilocks-cuda-rs binds
 * (goldilocks-cuda-rs/src/ffi.rs, implemented by goldilocks-cuda-rs/cuda/wrapper.cu):
 * same names, argument meaning and return codes (0 ok, -1 CUDA error; -2 invalid
 * argument where the reference would have launched out of bounds).  Every data
 * pointer is a caller-owned device pointer unless its name starts with h_.
 * Field elements are raw u64 (any representative mod p is accepted); Ext2
 * values are interleaved (c0, c1); folding tables are (point, weight) pairs;
 * digests are 4 u64.
 *
 * Part 2 (gb_*) adds entry points with no reference counterpart: stream
 * selection, whole-proof drivers that keep every round on the device, and the
 * batched prover.  Outputs of the gb_* drivers are canonical.
 *
 * All launches go to the calling thread's stream: the per-thread default stream
 * (as the reference, built with --default-stream per-thread) unless gb_set_stream
 * selected another.  Functions documented as synchronising wait for that stream.
 */
#ifndef GOLDILOCKS_CUDA_WRAPPER_H
#define GOLDILOCKS_CUDA_WRAPPER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ===================== Part 1: reference ABI ===================== */

/* goldilocks-cuda-rs/src/ffi.rs:11-12 (wrapper.cu:27-50).  Constants are compiled in,
 * so both only select/validate device 0 as the reference does. */
int goldilocks_cuda_init(void);
int poseidon2_cuda_init(void);

/* Memory / device (ffi.rs:18-26, :306-309) */
int cuda_malloc(void **ptr, size_t size);
int cuda_free(void *ptr);
int cuda_memcpy_htod(void *dst, const void *src, size_t size);
int cuda_memcpy_dtoh(void *dst, const void *src, size_t size);
int cuda_memcpy_dtod(void *dst, const void *src, size_t size);
int cuda_device_synchronize(void);
int cuda_get_last_error(void);
int cuda_peek_at_last_error(void);
int cuda_mem_get_info(size_t *free_bytes, size_t *total_bytes);
/* almost-goldilocks-cuda-rs/src/ffi.rs:85 (almost wrapper.cu:283-296): trim the current device's
 * stream-ordered pool to min_bytes_to_keep.  The library sets that pool's release threshold to
 * the maximum on first use, as the reference does, so pooled memory is kept until trimmed. */
int cuda_pool_trim(size_t min_bytes_to_keep);
int cuda_set_device(int device);
int cuda_get_device(int *device);
int cuda_get_device_count(int *count);
int cuda_get_device_name(int device, char *name, int max_len);

/* Batch field ops (ffi.rs:32-60, :185-260) */
int gl_batch_add(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int gl_batch_sub(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int gl_batch_mul(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int gl_batch_inverse(const uint64_t *d_a, uint64_t *d_result, int n);
int ext2_batch_add_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int ext2_batch_sub_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int ext2_batch_mul_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
/* The rest of the element-wise ops (ffi.rs:105-131, :163-280, :633-639; wrapper.cu:180-858,
 * :1790-1815, :2282, :2446), canonical outputs; Ext2 = F_p[X]/(X^2 - 7) as (c0, c1), Ext5 =
 * F_p[X]/(X^5 - 3) as (c0..c4); inverses (and divisions) by zero give zero.  The quantisation
 * helpers gl_scale_up/down and gl_decompose_bits32 belong to the einsum/ReLU basic blocks and are
 * not part of this library. */
int gl_batch_div(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int gl_batch_mul_scalar(uint64_t scalar, const uint64_t *d_a, uint64_t *d_result, int n);
int gl_batch_neg(const uint64_t *d_a, uint64_t *d_result, int n);
int gl_batch_square(const uint64_t *d_a, uint64_t *d_result, int n);
int gl_batch_double(const uint64_t *d_a, uint64_t *d_result, int n);
int gl_batch_exp(const uint64_t *d_a, uint64_t exp, uint64_t *d_result, int n);
int ext2_batch_inverse_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext2_batch_mul_scalar_ffi(uint64_t scalar, const uint64_t *d_a, uint64_t *d_result, int n);
int ext2_batch_neg_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext2_batch_square_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext2_batch_frobenius_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext2_batch_conjugate_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext2_batch_exp_ffi(const uint64_t *d_a, uint64_t exp, uint64_t *d_result, int n);
/* d_acc[i] += (scalar_c0 + scalar_c1 X) d_src[i], Ext2 */
int ext2_scale_accumulate_ffi(uint64_t scalar_c0, uint64_t scalar_c1, const uint64_t *d_src, uint64_t *d_acc, int n);
int ext5_batch_add_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int ext5_batch_sub_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int ext5_batch_mul_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_result, int n);
int ext5_batch_inverse_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext5_batch_mul_scalar_ffi(uint64_t scalar, const uint64_t *d_a, uint64_t *d_result, int n);
int ext5_batch_neg_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext5_batch_square_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext5_batch_frobenius_ffi(const uint64_t *d_a, uint64_t *d_result, int n);
int ext5_batch_exp_ffi(const uint64_t *d_a, uint64_t exp, uint64_t *d_result, int n);
int gl_to_ext2_batch_ffi(const uint64_t *d_input, uint64_t *d_output, int n);
int ext2_to_gl_batch_ffi(const uint64_t *d_input, uint64_t *d_output, int n);
int gl_to_ext5_batch_ffi(const uint64_t *d_input, uint64_t *d_output, int n);
int ext5_to_gl_batch_ffi(const uint64_t *d_input, uint64_t *d_output, int n);
int gl_memset_zero(uint64_t *d_buf, size_t n_u64);
int gl_zero_buffer(uint64_t *d_buf, int n);

/* Poseidon2 width 8 (ffi.rs:287-300; wrapper.cu:864-962).
 * hash_batch: full permutation of n 8-element states; compress/merkle_layer: 2-to-1. */
int poseidon2_hash_batch_ffi(const uint64_t *d_input, uint64_t *d_output, int n);
int poseidon2_compress_batch_ffi(const uint64_t *d_left, const uint64_t *d_right, uint64_t *d_output, int n);
int poseidon2_merkle_layer_ffi(const uint64_t *d_input, uint64_t *d_output, int n);

/* eq(r, x) tables (ffi.rs:396-410; wrapper.cu:1117-1160).  Result lands in d_buf_a or
 * d_buf_b; *d_result tells which.  Variable i <-> bit i of x. */
int eq_dp_all_ffi(const uint64_t *d_r, uint64_t *d_buf_a, uint64_t *d_buf_b, int log_n, uint64_t **d_result);
int ext2_eq_dp_all_ffi(const uint64_t *d_r, uint64_t *d_buf_a, uint64_t *d_buf_b, int log_n, uint64_t **d_result);

/* Basefold (ffi.rs:416-545; wrapper.cu:1223-1600) */
int basefold_bit_reverse_gl_ffi(uint64_t *d_data, int log_n);
int basefold_bit_reverse_ext2_ffi(uint64_t *d_data, int log_n);
/* evals -> Type2 monomial coefficients + bit-reversed copy of evals; synchronising */
int basefold_bhc_interpolate_ffi(const uint64_t *d_evals, uint64_t *d_coeffs, uint64_t *d_bh_evals, int num_vars);
/* repetition x 2^log_rate, num_vars +-1 butterfly layers, bit reversal; synchronising */
int basefold_encode_ffi(const uint64_t *d_coeffs, uint64_t *d_codeword, int num_vars, int log_rate);
int basefold_fold_gl_ffi(const uint64_t *d_codeword, const uint64_t *d_table, uint64_t challenge,
                         uint64_t *d_output, int pair_count);
int basefold_fold_mixed_ffi(const uint64_t *d_codeword, const uint64_t *d_table, uint64_t challenge_c0,
                            uint64_t challenge_c1, uint64_t *d_output, int pair_count);
int basefold_fold_ext2_ffi(const uint64_t *d_codeword, const uint64_t *d_table, uint64_t challenge_c0,
                           uint64_t challenge_c1, uint64_t *d_output, int pair_count);
int basefold_sumcheck_interp_gl_ffi(uint64_t *d_data, int pair_count);
int basefold_sumcheck_interp_ext2_ffi(uint64_t *d_data, int pair_count);
/* product kernels: per-block partials of (c0, c1, c2), num_blocks of each; the caller sums them */
int basefold_sumcheck_product_gl_ffi(const uint64_t *d_eq, const uint64_t *d_bh, uint64_t *d_partial_c0,
                                     uint64_t *d_partial_c1, uint64_t *d_partial_c2, int pair_count, int num_blocks);
int basefold_sumcheck_product_mixed_ffi(const uint64_t *d_eq, const uint64_t *d_bh, uint64_t *d_partial_c0,
                                        uint64_t *d_partial_c1, uint64_t *d_partial_c2, int pair_count,
                                        int num_blocks);
int basefold_sumcheck_product_ext2_ffi(const uint64_t *d_eq, const uint64_t *d_bh, uint64_t *d_partial_c0,
                                       uint64_t *d_partial_c1, uint64_t *d_partial_c2, int pair_count,
                                       int num_blocks);
int basefold_sumcheck_eval_gl_ffi(const uint64_t *d_data, uint64_t challenge, uint64_t *d_output, int pair_count);
int basefold_sumcheck_eval_mixed_ffi(const uint64_t *d_data, uint64_t challenge_c0, uint64_t challenge_c1,
                                     uint64_t *d_output, int pair_count);
int basefold_sumcheck_eval_ext2_ffi(const uint64_t *d_data, uint64_t challenge_c0, uint64_t challenge_c1,
                                    uint64_t *d_output, int pair_count);
int fused_sumcheck_round_ext2_ffi(const uint64_t *d_eq_in, const uint64_t *d_bh_in, uint64_t challenge_c0,
                                  uint64_t challenge_c1, uint64_t *d_eq_out, uint64_t *d_bh_out,
                                  uint64_t *d_partial_c0, uint64_t *d_partial_c1, uint64_t *d_partial_c2,
                                  int pair_count, int num_blocks);
int basefold_dot_product_gl_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_partial, int n, int num_blocks);
int basefold_dot_product_mixed_ffi(const uint64_t *d_a, const uint64_t *d_b, uint64_t *d_partial, int n,
                                   int num_blocks);

/* Merkle trees (ffi.rs:549-560; wrapper.cu:1604-1714).  d_tree holds (2 num_leaves - 1) digests,
 * layers packed leaves first, root last.  Synchronising. */
int poseidon2_merkle_tree_gl_ffi(const uint64_t *d_codeword, uint64_t *d_tree, int num_leaves);
int poseidon2_merkle_tree_ext2_ffi(const uint64_t *d_codeword, uint64_t *d_tree, int num_leaves);

/* Product sumcheck (ffi.rs:588-630; wrapper.cu:1716-1790).  d polynomials packed with
 * stride original_size (Ext2: 2*original_size u64).  round_message writes num_blocks*(d+1)
 * partial sums (Ext2: x2) whose sum is the round message; synchronising. */
int sumcheck_round_message_ffi(const uint64_t *d_polys, uint64_t *d_partial, int d, size_t original_size,
                               size_t half, int num_blocks);
int sumcheck_fold_ffi(const uint64_t *d_input, uint64_t *d_output, uint64_t challenge, int d,
                      size_t original_size, size_t half);
int sumcheck_round_message_ext2_ffi(const uint64_t *d_polys, uint64_t *d_partial, int d, size_t original_size,
                                    size_t half, int num_blocks);
int sumcheck_fold_ext2_ffi(const uint64_t *d_input, uint64_t *d_output, uint64_t challenge_c0,
                           uint64_t challenge_c1, int d, size_t original_size, size_t half);

/* ---- Monolith-12 Merkle trees (goldilocks-cuda-rs/src/ffi.rs:565-582; the crate's default Merkle
 * hash, Cargo.toml:22-24; semantics of src/cpu_monolith.rs): leaf i = H(cw[2i], cw[2i+1]) (gl) or
 * H(cw[4i..4i+3]) (ext2), parents H(left || right), digests the first 4 words (canonical),
 * layout as the Poseidon2 trees.  Synchronising.  monolith_permute_test_ffi permutes one
 * 12-word host state on the device.  monolith_cuda_init has nothing to set up (constants are
 * compiled in). */
int monolith_cuda_init(void);
int monolith_merkle_tree_gl_ffi(const uint64_t *d_codeword, uint64_t *d_tree, int num_leaves);
int monolith_merkle_tree_ext2_ffi(const uint64_t *d_codeword, uint64_t *d_tree, int num_leaves);
int monolith_permute_test_ffi(const uint64_t *h_input, uint64_t *h_output);

/* ---- Fiat-Shamir challengers on the device (goldilocks-cuda-rs/src/ffi.rs:314-372; semantics of
 * cuda/challenger.cuh:37-222): n independent duplex sponges over Poseidon2-w8, rate 4.  A state
 * is challenger_state_size() = 136 bytes (sponge[8], input[4], output[4] u64, input_count,
 * output_count int).  Batched entry points act on states 0..n-1; state i observes values
 * [i*count, (i+1)*count) (observe: count = 1, observe_ext2: 2) and writes its samples to
 * [i*count, ...) (sample: 1, ext2: 2, ext5: 5).  Sampled values are canonical.  Launch only. */
int challenger_state_size(void);
int challenger_alloc_states(void **d_states, int n);
int challenger_init_states(void *d_states, int n);
int challenger_observe_ffi(void *d_states, const uint64_t *d_values, int n);
int challenger_observe_slice_ffi(void *d_states, const uint64_t *d_values, int count, int n);
int challenger_sample_ffi(void *d_states, uint64_t *d_outputs, int n);
int challenger_sample_array_ffi(void *d_states, uint64_t *d_outputs, int count, int n);
int challenger_sample_ext2_ffi(void *d_states, uint64_t *d_outputs, int n);
int challenger_sample_ext5_ffi(void *d_states, uint64_t *d_outputs, int n);
int challenger_observe_ext2_ffi(void *d_states, const uint64_t *d_values, int n);
/* one state (challenger_state_size() bytes); synchronising */
int challenger_copy_state_to_host(void *h_state, const void *d_state);
int challenger_copy_state_to_device(void *d_state, const void *h_state);

/* ===================== Part 2: GB300 additions (no reference counterpart) ===================== */

/* Fiat-Shamir transcript state: the fields of zk-torch-3's Transcript
 * (zk-torch-3/src/transcript.rs:178-185) in a C layout. */
typedef struct gb_transcript {
    uint64_t st[8];
    uint64_t inb[4];
    uint64_t outb[4];
    uint32_t nin;
    uint32_t nout;
} gb_transcript;

/* Launch stream of the calling thread (NULL = per-thread default stream). */
int gb_set_stream(void *stream);
void *gb_get_stream(void);
/* Last error message of the calling thread ("" if none). */
const char *gb_last_error(void);
int gb_device_sm_count(void);
/* Number of kernels this library has launched in the process (all threads). */
unsigned long long gb_launch_count(void);
/* cudaFuncAttributes::binaryVersion of this library's kernels on the current device (103 for
 * sm_103a code), -1 on error. */
int gb_binary_version(void);
/* Measurement probe: blocks x 256 threads, each running 8 independent chains of `iters`
 * Goldilocks multiplications; d_out receives blocks*256 words.  Times the arithmetic
 * ceiling that the Poseidon2 kernels are compared against.  Launch only. */
int gb_mulmod_probe(uint64_t *d_out, int blocks, int iters);

/* Merkle scheduling knob of the calling thread: tree layers (and leaf hashes) of fewer than
 * `parents` permutations use 8 lanes per permutation (lowest latency); from there up to 2^16
 * permutations 2 lanes per permutation, and above that one thread per permutation (highest
 * throughput).  Default 16384; results do not depend on it.  Returns the previous value. */
size_t gb_set_coop_threshold(size_t parents);
size_t gb_get_coop_threshold(void);
/* Second Merkle knob of the calling thread: once a layer has at most `nodes` digests (2..2048,
 * default 16), one CTA finishes the tree in a single launch.  Larger values mean fewer launches
 * and a longer chain inside that CTA.  Returns the previous value. */
size_t gb_set_merkle_top_nodes(size_t nodes);
size_t gb_get_merkle_top_nodes(void);

/* Transcript helpers (host): new(label), append_u64(label), challenge_ext2(label). */
void gb_transcript_new(gb_transcript *t, const char *label);
void gb_transcript_append_u64(gb_transcript *t, const char *label, uint64_t v);
void gb_transcript_append_ext2(gb_transcript *t, const char *label, const uint64_t v[2]);
void gb_transcript_challenge_ext2(gb_transcript *t, const char *label, uint64_t out[2]);

/* Whole product-sumcheck proof, GpuLinearSumcheckProver::{new, prove} semantics
 * (zk-torch-3/src/sumcheck/gpu_prover.rs:21-89): appends num_var/num_poly, then per round
 * d+1 Ext2 messages and one Ext2 challenge.  polys: d x 2^n base-field values, on the
 * device (d_polys, left unchanged) or on the host (h_polys; the other must be NULL).
 * Outputs (host, canonical): h_msgs[n][d+1][2], h_challenges[n][2], h_finals[d][2],
 * h_final_eval[2].  Synchronising. */
int gb_sumcheck_prove_ext2(gb_transcript *t, int n, int d, const uint64_t *d_polys, const uint64_t *h_polys,
                           uint64_t *h_msgs, uint64_t *h_challenges, uint64_t *h_finals, uint64_t *h_final_eval);
/* CpuLinearSumcheckProverExt2::{new, prove} semantics (zk-torch-3/src/sumcheck/cpu_ext2_prover.rs:21-110):
 * as gb_sumcheck_prove_ext2 but the polynomials are Ext2, [d][2^n][c0, c1]. */
int gb_sumcheck_prove_ext2_polys(gb_transcript *t, int n, int d, const uint64_t *d_polys, const uint64_t *h_polys,
                                 uint64_t *h_msgs, uint64_t *h_challenges, uint64_t *h_finals, uint64_t *h_final_eval);
/* One fused round as a device building block: fold d polynomials (base-field input when
 * in_base, element stride in_stride) with the Ext2 challenge (r0, r1) into d_out (Ext2,
 * stride out_stride), producing pairs_out output pairs per polynomial, and write the next
 * round's d+1 Ext2 message values (canonical) to d_msg.  d_work: zeroed workspace of
 * gb_sumcheck_round_workspace_words() words (left zeroed again).  Launch only. */
size_t gb_sumcheck_round_workspace_words(void);
int gb_sumcheck_fold_round_ext2(const uint64_t *d_in, int in_base, size_t in_stride, uint64_t *d_out,
                                size_t out_stride, int d, size_t pairs_out, uint64_t r0, uint64_t r1,
                                uint64_t *d_msg, uint64_t *d_work);
/* LinearSumcheckProver::{new, prove} semantics (zk-torch-3/src/sumcheck/linear_prover.rs:23-63):
 * base-field messages and challenges.  h_msgs[n][d+1], h_challenges[n], h_finals[d], h_final_eval[1]. */
int gb_sumcheck_prove_base(gb_transcript *t, int n, int d, const uint64_t *d_polys, const uint64_t *h_polys,
                           uint64_t *h_msgs, uint64_t *h_challenges, uint64_t *h_finals, uint64_t *h_final_eval);

/* Basefold folding table: BasefoldTable::generate + upload (goldilocks-cuda-rs/src/basefold.rs:281-333).
 * The xorshift draws run on the host, the 2^(n+lr) inversions on the device.  Synchronising. */
int gb_basefold_table_create(int num_vars, int log_rate, int num_rounds, uint64_t seed, void **handle);
int gb_basefold_table_destroy(void *handle);
/* device pointer to the (point, weight) entries and the per-level entry offsets (num_rounds of them) */
int gb_basefold_table_info(void *handle, uint64_t **d_entries, uint64_t *h_level_offsets);

/* BasefoldCommitment::commit / commit_device (basefold.rs:382-427): evaluations (natural order,
 * variable i <-> bit i) on the device or the host; the codeword, its Merkle tree and the
 * evaluations stay device-resident in the returned handle.  root: canonical.  Synchronising. */
int gb_basefold_commit(const uint64_t *d_evals, const uint64_t *h_evals, int num_vars, int log_rate, void **handle,
                       uint64_t root[4]);
int gb_basefold_commitment_destroy(void *handle);
int gb_basefold_commitment_info(void *handle, uint64_t **d_codeword, uint64_t **d_tree, uint64_t **d_evals,
                                uint64_t root[4]);

/* Number of u64 in a flat open_ext2 proof: eval[2], oracles[n][3][2], folded_roots[n-1][4],
 * final_codeword[2^lr][2], then per query: index, values[n][2][2], auth paths of depths
 * n+lr-1, n+lr-2, ..., lr (4 u64 per digest) -- BasefoldProofExt2 (basefold.rs:124-132) flattened. */
size_t gb_basefold_proof_len(int num_vars, int log_rate, int num_queries);
/* BasefoldCommitment::open_ext2 (basefold.rs:578-870) with the zk-torch-3 transcript
 * (BasefoldTranscript for Transcript, zk-torch-3/src/transcript.rs:331-350).  h_point: n Ext2
 * values.  h_proof: gb_basefold_proof_len words, canonical.  Synchronising. */
int gb_basefold_open_ext2(void *commitment, void *table, const uint64_t *h_point, gb_transcript *t,
                          int num_queries, uint64_t *h_proof);

/* batch_open_ext2 (goldilocks-cuda-rs/src/basefold.rs:1202-1532; BatchBasefoldProofExt2,
 * :192-210): num_commitments commitments of equal num_vars and log_rate, opened at num_points
 * Ext2 points (h_points: num_points x num_vars Ext2).  Evaluation i claims that polynomial
 * eval_poly[i] at point eval_point[i] equals h_eval_values[2i..2i+1]; its transcript absorbs every
 * root, point and claim, as the reference does.  h_proof (gb_basefold_batch_proof_len words,
 * canonical): outer oracles [n][3][2] | combined root [4] | inner eval [2] | inner oracles
 * [n][3][2] | folded roots [n-1][4] | final codeword [2^lr][2] | num_queries combined queries in
 * the gb_basefold_open_ext2 query layout (round-0 values Ext2) | num_queries x num_evals
 * individual queries (base pair [2] + path [n+lr-1][4]).  Returns 0 or GB_EINVAL (empty input,
 * unequal shapes, an index out of range, a table that does not cover the commitments).
 * Synchronising. */
size_t gb_basefold_batch_proof_len(int num_vars, int log_rate, int num_queries, int num_evals);
int gb_basefold_batch_open_ext2(void *const *commitments, int num_commitments, const uint64_t *h_points,
                                int num_points, const int *eval_poly, const int *eval_point,
                                const uint64_t *h_eval_values, int num_evals, void *table, gb_transcript *t,
                                int num_queries, uint64_t *h_proof);

/* ---- Batched and served proving (no reference counterpart) ----
 * An instance is `degree` multilinear polynomials of 2^num_vars base-field values, proven by
 * (1) Basefold commit of each (log_rate 1), (2) the product sumcheck with Ext2 challenges on
 * Transcript::new("sumcheck") + append_ext2("", master_seed) + append_u64("", index) + the
 * roots' words (append_u64("", w) each), (3) open_ext2 of each polynomial j at the sumcheck
 * point on Transcript::new("bf-open") + append_ext2("", master_seed) + append_u64("", 8 index + j)
 * (the per-opening transcript of zk-torch-3/src/dag/mod.rs:1128-1133).
 * Proof (gb_instance_proof_len words, canonical): roots[d][4], msgs[n][d+1][2],
 * challenges[n][2], finals[d][2], final_eval[2], then d open proofs of
 * gb_basefold_proof_len(n, 1, num_queries) words.  2 <= num_vars <= 30, 1 <= degree <= 8. */
typedef struct gb_instance {
    int num_vars;
    int degree;
    uint64_t index;
    const uint64_t *h_polys; /* degree x 2^num_vars values on the host, or NULL */
    const uint64_t *d_polys; /* ... on the device (16-byte aligned), or NULL */
    uint64_t *h_proof;       /* output (host) */
} gb_instance;

typedef struct gb_job_stats {
    double queued_ms;  /* submit -> start */
    double run_ms;     /* start -> finish */
    double latency_ms; /* submit -> finish */
} gb_job_stats;

size_t gb_instance_proof_len(int num_vars, int degree, int num_queries);
/* Estimated peak device bytes of one instance (the admission charge). */
size_t gb_instance_hbm_bytes(int num_vars, int degree);
/* One instance on the calling thread's stream (the per-call path).  table: a
 * gb_basefold_table_create handle with log_rate 1 covering num_vars.  Synchronising. */
int gb_prove_instance(void *table, const uint64_t master_seed[2], int num_queries, const gb_instance *inst);

/* Prover service: `workers` host threads, each launching on a stream of its own, admit
 * submitted instances in arrival order as their estimated footprint fits in hbm_budget
 * bytes beside the running ones (a job larger than the budget runs alone).  The instance's
 * host buffers must stay valid until gb_prover_wait returns for its ticket. */
int gb_prover_create(void *table, const uint64_t master_seed[2], int num_queries, int workers, size_t hbm_budget,
                     void **handle);
/* The continuous prover service (no reference counterpart): `workers` threads run each admitted
 * job's steps before its openings (inputs, commits, sumcheck, partial evaluations, Ajtai) on their
 * own streams, then hand its openings to open engines, one per size class of opening (n < 19,
 * 19 <= n < 22, n >= 22), each a thread with a stream that keeps every opening of its class in
 * flight and advances all of them one round per step: each round's work of all of them in one
 * launch per kernel kind (and one per Merkle layer).  Openings join at their engine's next step
 * once their job's prologue is done, and leave when their queries are gathered; the job is then
 * complete and its budget share is freed.  A worker takes the next admitted job as soon as it has
 * handed over the last one, so admission follows the HBM budget alone.  Proofs are identical to
 * the per-call path's.  Same submit / wait / drain / destroy calls; table: log_rate 1. */
int gb_prover_create_continuous(void *table, const uint64_t master_seed[2], int num_queries, int workers,
                                size_t hbm_budget, void **handle);
/* Job slots (no reference counterpart): at most `slots` jobs are admitted and not yet complete at
 * a time, beside the HBM budget; 0 (the default) lifts the limit.  In the continuous service the
 * workers hand a job's openings over and take the next job at once, so without slots only the
 * budget bounds the jobs sharing the device: the most throughput, each job finishing later.
 * Fewer slots trade throughput for latency.  The whole-job service is bounded by its workers. */
int gb_prover_set_slots(void *prover, int slots);
/* Jobs admitted and not yet complete (either service), -1 for a null handle. */
int gb_prover_running(void *prover);
/* Openings in the continuous service's open engines (waiting to join or in flight); 0 for the
 * whole-job service. */
size_t gb_prover_openings_in_flight(void *prover);
int gb_prover_submit(void *prover, const gb_instance *inst, uint64_t *ticket); /* non-blocking */
/* Blocks until the ticket's job is done; returns the job's return code (its message in
 * gb_last_error()); stats may be NULL.  Each ticket is waited for once. */
int gb_prover_wait(void *prover, uint64_t ticket, gb_job_stats *stats);
int gb_prover_drain(void *prover); /* blocks until no job is queued or running */
/* Merkle cooperative threshold the service's workers use (see gb_set_coop_threshold); the
 * service starts with its creating thread's value. */
int gb_prover_set_coop_threshold(void *prover, size_t parents);
int gb_prover_set_merkle_top_nodes(void *prover, size_t nodes); /* see gb_set_merkle_top_nodes */
int gb_prover_destroy(void *prover);
/* All instances through a prover service of `workers` threads, largest first; returns the
 * first non-zero job return code.  Synchronising. */
int gb_batch_prove(void *table, const uint64_t master_seed[2], int num_queries, const gb_instance *insts, int count,
                   int workers, size_t hbm_budget);

/* The same batch as gb_batch_prove, round-synchronously: the commits of all polynomials, then
 * every round of every instance's product sumcheck as one launch per degree, then every round
 * of every polynomial's opening as one launch per step for all polynomials (and one per Merkle
 * layer), with one host round trip per round; the host steps of the per-instance transcripts
 * run on up to 16 threads.  `workers` must be >= 1 and is otherwise unused by this engine.
 * Instances that do not fit hbm_budget together run in waves, largest first.  Proofs are
 * identical to gb_prove_instance's.  table: log_rate 1.  Synchronising. */
int gb_batch_prove_lockstep(void *table, const uint64_t master_seed[2], int num_queries, const gb_instance *insts,
                            int count, int workers, size_t hbm_budget);
/* Host wall time of the calling thread's last gb_batch_prove_lockstep: the commit + sumcheck
 * phase, the opening phase and the sumcheck part of the first, summed over its waves (any
 * pointer may be NULL). */
void gb_lockstep_last_timing(double *commit_sumcheck_ms, double *open_ms, double *sumcheck_ms);
/* Schedule of the calling thread's gb_batch_prove_lockstep calls (no reference counterpart; the
 * autotuner's knobs, results never depend on them): a wave's instances are dealt out in size
 * order to `groups` staggered groups (group k + 1's commits start once group k's are done, each
 * group on its own stream and host thread), and each group's polynomials to `open_parts` parts
 * opened side by side on their own streams.  Both in [1, 8], else -2.  Default 2 and 2. */
int gb_set_lockstep_schedule(int groups, int open_parts);
void gb_get_lockstep_schedule(int *groups, int *open_parts);

/* A quantized matmul layer C = A B as a served job (no reference counterpart; the field work
 * of zk-torch-3/src/basicblock/einsum.rs:807-1000): A is m x k, B is k x n (row-major int8),
 * m, n, k powers of two with m k >= 2^16.  The proof (gb_matmul_proof_len words, canonical):
 * roots of A and B [2][4], claim C~(r_i, r_j) [2], sumcheck over the log k variables of the
 * inner index: msgs[log k][3][2], challenges r_k[log k][2], finals [2][2], final_eval [2]; then
 * open_ext2 proofs of A at (r_k, r_i) and of B at (r_j, r_k) (log_rate 1); then the Ajtai
 * commitment [16][64] of the first 2^16 entries of A as bytes v + 128 under the attached key.
 * r_i, r_j are Ext2 challenges of Transcript::new("matmul") + append_ext2("", master_seed) +
 * append_u64("", index), ("", m), ("", n), ("", k), the 8 root words ("" each); the sumcheck
 * continues on that transcript; the openings use "bf-open" transcripts with 8 index + 0 / 1. */
typedef struct gb_matmul_job {
    int m, n, k;
    uint64_t index;
    const int8_t *h_a; /* m x k (host) */
    const int8_t *h_b; /* k x n (host) */
    uint64_t *h_proof; /* output (host) */
} gb_matmul_job;

size_t gb_matmul_proof_len(int m, int n, int k, int num_queries);
size_t gb_matmul_hbm_bytes(int m, int n, int k);
/* One matmul job on the calling thread's stream.  table: log_rate 1, covering log(m k) and
 * log(k n) variables; ajtai_key: a gb_ajtai_key_create handle of 16 rows over 1024 ring columns.
 * Synchronising. */
int gb_prove_matmul(void *table, void *ajtai_key, const uint64_t master_seed[2], int num_queries,
                    const gb_matmul_job *job);
/* Attach the Ajtai key used by the service's matmul jobs (before submitting any). */
int gb_prover_set_ajtai_key(void *prover, void *ajtai_key);
int gb_prover_submit_matmul(void *prover, const gb_matmul_job *job, uint64_t *ticket); /* non-blocking */

/* ===================== Part 1 (continued): reference ABI =====================
 * Partial evaluation and bit permutation (the einsum input preparation). */
/* partial_eval_gl_ffi (ffi.rs:377-382, wrapper.cu:1166-1184): fix the low m of log_n variables of
 * d_data (2^log_n base values) at the m base values d_r, LSB first; the 2^(log_n-m) results replace
 * the front of d_data (canonical).  m <= 0 does nothing.  Scratch comes from the stream's pool. */
int partial_eval_gl_ffi(uint64_t *d_data, const uint64_t *d_r, int log_n, int m);
/* partial_eval_ext2_from_gl_ffi (ffi.rs:384-390, wrapper.cu:1186-1210): the same at m Ext2 values
 * d_r; d_output (room for 2^(log_n-1) Ext2) receives the 2^(log_n-m) Ext2 results at its front. */
int partial_eval_ext2_from_gl_ffi(const uint64_t *d_input, uint64_t *d_output, const uint64_t *d_r, int log_n, int m);
/* bit_permute_gl_ffi (ffi.rs:644-650, wrapper.cu:1824-1851): d_output[new] = d_input[old] with old
 * bit d_perm_map[k] taken from new bit k (the inverse permutation, as field.rs:195-224 passes it);
 * total = 2^n_bits.  Returns -2 for a map that is not a permutation.  Synchronising (the map is
 * read on the host to plan the tiles). */
int bit_permute_gl_ffi(const uint64_t *d_input, uint64_t *d_output, const int *d_perm_map, int n_bits, int total);
/* fused_permute_partial_eval_ffi (ffi.rs:657-668, wrapper.cu:1857-1885, fused_permute_peval.cuh):
 * d_output[j] = sum_{b < 2^m} d_evals[lo_lut[i & (2^half - 1)] | hi_lut[i >> half]] * d_eq_table[b],
 * i = j 2^m + b, for j < output_size <= 2^(n-m); d_eq_table holds 2^m Ext2 values, d_output
 * output_size Ext2 (canonical).  smem_bytes is accepted and unused (the LUTs are read through the
 * cache).  Asynchronous like the reference. */
int fused_permute_partial_eval_ffi(const uint64_t *d_evals, uint64_t *d_output, const uint64_t *d_eq_table,
                                   const uint32_t *d_lo_lut, const uint32_t *d_hi_lut, int n, int m, int half,
                                   int output_size, int smem_bytes);

#ifdef __cplusplus
}
#endif
#endif
