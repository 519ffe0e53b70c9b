/*
 * almost_goldilocks_cuda_wrapper.h -- C ABI of the GB300-native almost-Goldilocks part
 * (q = 2^64 - 2^32 - 31) of the prover library: the Ajtai commitment.
 *
 * Part 1 is a drop-in for the entry points of almost-goldilocks-cuda-rs on this path
 * (almost-goldilocks-cuda-rs/src/ffi.rs, implemented by almost-goldilocks-cuda-rs/cuda/wrapper.cu),
 * with the same names, argument meaning and return codes.  The memory entry points
 * (cuda_malloc, ...) are shared with goldilocks_cuda_wrapper.h.
 *
 * Part 2 (gb_*) is the batched tensor-core commitment, which has no reference counterpart.
 */
#ifndef ALMOST_GOLDILOCKS_CUDA_WRAPPER_H
#define ALMOST_GOLDILOCKS_CUDA_WRAPPER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ===================== Part 1: reference ABI ===================== */

/* almost-goldilocks-cuda-rs/src/ffi.rs:13 (wrapper.cu init): selects device 0. */
int almost_goldilocks_cuda_init(void);

/* Ajtai commitment of a full-width witness (ajtai_commit_wide_ffi, almost wrapper.cu:1188-1205;
 * Rust API commit_wide, almost-goldilocks-cuda-rs/src/ajtai.rs:299-344):
 *   d_key   8 u32 ChaCha8 key (device)
 *   d_z_wide N ring elements x 64 canonical coefficients (device), column-major [j][coefficient]
 *   col_offset first matrix column used (ring elements)
 *   chunk   the reference's column-chunk tuning knob: 64, 128, 256, 1024 or 4096 (-3 otherwise);
 *           the result does not depend on it
 *   d_out   KAPPA = 42 rows x 64 canonical coefficients (device).  Synchronising. */
int ajtai_commit_wide_ffi(const uint32_t *d_key, const uint64_t *d_z_wide, uint64_t N, uint64_t col_offset, int chunk,
                          uint64_t *d_out);

/* Binary witnesses, batched (commit_dense_batched_kernel, cuda_almost_goldilocks/ajtai.cuh:82-162;
 * almost wrapper.cu:1139-1170): d_z is [B][N] u64 bitmasks (bit l of word (b, j) = coefficient l
 * of ring element j of witness b); d_out is [B][KAPPA][64] canonical.  1 <= B <= 16 (-2
 * otherwise); chunk as for ajtai_commit_wide_ffi.  The _at form uses matrix columns from
 * col_offset.  Synchronising. */
int ajtai_commit_dense_batched_ffi(const uint32_t *d_key, const uint64_t *d_z, uint64_t N, int B, int chunk,
                                   uint64_t *d_out);
int ajtai_commit_dense_batched_at_ffi(const uint32_t *d_key, const uint64_t *d_z, uint64_t N, int B, int chunk,
                                      uint64_t col_offset, uint64_t *d_out);
/* Ternary witnesses of a split (commit_ternary_kernel, ajtai.cuh:1262-1370; almost
 * wrapper.cu:1642-1660): 13 witnesses, coefficient l of ring element j of witness i is bit l of
 * d_pos[i N_ring + j] minus bit l of d_neg[i N_ring + j]; d_out [13][KAPPA][64].  Synchronising. */
int ajtai_commit_ternary_ffi(const uint32_t *d_key, const uint64_t *d_pos, const uint64_t *d_neg, uint64_t N_ring,
                             int chunk, uint64_t *d_out);
/* ajtai_materialize_m_ffi (ajtai_premat.cuh:35-85, almost wrapper.cu:1662-1670): d_M[j][i][0..63] =
 * M_{i,j} for j < N, i < KAPPA (7680 N bytes).  ajtai_commit_ternary_premat_ffi: the ternary commit
 * reading that matrix instead of generating it (same result as ajtai_commit_ternary_ffi).
 * The commit is synchronising. */
int ajtai_materialize_m_ffi(const uint32_t *d_chacha_key, uint64_t *d_M, uint64_t N);
int ajtai_commit_ternary_premat_ffi(const uint64_t *d_M, const uint64_t *d_pos, const uint64_t *d_neg, uint64_t N_ring,
                                    int chunk, uint64_t *d_out);

/* ---- Fold tree (ajtai.cuh:700-1260; almost wrapper.cu:1468-1620, :1717-1740).  r: 64 int8
 * challenge coefficients; r . z is the product in R_q = F_q[X]/(X^64 + 1).  Witnesses are u64
 * bitmasks per ring element ([instance][N_ring]); ternary ones are (pos, neg) pairs. ---- */
/* out[j] = z1[j] + r . z2[j], canonical F_q [N_ring][64]; r_coeffs on the host; chunk as the
 * other commits (-3 otherwise). */
int ajtai_fold_witness_ffi(const uint64_t *d_z1, const uint64_t *d_z2, const int8_t *r_coeffs, uint64_t N_ring,
                           int chunk, uint64_t *d_out);
/* out[j] = sum_i r_i . z_i[j] as int16 [N_ring][64] (the int32 sum cast to int16); d_r_all
 * [num_instances][64] on the device.  chunk_size only has to be nonzero. */
int ajtai_multifold_witness_ffi(const uint64_t *d_z_packed, const int8_t *d_r_all, int16_t *d_out, int num_instances,
                                uint64_t N_ring, uint64_t chunk_size);
/* binary instances then ternary ones: r_all [(num_binary + num_ternary)][64] */
int ajtai_multifold_mixed_witness_ffi(const uint64_t *d_z_bin_packed, const uint64_t *d_pos_packed,
                                      const uint64_t *d_neg_packed, const int8_t *d_r_all, int16_t *d_out,
                                      int num_binary, int num_ternary, uint64_t N_ring, uint64_t chunk_size);
/* The reference's tensor-core forms of the mixed fold (same result); here all three run the
 * plane-popcount kernel. */
int ajtai_multifold_mixed_witness_tc_ffi(const uint64_t *d_z_bin_packed, const uint64_t *d_pos_packed,
                                         const uint64_t *d_neg_packed, const int8_t *d_r_all, int16_t *d_out,
                                         int num_binary, int num_ternary, uint64_t N_ring);
int ajtai_multifold_mixed_witness_tc_fused_ffi(const uint64_t *d_z_bin_packed, const uint64_t *d_pos_packed,
                                               const uint64_t *d_neg_packed, const int8_t *d_r_all, int16_t *d_out,
                                               int num_binary, int num_ternary, uint64_t N_ring);
/* int16 witness [N_ring][64] -> 13 ternary chunks: v = sum_i 2^i (pos_i - neg_i), bits of |v|
 * routed by sign; d_pos_chunks / d_neg_chunks [13][N_ring]. */
int ajtai_split_witness_ffi(const int16_t *d_z_wide, uint64_t *d_pos_chunks, uint64_t *d_neg_chunks, uint64_t N_ring);
/* c = sum_i r_i . c_i over [KAPPA][64] rows (d_c_packed [num_instances][KAPPA][64], d_r_all on
 * the device); fold: c1 + r . c2 with r_coeffs on the host.  Canonical outputs. */
int ajtai_multifold_commitment_ffi(const uint64_t *d_c_packed, const int8_t *d_r_all, int num_instances,
                                   uint64_t *d_out);
int ajtai_fold_commitment_ffi(const uint64_t *d_c1, const uint64_t *d_c2, const int8_t *r_coeffs, uint64_t *d_out);
/* Sparse binary witness (commit_sparse_partial_kernel, ajtai.cuh:382-440; almost wrapper.cu:1741-1756):
 * d_positions holds K coefficient indices 64 j + l with value 1 (a repeated index counts once
 * per occurrence); d_out [KAPPA][64].  Synchronising. */
int ajtai_commit_sparse_ffi(const uint32_t *d_key, const uint64_t *d_positions, uint64_t K, int chunk,
                            uint64_t *d_out);

/* ---- memory and streams (almost-goldilocks-cuda-rs/src/ffi.rs:77-100, almost wrapper.cu:255-411);
 * cuda_malloc, cuda_free, cuda_memcpy_{htod,dtoh,dtod}, cuda_pool_trim, cuda_device_synchronize,
 * cuda_get/peek_last_error, cuda_mem_get_info and the device calls are the shared ones of
 * goldilocks_cuda_wrapper.h. */
const char *agl_cuda_error_string(int code);
int cuda_memset(void *dst, int value, size_t size);
/* Waits for this thread's launch stream ("my kernels are done"). */
int cuda_sync_mine(void);
int cuda_stream_create(void **stream);
int cuda_stream_destroy(void *stream);
int cuda_stream_synchronize(void *stream);
int cuda_memcpy_dtod_async(void *dst, const void *src, size_t size, void *stream);
int cuda_memcpy_htod_async(void *dst, const void *src, size_t size, void *stream);
/* Device memory the stream-ordered pool of the current device holds (reserved, in use or not). */
size_t agl_cached_bytes(void);
/* High-water mark of the memory in use from that pool since the last reset (no counterpart in the
 * reference).  reset != 0 then restarts the mark from the memory in use now.  (size_t)-1 on error. */
size_t gb_pool_used_high(int reset);
/* Synchronous copies through pinned staging (any host memory). */
int agl_d2h_staged(void *h_dst, const void *d_src, size_t bytes);
int agl_h2d_staged(void *d_dst, const void *h_src, size_t bytes);

/* ---- almost-Goldilocks sumcheck (cuda_almost_goldilocks/almost_sumcheck_prover.cuh:24-225):
 * d polynomials at stride original_size (Ext2: [poly][original_size][2]); round k uses pairs
 * (2y, 2y + 1), y < half.  The message entry points write per-block partial sums
 * d_partial[block][c] (Ext2: [block][c][2]), c = 0..d, for num_blocks blocks of 256 threads
 * over a grid-stride loop (the caller adds them up mod q); the folds write
 * p_i[y] = p_i[2y] + r (p_i[2y+1] - p_i[2y]) at the same stride.  Launch only; 1 <= d <= 8. */
int agl_sumcheck_round_message_ffi(const uint64_t *d_polys, uint64_t *d_partial, int d, size_t original_size,
                                   size_t half, int num_blocks);
int agl_sumcheck_fold_ffi(const uint64_t *d_input, uint64_t *d_output, uint64_t challenge, int d,
                          size_t original_size, size_t half);
int aext2_sumcheck_round_message_ffi(const uint64_t *d_polys, uint64_t *d_partial, int d, size_t original_size,
                                     size_t half, int num_blocks);
int aext2_sumcheck_fold_ffi(const uint64_t *d_input, uint64_t *d_output, uint64_t challenge_c0,
                            uint64_t challenge_c1, int d, size_t original_size, size_t half);
/* Batched same-point degree-2 sumcheck (almost_sumcheck_prover.cuh:220-368): per leaf the pair
 * (eq, f) of original_size Ext2 values each, leaf l at d_polys + 4 l original_size; partials
 * [block_x][leaf][c][2], c = 0, 1, 2, grid (num_blocks_x, num_leaves).  Launch only. */
int aext2_sumcheck_batched_round_message_ffi(const uint64_t *d_polys, uint64_t *d_partial, size_t original_size,
                                             size_t half, int num_leaves, int num_blocks_x);
int aext2_sumcheck_batched_fold_ffi(const uint64_t *d_input, uint64_t *d_output, uint64_t challenge_c0,
                                    uint64_t challenge_c1, size_t original_size, size_t half, int num_leaves);

/* ---- eq tables (almost_eq_lagrange.cuh:23-219): eq(r, x), variable i <-> bit i of x.  As with
 * the reference's ping-pong DP the table ends in d_buf_a when log_n is even and in d_buf_b when
 * it is odd; *d_result is set to that buffer, the other one is scratch.  The batched form takes
 * num_leaves points [leaf][log_n] and buffers of num_leaves x leaf_stride entries. */
int agl_eq_dp_all_ffi(const uint64_t *d_r, uint64_t *d_buf_a, uint64_t *d_buf_b, int log_n, uint64_t **d_result);
int aext2_eq_dp_all_ffi(const uint64_t *d_r, uint64_t *d_buf_a, uint64_t *d_buf_b, int log_n, uint64_t **d_result);
int aext2_eq_dp_all_stream_ffi(const uint64_t *d_r, uint64_t *d_buf_a, uint64_t *d_buf_b, int log_n,
                               uint64_t **d_result, void *stream);
int aext2_eq_dp_all_batched_ffi(const uint64_t *d_r_all, uint64_t *d_buf_a_all, uint64_t *d_buf_b_all, int log_n,
                                int num_leaves, size_t leaf_stride, uint64_t **d_result, void *stream);

/* ===================== Part 2: GB300 additions (no reference counterpart) ===================== */

/* Matrix rows [row_lo, row_lo + rows) over n_ring ring columns of the ChaCha8 key h_seed, with
 * the device-resident operands of the tensor-core commitments: the 8 bf16 digit planes
 * (ceil(rows / 16) * 128 * roundup(64 n_ring, 1024) * 2 bytes, 16 MB for 16 rows x 1024 columns),
 * built here; their Hankel windows (4 * rows * roundup(n_ring, 16) * 3840 bytes, 252 MB), built
 * by the first gb_ajtai_commit_u8_batched call that takes the Hankel form; and their negacyclic
 * expansion (8 * rows * 64 * roundup(64 n_ring, 1024) * 2 bytes, 1.07 GB), built only by a call
 * that takes a key-Toeplitz form (such a first call synchronises for the build; concurrent callers
 * wait for the one build).  Synchronising. */
int gb_ajtai_key_create(const uint32_t *h_seed, int row_lo, int rows, uint64_t n_ring, void **handle);
int gb_ajtai_key_destroy(void *handle);
/* The key's first row, row count and ring columns (any output pointer may be NULL). */
int gb_ajtai_key_info(void *handle, int *row_lo, int *rows, uint64_t *n_ring);
/* Commit num_witnesses witnesses with coefficients in [0, 256): d_z is [num_witnesses][n_ring * 64]
 * bytes (device); d_out is [num_witnesses][rows][64] canonical u64 (device).  Rows are those of
 * the key; the result equals ajtai_commit_wide_ffi restricted to those rows.  Synchronising. */
int gb_ajtai_commit_u8_batched(void *key, const uint8_t *d_z, int num_witnesses, uint64_t *d_out);
/* Form of the calling thread's gb_ajtai_commit_u8_batched calls (no reference counterpart):
 * 0 chooses by batch size (the default), 1 the witness-circulant tensor-core GEMM (work
 * proportional to the batch; the automatic choice up to 104 witnesses), 2 the key-Toeplitz
 * tensor-core GEMM (streams the key's 1.07 GB expansion once per batch of up to 256 witnesses),
 * 3 the key-Toeplitz GEMM on CTA pairs (clusters of two CTAs, M = 256 tcgen05 MMAs), 4 the
 * same CTA-pair GEMM reading the key's Hankel windows instead of its expansion (252 MB for 16 rows
 * x 1024 ring columns, built on first use; the automatic choice above 104 witnesses, or form 2
 * where the device cannot run the pairs).  Results never depend on it.  Returns the previous
 * form, or -2 for a form outside 0..4. */
int gb_ajtai_set_batch_form(int form);
/* Test switch of the calling thread for the GEMM's bounded waits: with on != 0 the following
 * gb_ajtai_commit_u8_batched calls launch the tensor-core GEMM with its operand loads left out and
 * short wait limits, so that its pipeline waits run out; the call then returns -1 with
 * "pipeline wait timed out (code N)" in gb_last_error(), with no load in flight and TMEM
 * released.  Returns the previous setting. */
int gb_ajtai_test_starve(int on);

/* ajtai_commit_wide_ffi without any device allocation (no counterpart in the reference).
 * Same arguments, result and return codes as ajtai_commit_wide_ffi, whose every call
 * allocates and frees its per-column-chunk partial sums.  This variant keeps them in a
 * static device array of the library sized for N <= 4096 ring elements (5.25 MiB); a larger
 * N returns -2 with a message in gb_last_error().  It is for callers that must not allocate
 * on their request path: a service that has reserved its whole HBM budget up front, where an
 * allocation inside the call could fail or wait on the memory pool.
 *   - Every call looks the scratch address up on the current device (cudaGetSymbolAddress).
 *     The first call on each device is a warm-up: with lazy module loading it may load the
 *     library's module and map its static device memory, this array included.  Make that call
 *     before reserving the HBM budget, before serving starts and before any stream capture;
 *     from the second call on nothing is allocated.
 *   - Calls share the one scratch: calls that overlap in time (other threads, other streams)
 *     race on it and must be serialised by the caller.
 *   - Nothing in the scratch needs clearing: every word read is written by the same call.
 * Synchronising. */
int ajtai_commit_wide_noalloc_ffi(const uint32_t *d_key, const uint64_t *d_z_wide, uint64_t N, uint64_t col_offset,
                                  int chunk, uint64_t *d_out);

/* ---- Binary round 0 and lifts of the batched same-point sumcheck (almost-goldilocks-cuda-rs
 * GpuBatchedSamePointState, src/sumcheck_prover.rs:468-1006; almost_sumcheck_prover.cuh:709-1005;
 * almost wrapper.cu:862-1060).  Layout as aext2_sumcheck_batched_*: leaf l's eq then f, each
 * original_size Ext2, at d_polys + 4 l original_size; bit i of leaf l's binary f is bit i % 64 of
 * d_packed[l packed_size_u64 + i / 64].  Same grid shapes as the reference (partials
 * [num_blocks_x][leaf][c][2]). ---- */
/* round 0 with f binary: c = 0: sum e0 f0, c = 1: sum e1 f1, c = 2: sum (2 e1 - e0)(2 f1 - f0) */
int aext2_sumcheck_batched_round0_binary_msg_ffi(const uint64_t *d_polys, const uint64_t *d_packed,
                                                 uint64_t *d_partial, size_t original_size, size_t half,
                                                 int num_leaves, int num_blocks_x, size_t packed_size_u64);
/* the fold of that round: eq and the lifted f folded with the challenge into d_output (same layout) */
int aext2_sumcheck_batched_round0_binary_fold_ffi(const uint64_t *d_polys, const uint64_t *d_packed,
                                                  uint64_t *d_output, uint64_t challenge_c0, uint64_t challenge_c1,
                                                  size_t original_size, size_t half, int num_leaves,
                                                  size_t packed_size_u64);
/* lift binary (or ternary pos - neg) bits into the f slot of each leaf, Ext2 (bit, 0) */
int aext2_batched_lift_binary_ffi(const uint64_t *d_packed, uint64_t *d_polys, size_t original_size, int num_leaves,
                                  size_t packed_size_u64);
int aext2_batched_lift_ternary_single_ffi(const uint64_t *d_pos, const uint64_t *d_neg, uint64_t *d_polys,
                                          size_t original_size, int num_leaves, size_t packed_size_u64);
/* the same into a contiguous [leaf][original_size] Ext2 array */
int aext2_lift_binary_contig_ffi(const uint64_t *d_packed, uint64_t *d_f, size_t original_size, int num_leaves,
                                 size_t packed_size_u64);
/* per-(block, plane) partial sums of the shared eq table over each plane's set bits
 * (almost_sumcheck_prover.cuh:920-970; almost-goldilocks-cuda-rs/src/eq_lagrange.rs) */
int aext2_selective_add_batched_planes_ffi(const uint64_t *d_eq, const uint64_t *d_packed_planes, uint64_t *d_partial,
                                           size_t total, int n_planes, size_t packed_size_u64, int num_blocks_x);

/* ---- The fold tree's other sumcheck provers (almost-goldilocks-cuda-rs/src/sumcheck_prover.rs,
 * ffi.rs:141-160, :319-400; almost_sumcheck_prover.cuh:360-700; almost wrapper.cu:931-1028,
 * :2652-2980).  Same launch shapes as the reference (partials per (block, unique / leaf / term)).
 * ---- */
/* F_u[x] = sum over leaves d_leaf_idx_sorted[d_unique_offsets[u] .. d_unique_offsets[u+1]) of
 * alpha_leaf * bit (binary) or * (pos bit - neg bit) (ternary); d_Fu [num_unique][original_size] Ext2 */
int aext2_build_fu_ffi(const uint64_t *d_packed, const uint64_t *d_alphas, const int *d_leaf_idx_sorted,
                       const int *d_unique_offsets, uint64_t *d_Fu, size_t original_size, int num_unique,
                       size_t packed_size_u64);
int aext2_build_fu_ternary_ffi(const uint64_t *d_pos, const uint64_t *d_neg, const uint64_t *d_alphas,
                               const int *d_leaf_idx_sorted, const int *d_unique_offsets, uint64_t *d_Fu,
                               size_t original_size, int num_unique, size_t packed_size_u64);
/* i16 witness [n_ring][64] -> k_chunks signed bit planes [k][n_ring] (pos, neg); *d_err = 1 when
 * some |v| >= 2^k_chunks; k_chunks > 16 returns -1 */
int aext2_wide_to_ternary_ffi(const int16_t *d_wide, uint64_t *d_pos, uint64_t *d_neg, int *d_err, size_t n_ring,
                              int k_chunks);
/* all suffix tables eqsuf_t (t = log_n .. 1) of each unique point's r (d_r_all [u][log_n] Ext2):
 * eqsuf_t at element offset 2^(log_n-t) - 1 of the unique's region (stride eqsuf_stride_u64 words) */
int aext2_eq_suffix_dp_ffi(const uint64_t *d_r_all, uint64_t *d_eqsuf, int log_n, int num_unique,
                           size_t eqsuf_stride_u64);
/* partials [block][u][A, B]: A = sum_y eqsuf[y] F_u[2y], B = sum_y eqsuf[y] F_u[2y+1] */
int aext2_sharedeq_factored_msg_ffi(const uint64_t *d_eqsuf, const uint64_t *d_fu, uint64_t *d_partial,
                                    size_t eqsuf_off_elems, size_t eqsuf_stride_u64, size_t poly_stride_u64,
                                    size_t half, int num_unique, int num_blocks_x);
/* partials [block][leaf][c][2] of the degree-2 message of eq[leaf_to_unique[leaf]] * f[leaf] */
int aext2_sharedeq_msg_ffi(const uint64_t *d_eq, const uint64_t *d_f, const int *d_leaf_to_unique,
                           uint64_t *d_partial, size_t original_size, size_t half, int num_leaves, int num_blocks_x);
/* fold count independent Ext2 polynomials (stride original_size) by one challenge */
int aext2_fold_single_ffi(const uint64_t *d_in, uint64_t *d_out, uint64_t challenge_c0, uint64_t challenge_c1,
                          size_t original_size, size_t half, int count);
/* Sparse boolean check: n entries (d_idx, d_val Ext2) grouped into n_terms terms by d_term_off.
 * init: every value (1, 0).  round_msg: flags (first entry of each pair {2y, 2y+1}), their exclusive
 * scan into d_gid (d_scan_scratch: at least 4 ceil(n / 256) + 8 words), h_msg = the degree-3
 * message sum_t w_t v (v - 1) eq at 0..3 (4 Ext2, canonical), *h_total = number of pairs.
 * fold: each pair folded to position d_gid of d_out_idx / d_out_val, new term offsets.  finish:
 * d_out[t] = the value at position 0 of term t (or 0).  All synchronising. */
int agl_bool_init_val_ffi(uint64_t *d_val, size_t n);
int agl_bool_round_msg_ffi(const uint32_t *d_idx, const uint64_t *d_val, const uint32_t *d_term_off,
                           const uint64_t *d_w, const uint64_t *d_eq, int n_terms, size_t n, uint32_t *d_flags,
                           uint32_t *d_gid, uint64_t *d_partial, int grid_x, uint32_t *d_scan_scratch,
                           size_t scan_scratch_len, uint64_t *h_msg, uint32_t *h_total);
int agl_bool_fold_ffi(const uint32_t *d_idx, const uint64_t *d_val, const uint32_t *d_flags, const uint32_t *d_gid,
                      const uint32_t *d_term_off, int n_terms, size_t n, uint64_t r0, uint64_t r1, uint32_t total,
                      int grid_x, uint32_t *d_out_idx, uint64_t *d_out_val, uint32_t *d_new_off);
int agl_bool_finish_ffi(const uint32_t *d_idx, const uint64_t *d_val, const uint32_t *d_term_off, int n_terms, size_t n,
                        uint64_t *d_out);

/* ---- Runtime helpers (almost wrapper.cu:268-279, :327-328, :2989-2997, :3943-3958) ---- */
int cuda_memcpy_peer(void *dst, int dst_dev, const void *src, int src_dev, size_t size);
int cuda_enable_peer_access(int peer); /* 0 when enabled or already enabled, else -1 */
void agl_nvtx_push(const char *name);  /* NVTX profiler range */
void agl_nvtx_pop(void);
int agl_i64_to_i32(const int64_t *s, int32_t *d, uint64_t n);   /* d = (i32) s; synchronising */
int agl_add_i32_i64(int64_t *d, const int32_t *s, uint64_t n);  /* d += (i64) s; synchronising */
int agl_gauss_low_priority(int on); /* the calling thread's low-priority stream on or off */

/* ---- Element-wise ops over q and its Ext2 (almost-goldilocks-cuda-rs/src/ffi.rs:95-140;
 * almost wrapper.cu:420-640): canonical outputs, Ext2 = F_q[X]/(X^2 - 3) as (c0, c1), inverses of
 * zero are zero. ---- */
int agl_batch_add_ffi(const uint64_t *a, const uint64_t *b, uint64_t *r, int n);
int agl_batch_sub_ffi(const uint64_t *a, const uint64_t *b, uint64_t *r, int n);
int agl_batch_mul_ffi(const uint64_t *a, const uint64_t *b, uint64_t *r, int n);
int agl_batch_div_ffi(const uint64_t *a, const uint64_t *b, uint64_t *r, int n);
int agl_batch_inverse_ffi(const uint64_t *a, uint64_t *r, int n);
int agl_batch_mul_scalar_ffi(uint64_t scalar, const uint64_t *a, uint64_t *r, int n);
int agl_batch_neg_ffi(const uint64_t *a, uint64_t *r, int n);
int agl_batch_square_ffi(const uint64_t *a, uint64_t *r, int n);
int agl_batch_double_ffi(const uint64_t *a, uint64_t *r, int n);
int agl_batch_exp_ffi(const uint64_t *a, uint64_t exp, uint64_t *r, int n);
int aext2_batch_add_ffi(const uint64_t *a, const uint64_t *b, uint64_t *r, int n);
int aext2_batch_sub_ffi(const uint64_t *a, const uint64_t *b, uint64_t *r, int n);
int aext2_batch_mul_ffi(const uint64_t *a, const uint64_t *b, uint64_t *r, int n);
int aext2_batch_inverse_ffi(const uint64_t *a, uint64_t *r, int n);
int aext2_batch_mul_scalar_ffi(uint64_t scalar, const uint64_t *a, uint64_t *r, int n);
int aext2_batch_neg_ffi(const uint64_t *a, uint64_t *r, int n);
int aext2_batch_square_ffi(const uint64_t *a, uint64_t *r, int n);
int aext2_batch_frobenius_ffi(const uint64_t *a, uint64_t *r, int n);
int aext2_batch_conjugate_ffi(const uint64_t *a, uint64_t *r, int n);
int aext2_batch_exp_ffi(const uint64_t *a, uint64_t exp, uint64_t *r, int n);
int aext2_scale_accumulate_ffi(uint64_t scalar_c0, uint64_t scalar_c1, const uint64_t *d_src, uint64_t *d_acc, int n);
int agl_to_aext2_batch_ffi(const uint64_t *in, uint64_t *out, int n);
int aext2_to_agl_batch_ffi(const uint64_t *in, uint64_t *out, int n);
int agl_zero_buffer_ffi(uint64_t *d_buf, int n);

/* ---- Partial evaluation and bit permutation over q (almost-goldilocks-cuda-rs/src/ffi.rs:113-119,
 * :198-226; wrapper.cu:713-805, :1061-1085).  Same arguments and results as the Goldilocks forms
 * (goldilocks_cuda_wrapper.h), over q = 2^64 - 2^32 - 31 and its Ext2 (X^2 - 3). ---- */
int agl_partial_eval_ffi(uint64_t *d_data, const uint64_t *d_r, int log_n, int m);
int agl_partial_eval_ext2_from_base_ffi(const uint64_t *d_input, uint64_t *d_output, const uint64_t *d_r, int log_n,
                                        int m);
int agl_bit_permute_ffi(const uint64_t *d_input, uint64_t *d_output, const int *d_perm_map, int n_bits, int total);
int agl_fused_permute_partial_eval_ffi(const uint64_t *d_evals, uint64_t *d_output, const uint64_t *d_eq_table,
                                       const uint32_t *d_lo_lut, const uint32_t *d_hi_lut, int n, int m, int half,
                                       int output_size, int smem_bytes);

#ifdef __cplusplus
}
#endif
#endif
