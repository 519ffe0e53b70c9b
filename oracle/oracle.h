/*
 * oracle.h -- CPU restatement of the zk-torch prover field hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * product is compared against; it is never linked into, loaded by, or
 * called from the product (morpheus_gb300/).  Only tests/, the smoke()
 * entry point and the bench's CPU-baseline leg use it.
 *
 * Every value this oracle returns is canonical (in [0, p)).  The reference
 * compares GPU output with its CPU provers after reduction mod p
 * (zk-torch-3/src/util/arith.rs:158-164, goldilocks-cuda-rs/src/basefold.rs:25-30),
 * so equality after canonicalisation is the parity criterion.
 *
 * Flat proof layout for Basefold open_ext2 (all u64, canonical), mirroring
 * BasefoldProofExt2 (goldilocks-cuda-rs/src/basefold.rs:124-132):
 *   eval[2]
 *   oracles[n][3][2]                (c0, c1, c2 as Ext2)
 *   folded_roots[n-1][4]
 *   final_codeword[2^lr][2]
 *   per query q (num_queries of them):
 *     index[1]
 *     values[n][2][2]               (pair (v0, v1) of Ext2 per round)
 *     paths: for r in 0..n-1, (n+lr-1-r) digests of 4 u64
 */
#ifndef MORPHEUS_ORACLE_H
#define MORPHEUS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- Host threads for the large loops of one proof (results do not depend on them);
 * default 1, at most 256 ---- */
void or_set_threads(int k);
int or_get_threads(void);

/* ---- Goldilocks scalar + Ext2 (X^2 - 7) ---- */
uint64_t or_gl_add(uint64_t a, uint64_t b);
uint64_t or_gl_sub(uint64_t a, uint64_t b);
uint64_t or_gl_mul(uint64_t a, uint64_t b);
uint64_t or_gl_inv(uint64_t a);
void or_ext2_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]);
void or_ext2_inv(const uint64_t a[2], uint64_t out[2]);

/* ---- Poseidon2 width 8 ---- */
void or_poseidon2_permute(uint64_t state[8]);
void or_poseidon2_hash_gl_leaf(uint64_t a, uint64_t b, uint64_t out[4]);
void or_poseidon2_hash_ext2_leaf(const uint64_t a[2], const uint64_t b[2], uint64_t out[4]);
void or_poseidon2_compress(const uint64_t l[4], const uint64_t r[4], uint64_t out[4]);

/* ---- Fiat-Shamir transcript (zk-torch-3/src/transcript.rs:174-350) ---- */
typedef struct {
    uint64_t st[8];
    uint64_t inb[4];
    uint64_t outb[4];
    int nin;
    int nout;
} or_transcript;
size_t or_transcript_size(void);
void or_tr_new(or_transcript *t, const uint8_t *label, size_t len);
void or_tr_append_u64(or_transcript *t, const uint8_t *label, size_t len, uint64_t v);
void or_tr_append_scalar(or_transcript *t, const uint8_t *label, size_t len, uint64_t v);
void or_tr_append_ext2(or_transcript *t, const uint8_t *label, size_t len, const uint64_t v[2]);
uint64_t or_tr_challenge_scalar(or_transcript *t, const uint8_t *label, size_t len);
void or_tr_challenge_ext2(or_transcript *t, const uint8_t *label, size_t len, uint64_t out[2]);

/* ---- Product sumcheck ----
 * polys: d polynomials of 2^n base-field values, packed [poly][index].
 * Ext2 mode (CpuLinearSumcheckProverExt2 / GpuLinearSumcheckProver):
 *   msgs[n][d+1][2], challenges[n][2], finals[d][2], final_eval[2].
 * Base mode (LinearSumcheckProver): msgs[n][d+1], challenges[n], finals[d], final_eval[1]. */
int or_sumcheck_prove_ext2(or_transcript *t, int n, int d, const uint64_t *polys,
                           uint64_t *msgs, uint64_t *challenges, uint64_t *finals,
                           uint64_t *final_eval);
int or_sumcheck_prove_ext2_polys(or_transcript *t, int n, int d, const uint64_t *polys, uint64_t *msgs,
                                 uint64_t *challenges, uint64_t *finals, uint64_t *final_eval);
int or_sumcheck_prove_base(or_transcript *t, int n, int d, const uint64_t *polys,
                           uint64_t *msgs, uint64_t *challenges, uint64_t *finals,
                           uint64_t *final_eval);
/* SumcheckVerifier::verify (zk-torch-3/src/sumcheck/verifier.rs:17-65).  Returns 1 if accepted. */
int or_sumcheck_verify_ext2(or_transcript *t, int n, int d, const uint64_t claimed[2],
                            const uint64_t *msgs, const uint64_t final_eval[2]);

/* ---- eq / Lagrange basis (zk-torch-3/src/poly/mod.rs:106-161) ---- */
void or_eq_table_base(const uint64_t *r, int n, uint64_t *out);
void or_eq_table_ext2(const uint64_t *r, int n, uint64_t *out);
void or_ml_eval_ext2(const uint64_t *evals, int n, const uint64_t *point, uint64_t out[2]);

/* ---- Basefold ---- */
/* BasefoldTable::generate (goldilocks-cuda-rs/src/basefold.rs:281-321).
 * entries: total_entries * 2 u64 (point, weight); level_offsets[num_rounds] in entries. */
size_t or_basefold_table_entries(int num_vars, int log_rate, int num_rounds);
void or_basefold_table_generate(int num_vars, int log_rate, int num_rounds, uint64_t seed,
                                uint64_t *entries, uint64_t *level_offsets);
void or_bit_reverse_u64(uint64_t *data, int log_n, int stride_words);
void or_bhc_interpolate(const uint64_t *evals, int n, uint64_t *coeffs, uint64_t *bh_evals);
void or_basefold_encode(const uint64_t *coeffs, int n, int log_rate, uint64_t *codeword);
/* tree layout: layers packed [leaves][parents]...[root], 4 u64 per digest (merkle.rs:1-10). */
void or_merkle_tree_gl(const uint64_t *codeword, size_t num_leaves, uint64_t *tree);
void or_merkle_tree_ext2(const uint64_t *codeword, size_t num_leaves, uint64_t *tree);
/* BasefoldCommitment::commit_device: returns root; codeword (2^(n+lr)), bh_evals (2^n), tree. */
void or_basefold_commit(const uint64_t *evals, int n, int log_rate, uint64_t *codeword,
                        uint64_t *bh_evals, uint64_t *tree, uint64_t root[4]);
size_t or_basefold_proof_len(int n, int log_rate, int num_queries);
/* cpu_full_open_ext2 (zk-torch-3/src/commit/cpu_basefold.rs:235-425). */
int or_basefold_open_ext2(const uint64_t *codeword, const uint64_t *bh_evals, const uint64_t *tree,
                          const uint64_t root[4], int n, int log_rate, const uint64_t *point,
                          const uint64_t *table_entries, const uint64_t *level_offsets,
                          or_transcript *t, int num_queries, uint64_t *proof);
/* BasefoldVerifier::verify_ext2 (goldilocks-cuda-rs/src/basefold.rs:1759-1929). */
int or_basefold_verify_ext2(const uint64_t root[4], int n, int log_rate, const uint64_t *point,
                            const uint64_t *proof, int num_queries,
                            const uint64_t *table_entries, const uint64_t *level_offsets,
                            or_transcript *t);

/* batch_open_ext2 (goldilocks-cuda-rs/src/basefold.rs:1202-1532): several committed polynomials
 * (same num_vars, log_rate) opened at Ext2 points.  Commitment c: codewords[c], bh_evals[c],
 * trees[c], roots[4c..4c+3]; points: num_points x n Ext2; evaluation i claims poly ev_poly[i] at
 * point ev_point[i] equals ev_vals[2i..2i+1].  Proof layout: or_basefold_batch_proof_len words
 * (outer oracles | combined root | inner eval | inner oracles | folded roots | final codeword |
 * combined queries | individual queries). */
size_t or_basefold_batch_proof_len(int n, int log_rate, int num_queries, int num_evals);
int or_basefold_batch_open_ext2(const uint64_t *const *codewords, const uint64_t *const *bh_evals,
                                const uint64_t *const *trees, const uint64_t *roots, int num_comms, int n,
                                int log_rate, const uint64_t *points, int num_points, const int *ev_poly,
                                const int *ev_point, const uint64_t *ev_vals, int num_evals,
                                const uint64_t *table_entries, const uint64_t *level_offsets, or_transcript *t,
                                int num_queries, uint64_t *proof);
/* BasefoldVerifier::batch_verify_ext2 (goldilocks-cuda-rs/src/basefold.rs:1931-2220): 1 accepts. */
int or_basefold_batch_verify_ext2(const uint64_t *roots, int num_comms, int n, int log_rate, const uint64_t *points,
                                  int num_points, const int *ev_poly, const int *ev_point, const uint64_t *ev_vals,
                                  int num_evals, const uint64_t *proof, int num_queries,
                                  const uint64_t *table_entries, const uint64_t *level_offsets, or_transcript *t);

/* ---- Monolith-12 over Goldilocks (goldilocks-cuda-rs/src/cpu_monolith.rs:13-226) ---- */
/* The permutation (concrete layer, then 6 rounds of bars, bricks, concrete); canonical in/out. */
void or_monolith_permute(uint64_t s[12]);
/* Merkle trees with the Monolith leaf hash and compression, layout as or_merkle_tree_gl:
 * leaves (4 words each), then each layer up to the root.  gl: leaf i = H(cw[2i], cw[2i+1]);
 * ext2: leaf i = H(cw[4i..4i+3]). */
void or_monolith_tree_gl(const uint64_t *cw, size_t leaves, uint64_t *tree);
void or_monolith_tree_ext2(const uint64_t *cw, size_t leaves, uint64_t *tree);

/* ---- almost-Goldilocks (q = 2^64 - 2^32 - 31) + Ext2 (X^2 - 3) ---- */
uint64_t or_agl_add(uint64_t a, uint64_t b);
uint64_t or_agl_sub(uint64_t a, uint64_t b);
uint64_t or_agl_mul(uint64_t a, uint64_t b);
void or_aext2_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]);

/* ---- partial evaluation / bit permutation (field 0: Goldilocks, 1: almost-Goldilocks) ---- */
/* cuda/partial_eval.cuh (goldilocks-cuda-rs/src/partial_eval.rs:449-520 CPU helpers):
 * fix the low m variables, LSB first; canonical outputs. */
void or_partial_eval_base(int field, const uint64_t *evals, int log_n, const uint64_t *r, int m, uint64_t *out);
void or_partial_eval_ext2(int field, const uint64_t *evals, int log_n, const uint64_t *r, int m, uint64_t *out);
/* wrapper.cu:1824-1841: out[new] = in[old], old bit inv[k] <- new bit k. */
void or_bit_permute(const uint64_t *in, uint64_t *out, const int *inv, int n_bits);
/* cuda/fused_permute_peval.cuh: out[j] = sum_b evals[lo[i & mask] | hi[i >> half]] eq[b], i = j 2^m + b. */
void or_fused_permute_peval(int field, const uint64_t *evals, int n, int m, int half, const uint64_t *eq,
                            const uint32_t *lo, const uint32_t *hi, uint64_t *out);

/* ---- Ajtai commitment ---- */
void or_chacha8_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3], uint32_t out[16]);
void or_ajtai_ring_elem(const uint32_t key[8], uint32_t row, uint64_t j, uint64_t out[64]);
/* commit_wide restricted to rows [row_lo, row_lo+nrows): out[nrows][64] canonical.
 * z: N ring elements x 64 coefficients, entries canonical in [0, q). */
void or_ajtai_commit_wide(const uint32_t key[8], const uint64_t *z, uint64_t N, uint64_t col_offset,
                          int row_lo, int nrows, uint64_t *out);
/* Same commitment for a batch of B witnesses with small (u8) coefficients, M generated once.
 * z8: [B][N*64] bytes; out: [B][nrows][64]. */
void or_ajtai_commit_u8_batch(const uint32_t key[8], const uint8_t *z8, uint64_t N, int B,
                              int row_lo, int nrows, uint64_t *out);

#ifdef __cplusplus
}
#endif
#endif
