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

/* ===================== Part 2: GB300 additions (no reference counterpart) ===================== */

/* Matrix rows [row_lo, row_lo + rows) over n_ring ring columns of the ChaCha8 key h_seed,
 * expanded once into the device-resident operand of the tensor-core commitment (8 bf16 digit
 * planes of the negacyclic expansion: 8 * rows * 64 * roundup(64 n_ring, 1024) * 2 bytes).
 * Synchronising. */
int gb_ajtai_key_create(const uint32_t *h_seed, int row_lo, int rows, uint64_t n_ring, void **handle);
int gb_ajtai_key_destroy(void *handle);
/* The key's first row, row count and ring columns (any output pointer may be NULL). */
int gb_ajtai_key_info(void *handle, int *row_lo, int *rows, uint64_t *n_ring);
/* Commit num_witnesses witnesses with coefficients in [0, 256): d_z is [num_witnesses][n_ring * 64]
 * bytes (device); d_out is [num_witnesses][rows][64] canonical u64 (device).  Rows are those of
 * the key; the result equals ajtai_commit_wide_ffi restricted to those rows.  Synchronising. */
int gb_ajtai_commit_u8_batched(void *key, const uint8_t *d_z, int num_witnesses, uint64_t *d_out);

/* ajtai_commit_wide_ffi without any device allocation (no counterpart in the reference).
 * Same arguments, result and return codes as ajtai_commit_wide_ffi, whose every call
 * allocates and frees its per-column-chunk partial sums.  This variant keeps them in a
 * static device array of the library sized for N <= 4096 ring elements (5.25 MiB); a larger
 * N returns -2 with a message in gb_last_error().  It is for callers that must not allocate
 * on their request path: a service that has reserved its whole HBM budget up front, where an
 * allocation inside the call could fail or wait on the memory pool.
 *   - The first call on each device (with that device current) looks the scratch address up
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *   - Calls share the one scratch: calls that overlap in time (other threads, other streams)
 *     race on it and must be serialised by the caller.
 *   - Nothing in the scratch needs clearing: every word read is written by the same call.
 * Synchronising. */
int ajtai_commit_wide_noalloc_ffi(const uint32_t *d_key, const uint64_t *d_z_wide, uint64_t N, uint64_t col_offset,
                                  int chunk, uint64_t *d_out);

#ifdef __cplusplus
}
#endif
#endif
