// Ajtai commitment over R_q = F_q[X]/(X^64 + 1), q = 2^64 - 2^32 - 31.
//
//   c_i = sum_j M[i][j] * z_j,   c_i[r] = sum_j sum_l s(r,l) M[i][j][(r-l) mod 64] z_j[l],
//   s = -1 when l > r (negacyclic wrap)     (cuda_almost_goldilocks/ajtai.cuh:164-275)
// with M[i][j] drawn by the ChaCha8 PRG keyed by the seed (ajtai_chacha8.cuh:115-178).
//
// Batched small-witness path (witness coefficients in [0, 256)): one exact GEMM on the
// tcgen05 tensor cores, in one of two forms chosen by batch size (below).  sm_103a has no
// integer MMA (ptxas rejects tcgen05 kind::i8), so the contraction runs in bf16 with fp32
// accumulation, kept exact by construction:
//   * every matrix coefficient m is centred (v = m or m - q, |v| < q/2) and split into
//     8 balanced base-256 digits d_p with |d_p| <= 128 (v = sum_p d_p 256^p);
//   * witness coefficients are centred, z' = z - 128 in [-128, 127];
//   * so every product has |d z'| <= 2^14 and a sum of 1024 of them stays <= 2^24, which
//     fp32 represents exactly.  The K dimension is cut into 1024-long chunks; after each
//     chunk the fp32 accumulator (TMEM) is drained into int32 registers (|sum| <= 2^30 over
//     K = 2^16) while the tensor core fills the other accumulator buffer.
//   Key-Toeplitz form (large batches): S_p = T_p . Z'^T with T_p the negacyclic Toeplitz
//   expansion of digit p (rows (p, i, r), columns (j, l)), and c = sum_p 256^p S_p +
//   128 * rowsum(T) mod q.  M128 x N256 MMAs over every witness of a 256-witness tile; the
//   1.07 GB expansion (16 rows x 1024 columns) is streamed once per batch whatever its size.
//   Witness-circulant form (batches up to AJ_WC_MAX_AUTO): the Toeplitz structure on the
//   witness side (ajtai_gemm_wc_kernel), the key as its plain 16 MB of digit planes; one N = 64
//   MMA per witness and K step, so the work follows the batch size.
// Both key operands are built once per (key, rows, columns) and kept in HBM.
//
// The full-width entry point ajtai_commit_wide_ffi (arbitrary field coefficients) runs
// on the CUDA cores with modular multiplications.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "agl.cuh"
#include "common.cuh"

extern "C" const char* gb_last_error(void);  // the calling thread's message (runtime.cu)

namespace gb {

constexpr int AJ_D = 64;
constexpr int AJ_KAPPA = 42;
constexpr int AJ_SPLIT_K = 13;  // ternary chunks of a split witness (ajtai.cuh:1185)
constexpr u64 AJ_HALF_Q = AGL_Q / 2;  // centred representatives: m > q/2 maps to m - q

// ---------------------------------------------------------------------------
// matrix PRG: M[i][j][0..63] for rows [row_lo, row_lo + rows), columns [col0, col0 + N)
// ---------------------------------------------------------------------------
__global__ void ajtai_prg_kernel(const u32* __restrict__ key, int row_lo, int rows, u64 col0, u64 N,
                                 u64* __restrict__ M) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    size_t total = (size_t)rows * N * 8;
    if (t >= total) return;
    u32 k[8];
#pragma unroll
    for (int q = 0; q < 8; q++) k[q] = __ldg(key + q);
    u32 blk = (u32)(t & 7);
    size_t ij = t >> 3;
    u64 j = ij % N;
    int i = (int)(ij / N);
    u64 out[8];
    ajtai_prg_block(k, (u32)(row_lo + i), j + col0, blk, out);
    u64* dst = M + ij * AJ_D + 8 * blk;
#pragma unroll
    for (int q = 0; q < 8; q++) dst[q] = out[q];
}

// balanced base-256 digits of the centred value of m in [0, q)
__device__ __forceinline__ void centred_digits(u64 m, int* d) {
    bool neg = m > AJ_HALF_Q;
    u64 mag = neg ? (AGL_Q - m) : m;  // |v| < 2^63
    long long v = neg ? -(long long)mag : (long long)mag;
#pragma unroll
    for (int p = 0; p < 7; p++) {
        int lo = (int)(v & 255);
        if (lo >= 128) lo -= 256;
        d[p] = lo;
        v = (v - lo) >> 8;
    }
    d[7] = (int)v;  // |d7| <= 128
}

// T[(p, i, r)][(j, l)] = s(r,l) d_p(M[i][j][(r-l) mod 64]) as bf16, stored tile by tile as the
// GEMM reads it: the 128 x 64 tile (m / 128, j) of row m = (p rows + i) 64 + r is 16 KB contiguous
// at ((m / 128) KT + j) 16 KB, already in the 128-byte swizzled layout (16-byte chunk c of tile
// row R at (R / 8) 1024 + (R mod 8) 128 + (c ^ (R mod 8)) 16), so that one bulk copy moves it.
// Tiles past the last ring column (K padded to Kp) are zero.  One block per (i, j), 64 threads
// (thread r writes 8 rows x 64 columns).
__global__ void __launch_bounds__(64) ajtai_expand_kernel(const u64* __restrict__ M, int rows, u64 N, size_t KT,
                                                          __nv_bfloat16* __restrict__ T) {
    __shared__ short dig[AJ_D][8];  // the top digit can be +128: not a signed char
    const u64 j = blockIdx.x;
    const int i = blockIdx.y;
    const int r = threadIdx.x;
    {
        int d[8];
        centred_digits(M[((size_t)i * N + j) * AJ_D + r], d);
#pragma unroll
        for (int p = 0; p < 8; p++) dig[r][p] = (short)d[p];
    }
    __syncthreads();
    const size_t row_stride = (size_t)rows * AJ_D;  // rows per digit
#pragma unroll 1
    for (int p = 0; p < 8; p++) {
        const size_t m = (size_t)p * row_stride + (size_t)i * AJ_D + r;
        const int R = (int)(m & 127);
        uint8_t* tile = reinterpret_cast<uint8_t*>(T) + ((m >> 7) * KT + j) * 16384 + (R >> 3) * 1024 + (R & 7) * 128;
#pragma unroll
        for (int v = 0; v < 8; v++) {
            __align__(16) __nv_bfloat16 w[8];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                int l = v * 8 + e;
                int k = (r - l) & 63;
                int val = dig[k][p];
                w[e] = __int2bfloat16_rn(l <= r ? val : -val);
            }
            *reinterpret_cast<uint4*>(tile + ((v ^ (R & 7)) << 4)) = *reinterpret_cast<uint4*>(w);
        }
    }
}

// The key's Hankel windows: with K reversed inside each ring column (kappa = 63 - l) the 64 x 64
// negacyclic block of (digit plane p, ring row i, ring column j) is
//   H[r][kappa] = G[r + kappa],   G[t] = d_p(M[i][j][t - 63]) (t >= 63), -d_p(M[i][j][t + 1]) (t < 63),
// so its 8 x 8 core matrix (row group a, column group b) depends only on q = a + b: row rho of
// core matrix q is G[8 q + rho .. 8 q + rho + 7].  Block (p, i) is half beta = (p rows + i) % 2 of
// the 128-row key tile m = (p rows + i) / 2, and the tile's two halves interleave by core
// matrix: core matrix q of half beta sits at byte (2 q + beta) 128 of the tile's 3840-byte window
// for ring column j, window (m, j) at (m KT + j) 3840.  A no-swizzle K-major descriptor with a
// 256-byte step along K and a 128-byte step per 8 rows then reads the tile's 128 rows x 64 columns
// in place, row group 2 a' + beta being group a' of half beta.  Padding columns stay zero.  One
// block per (j, i): thread k takes the digits of M[i][j][k], then thread (q, rho) writes row rho of
// core matrix q for every plane.
constexpr int GW_A_BYTES = 15 * 2 * 128;  // a 128-row tile's window for one ring column
__global__ void __launch_bounds__(128) ajtai_window_kernel(const u64* __restrict__ M, int rows, u64 N, size_t KT,
                                                           uint8_t* __restrict__ W) {
    __shared__ short dig[AJ_D][8];  // the top digit can be +128: not a signed char
    const u64 j = blockIdx.x;
    const int i = blockIdx.y;
    if (threadIdx.x < AJ_D) {
        int d[8];
        centred_digits(M[((size_t)i * N + j) * AJ_D + threadIdx.x], d);
#pragma unroll
        for (int p = 0; p < 8; p++) dig[threadIdx.x][p] = (short)d[p];
    }
    __syncthreads();
    const int q = threadIdx.x >> 3, rho = threadIdx.x & 7;
    if (q >= 15) return;  // 120 rows of 16 bytes per plane
#pragma unroll 1
    for (int p = 0; p < 8; p++) {
        const int blk = p * rows + i;
        uint8_t* dst = W + ((size_t)(blk >> 1) * KT + j) * GW_A_BYTES + (2 * q + (blk & 1)) * 128 + rho * 16;
        __align__(16) __nv_bfloat16 w[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int t = 8 * q + rho + c;  // 0 .. 126
            w[c] = __int2bfloat16_rn(t >= 63 ? (int)dig[t - 63][p] : -(int)dig[t + 1][p]);
        }
        *reinterpret_cast<uint4*>(dst) = *reinterpret_cast<const uint4*>(w);
    }
}

// Key operand of the witness-circulant GEMM: A[m][(j, kappa)] = d_p(M[i][j][63 - kappa]) as bf16,
// m = 16 p + (i mod 16) in the 128-row tile i / 16, stored tile by tile like ajtai_expand_kernel's
// output (tile (i / 16, j) 16 KB contiguous at ((i / 16) KT + j) 16 KB, 128-byte swizzled).  Rows
// of absent ring rows and tiles past the last ring column stay zero.  One block per (i, j):
// thread k takes the digits of M[i][j][k], then thread (p, c) writes row 16 p + (i mod 16),
// 16-byte chunk c (kappa = 8c .. 8c + 7).
__global__ void __launch_bounds__(64) ajtai_planes_kernel(const u64* __restrict__ M, u64 N, size_t KT,
                                                          __nv_bfloat16* __restrict__ A) {
    __shared__ short dig[AJ_D][8];
    const u64 j = blockIdx.x;
    const int i = blockIdx.y;
    {
        int d[8];
        centred_digits(M[((size_t)i * N + j) * AJ_D + threadIdx.x], d);
#pragma unroll
        for (int p = 0; p < 8; p++) dig[threadIdx.x][p] = (short)d[p];
    }
    __syncthreads();
    const int p = threadIdx.x >> 3, c = threadIdx.x & 7;
    const int R = 16 * p + (i & 15);
    __align__(16) __nv_bfloat16 w[8];
#pragma unroll
    for (int e = 0; e < 8; e++) w[e] = __int2bfloat16_rn(dig[63 - (8 * c + e)][p]);
    uint8_t* tile = reinterpret_cast<uint8_t*>(A) + ((size_t)(i >> 4) * KT + j) * 16384 + (R >> 3) * 1024 + (R & 7) * 128;
    *reinterpret_cast<uint4*>(tile + ((c ^ (R & 7)) << 4)) = *reinterpret_cast<uint4*>(w);
}

// rowsum(T)[i][r] mod q = sum_j (2 prefix_r(M_ij) - total(M_ij)), one thread per (i, r)
// Canonical residue mod q of a signed 128-bit value x with |x| < 2^88 (the GEMMs' digit-plane
// combinations: 8 planes of int32 sums, sum_p 256^p S_p; the key's column sums over at most 2^24
// ring columns).  Adding q 2^25 makes it positive and
// below 2^90; then 2^64 == 2^32 + 31 (mod q) folds the high word in twice.
__device__ __forceinline__ u64 agl_from_i128(__int128 x) {
    const unsigned __int128 a = (unsigned __int128)(x + ((__int128)AGL_Q << 25));
    const u64 lo = (u64)a, hi = (u64)(a >> 64);  // hi < 2^26
    constexpr u64 C = (1ull << 32) + 31;         // 2^64 mod q
    const unsigned __int128 r = (unsigned __int128)lo + (unsigned __int128)hi * C;  // < 2^64 + 2^59
    const u64 r_lo = (u64)r, r_hi = (u64)(r >> 64);  // r_hi <= 1, and r_lo < 2^59 when it is 1
    const u64 v = r_lo + r_hi * C;
    return v >= AGL_Q ? v - AGL_Q : v;
}

// RS[i][r] = sum_j sum_k s(k, r) M[i][j][k], s = +1 for k <= r, -1 above: the row sums of the
// negacyclic expansion, used for the witnesses' -128 offset.  It factors through the column sums
// C[i][k] = sum_j M[i][j][k]: RS[i][r] = sum_{k <= r} C[i][k] - sum_{k > r} C[i][k].  One block per
// ring row: thread (slice, k) sums column k over a quarter of the ring columns exactly in 128 bits
// (coalesced along k), the quarters meet in shared memory, then thread r forms its signed sum.
__global__ void __launch_bounds__(256) ajtai_rowsum_kernel(const u64* __restrict__ M, u64 N, u64* __restrict__ RS) {
    __shared__ unsigned __int128 part[4][AJ_D];
    __shared__ u64 col[AJ_D];
    const int i = blockIdx.x, k = threadIdx.x & 63, slice = threadIdx.x >> 6;
    unsigned __int128 acc = 0;  // < 2^24 ring columns x 2^64
    for (u64 j = slice; j < N; j += 4) acc += M[((size_t)i * N + j) * AJ_D + k];
    part[slice][k] = acc;
    __syncthreads();
    if (threadIdx.x < AJ_D) {
        const unsigned __int128 t = part[0][k] + part[1][k] + part[2][k] + part[3][k];
        col[k] = agl_canon(agl_from_i128((__int128)t));
    }
    __syncthreads();
    if (threadIdx.x < AJ_D) {
        const int r = threadIdx.x;
        u64 v = 0;
        for (int c = 0; c < AJ_D; c++) v = c <= r ? agl_add(v, col[c]) : agl_sub(v, col[c]);
        RS[(size_t)i * AJ_D + r] = agl_canon(v);
    }
}

// z'[b][k] = z[b][k] - 128 (bf16); padded witnesses / columns are 0.  With REV the K index is
// reversed inside each ring column, z'[b][64 j + kappa] = z[b][64 j + 63 - kappa] - 128 (the
// operand of the Hankel key form).  Eight coefficients per thread: one 8-byte load (K and Kp are
// multiples of 64; the host checks z's alignment) and one 16-byte store.
template <bool REV>
__global__ void ajtai_zprep_kernel(const uint8_t* __restrict__ z, int B, size_t K, int Bp, size_t Kp,
                                   __nv_bfloat16* __restrict__ zc) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    const size_t per_row = Kp / 8;
    if (t >= (size_t)Bp * per_row) return;
    const size_t b = t / per_row, k = (t % per_row) * 8;
    // REV: outputs kappa = k % 64 .. +7 of ring column k / 64 read bytes 56 - kappa .. 63 - kappa
    const size_t src = REV ? (k & ~(size_t)63) + 56 - (k & 63) : k;
    uint2 raw = make_uint2(0x80808080u, 0x80808080u);  // 128 - 128 = 0 for padding
    if (b < (size_t)B && src < K) raw = __ldg(reinterpret_cast<const uint2*>(z + b * K + src));
    __align__(16) __nv_bfloat16 w[8];
#pragma unroll
    for (int e = 0; e < 8; e++) {
        const int byte = REV ? 7 - e : e;
        const u32 word = byte < 4 ? raw.x : raw.y;
        w[e] = __int2bfloat16_rn((int)((word >> (8 * (byte & 3))) & 0xFF) - 128);
    }
    *reinterpret_cast<uint4*>(zc + b * Kp + k) = *reinterpret_cast<const uint4*>(w);
}
// the same, one coefficient per thread, for witness arrays that are not 8-byte aligned
template <bool REV>
__global__ void ajtai_zprep_scalar_kernel(const uint8_t* __restrict__ z, int B, size_t K, int Bp, size_t Kp,
                                          __nv_bfloat16* __restrict__ zc) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)Bp * Kp) return;
    size_t b = t / Kp, k = t % Kp;
    const size_t src = REV ? (k & ~(size_t)63) + 63 - (k & 63) : k;
    int v = (b < (size_t)B && src < K) ? (int)z[b * K + src] - 128 : 0;
    zc[t] = __int2bfloat16_rn(v);
}

constexpr int GM_BM_C = 128, GM_BN_C = 256;  // the GEMM's M and N tiles (GM_BM, GM_BN below)

// Persistent schedule of the GEMM: the (tile, K chunk) units, tile-major (tile t = nt tiles_m +
// mt), split into `ctas` equal contiguous ranges, one per CTA.  A tile's partial sums come from
// the CTAs whose range meets it, each writing its own slot of the tile: slot k of tile t belongs
// to CTA gm_cta_of(t chunks) + k.
struct GmSched {
    int tiles_m, chunks;  // M tiles; K chunks per tile
    long long units;      // tiles x chunks
    int ctas, slots;      // grid size (CTAs, or CTA pairs); slots per tile (the most CTAs meeting one tile)
    unsigned long long spin_limit;  // iterations of each bounded mbarrier wait
    int starve;  // test mode: the producer issues no loads, so that every consumer wait runs out
    int pair = 0;  // 1: an M tile is 256 rows, two 128-row halves, one per CTA of a pair
};
__host__ __device__ inline long long gm_unit_begin(const GmSched& g, long long c) { return c * g.units / g.ctas; }
__host__ __device__ inline int gm_cta_of(const GmSched& g, long long u) {  // the CTA whose range holds u
    return (int)(((u + 1) * g.ctas - 1) / g.units);
}

// c[b][i][r] = sum_p 256^p S[(p, i, r)][b] + 128 rowsum[i][r]  mod q, canonical; S[(p, i, r)][b]
// is the sum of the slots of its tile.  A block takes 32 witnesses x 8 output coefficients, one
// output per thread with all of its slot loads in flight together (the work is ~20 MB of loads,
// so latency, not bandwidth, sets its time), and writes them out along (i, r) through shared
// memory.
constexpr int AJ_CB = 32, AJ_CR = 8;
__global__ void __launch_bounds__(256) ajtai_combine_kernel(const int* __restrict__ S, GmSched sched, int rows,
                                                            int B, const u64* __restrict__ RS,
                                                            u64* __restrict__ out) {
    __shared__ u64 tile[AJ_CR][AJ_CB + 1];
    __shared__ const int* s_base[8];  // per digit plane: the block's first output row in slot 0 of its tile
    __shared__ int s_slots[8];        // and how many slots that tile has
    const int IR = rows * AJ_D;
    const int b0 = blockIdx.x * AJ_CB, ir0 = blockIdx.y * AJ_CR;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // witness b0 + tx, output ir0 + ty
    if (threadIdx.x < 8) {
        // rows p IR + ir0 .. +7 lie in one 128-row tile (IR is a multiple of 64, ir0 of 8); with
        // pairs, 128-row tile mt is half mt % 2 of the schedule's tile mt / 2, and the halves of
        // one tile keep their slots one after the other
        const int p = threadIdx.x, m = p * IR + ir0, nt = b0 / GM_BN_C;
        const int w = sched.pair ? 2 : 1, mt = m / GM_BM_C;
        const long long t = (long long)nt * sched.tiles_m + mt / w;
        s_slots[p] = gm_cta_of(sched, (t + 1) * sched.chunks - 1) - gm_cta_of(sched, t * sched.chunks) + 1;
        s_base[p] = S + (((size_t)t * w + mt % w) * sched.slots * GM_BM_C + m % GM_BM_C) * GM_BN_C + b0 % GM_BN_C;
    }
    __syncthreads();
    const size_t slot = (size_t)GM_BM_C * GM_BN_C;
    const int ir = ir0 + ty, b = b0 + tx;
    u64 val = 0;
    if (ir < IR && b < B) {
        long long part[8];  // |each slot| < 2^31
        // up to 4 slots per tile (any full 256-witness batch of 16 rows): every load unrolled
        bool few = true;
#pragma unroll
        for (int p = 0; p < 8; p++) few = few && s_slots[p] <= 4;
        if (few) {
#pragma unroll
            for (int p = 0; p < 8; p++) {
                const int* sp = s_base[p] + (size_t)ty * GM_BN_C + tx;  // row ir0 + ty, witness b0 + tx
                const int ns = s_slots[p];
                const long long v0 = __ldg(sp), v1 = ns > 1 ? __ldg(sp + slot) : 0;
                const long long v2 = ns > 2 ? __ldg(sp + 2 * slot) : 0, v3 = ns > 3 ? __ldg(sp + 3 * slot) : 0;
                part[p] = v0 + v1 + v2 + v3;
            }
        } else {
            for (int p = 0; p < 8; p++) {
                const int* sp = s_base[p] + (size_t)ty * GM_BN_C + tx;
                long long sum = 0;
                for (int k = 0; k < s_slots[p]; k++) sum += __ldg(sp + (size_t)k * slot);
                part[p] = sum;
            }
        }
        __int128 acc = 0;
#pragma unroll
        for (int p = 7; p >= 0; p--) acc = acc * 256 + (__int128)part[p];
        const u64 rs128 = agl_mul(__ldg(RS + ir), 128);
        val = agl_canon(agl_add(agl_from_i128(acc), agl_canon(rs128)));
    }
    tile[ty][tx] = val;
    __syncthreads();
    {
        const int bo = b0 + (threadIdx.x >> 3), io = ir0 + (threadIdx.x & 7);  // 8 outputs of one witness
        if (bo < B && io < IR) out[(size_t)bo * IR + io] = tile[threadIdx.x & 7][threadIdx.x >> 3];
    }
}

// ---------------------------------------------------------------------------
// tcgen05 GEMM:  S[m][n] = sum_k A[m][k] B[n][k]   (bf16, K-major both, fp32 in TMEM,
// exact per 1024-K chunk, int32 totals), M tile 128, N tile 256 (every witness of a batch of
// 256 in one tile, so each key tile is loaded once), K tile 64 (128-byte swizzled rows),
// 4-stage TMA pipeline of 48 KB stages.  Persistent: CTA c takes the (tile, K chunk) units of
// its GmSched range, which may span tiles; at each tile's last unit it writes its int32 sums to
// its slot of that tile, and the combine adds the slots.
//   warp 0: TMA producer   warp 1: MMA issuer (one thread)   warps 2..17: epilogue, warp w owning
//   TMEM lanes 32 (w % 4) .. +31 and columns 64 ((w - 2) / 4) .. +63 of each accumulator
// ---------------------------------------------------------------------------
constexpr int GM_BM = 128, GM_BN = 256, GM_BK = 64, GM_STAGES = 4, GM_CHUNK_TILES = 16;
static_assert(GM_BM == GM_BM_C && GM_BN == GM_BN_C, "combine tile sizes");
constexpr int GM_A_BYTES = GM_BM * GM_BK * 2;  // 16 KB
constexpr int GM_B_BYTES = GM_BN * GM_BK * 2;  // 32 KB
constexpr int GM_STAGE_BYTES = GM_A_BYTES + GM_B_BYTES;
constexpr int GM_EPI_WARPS = 16;  // four warps per TMEM lane quarter, one per 64-column group
constexpr int GM_THREADS = 64 + 32 * GM_EPI_WARPS;
constexpr int GM_SMEM = GM_STAGES * GM_STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
constexpr unsigned long long GM_SPIN_LIMIT = 1ull << 26;  // bounded waits (seconds at worst)
constexpr unsigned long long GM_SPIN_LIMIT_TEST = 1ull << 14;  // the starved test mode's limit

__device__ __forceinline__ u32 smem_u32(const void* p) { return (u32)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(u32 bar, u32 count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(u32 bar, u32 bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(u32 bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(u32 bar, u32 parity) {
    u32 ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false (and the error flag set) when the limit is reached
__device__ __forceinline__ bool mbar_wait(u32 bar, u32 parity, int* err, int code,
                                          unsigned long long limit = GM_SPIN_LIMIT) {
    for (unsigned long long it = 0; it < limit; it++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 1023) == 1023 && *(volatile int*)err) return false;  // another role already gave up
    }
    atomicCAS(err, 0, code);
    return false;
}

__device__ __forceinline__ void tma_load_2d(u32 dst, const CUtensorMap* map, int x, int y, u32 bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(map), "r"(x), "r"(y), "r"(bar)
        : "memory");
}

// one contiguous global -> shared copy by the async proxy (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_load(u32 dst, const void* src, u32 bytes, u32 bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// the same copy with an L2 eviction-priority policy (a createpolicy value)
__device__ __forceinline__ void bulk_load_hint(u32 dst, const void* src, u32 bytes, u32 bar, u64 policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
            dst),
        "l"(src), "r"(bytes), "r"(bar), "l"(policy)
        : "memory");
}
// L2 policy for data read once while other data should stay: evicted first
__device__ __forceinline__ u64 l2_evict_first() {
    u64 p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart
__device__ __forceinline__ u64 umma_desc_sw128(u32 saddr) {
    u64 d = 0;
    d |= (u64)((saddr & 0x3FFFF) >> 4);  // start address
    d |= (u64)1 << 16;                   // leading-dimension offset (unused for swizzled K-major)
    d |= (u64)(1024 >> 4) << 32;         // stride-dimension offset
    d |= (u64)1 << 46;                   // descriptor version for tcgen05
    d |= (u64)2 << 61;                   // 128-byte swizzle
    return d;
}

// shared-memory matrix descriptor of a Hankel window (ajtai_window_kernel): K-major, no swizzle,
// core matrices 256 bytes apart along K and 128 bytes apart per 8 rows
__device__ __forceinline__ u64 umma_desc_hankel(u32 saddr) {
    u64 d = (u64)((saddr & 0x3FFFF) >> 4);
    d |= (u64)(256 >> 4) << 16;  // leading-dimension (K) offset
    d |= (u64)(128 >> 4) << 32;  // stride-dimension (8-row group) offset
    d |= (u64)1 << 46;           // descriptor version for tcgen05; layout 0 = no swizzle
    return d;
}

// instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = 256
constexpr u32 GM_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((u32)(GM_BN >> 3) << 17) | ((u32)(GM_BM >> 4) << 24);

__global__ void __launch_bounds__(GM_THREADS, 1) ajtai_gemm_kernel(const __nv_bfloat16* __restrict__ A_tiled,
                                                                   const __grid_constant__ CUtensorMap tmB, int k_tiles,
                                                                   GmSched sched, int* __restrict__ S,
                                                                   int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + GM_STAGES * GM_STAGE_BYTES);
    // bars: full[S], empty[S], acc_full[2], acc_empty[2], mma_done; tmem base address after them
    u32* tmem_slot = (u32*)(bars + 2 * GM_STAGES + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // this CTA's units [u0, u0 + chunks) (at least one: the host launches at most `units` CTAs)
    const long long u0 = gm_unit_begin(sched, blockIdx.x);
    const int chunks = (int)(gm_unit_begin(sched, blockIdx.x + 1) - u0);
    // unit -> tile and its operand rows, and the unit's first K tile
    auto unit_tile = [&](int lu) { return (u0 + lu) / sched.chunks; };
    auto unit_m0 = [&](int lu) { return (int)(unit_tile(lu) % sched.tiles_m) * GM_BM; };
    auto unit_n0 = [&](int lu) { return (int)(unit_tile(lu) / sched.tiles_m) * GM_BN; };
    auto unit_k0 = [&](int lu) { return (int)((u0 + lu) % sched.chunks) * GM_CHUNK_TILES; };

    auto full = [&](int s) { return smem_u32(bars + s); };
    auto empty = [&](int s) { return smem_u32(bars + GM_STAGES + s); };
    auto acc_full = [&](int a) { return smem_u32(bars + 2 * GM_STAGES + a); };
    auto acc_empty = [&](int a) { return smem_u32(bars + 2 * GM_STAGES + 2 + a); };
    const u32 mma_done = smem_u32(bars + 2 * GM_STAGES + 4);

    if (threadIdx.x == 0) {
        for (int s = 0; s < GM_STAGES; s++) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(acc_full(a), 1);
            mbar_init(acc_empty(a), 32 * GM_EPI_WARPS);
        }
        mbar_init(mma_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {  // TMEM: two 256-column fp32 accumulators (all 512 columns; one CTA per SM)
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const u32 tmem = *(volatile u32*)tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // kt counts this CTA's K tiles from 0 (stage and phase); unit kt / 16 gives the coordinates
            const int my_tiles = sched.starve ? 0 : chunks * GM_CHUNK_TILES;
            // the key expansion is read once: evicted first, so that the witness digits (read
            // once per M tile) stay in L2
            const u64 pol_key = l2_evict_first();
            int issued = 0;
            for (int kt = 0; kt < my_tiles; kt++) {
                int s = kt % GM_STAGES;
                u32 ph = (kt / GM_STAGES) & 1;
                if (!mbar_wait(empty(s), ph ^ 1, err, 1, sched.spin_limit)) break;
                mbar_expect_tx(full(s), GM_STAGE_BYTES);
                uint8_t* sa = smem + s * GM_STAGE_BYTES;
                const int lu = kt / GM_CHUNK_TILES, x = (unit_k0(lu) + kt % GM_CHUNK_TILES) * GM_BK;
                // the key tile (m0 / 128, x / 64) is 16 KB contiguous and already swizzled
                bulk_load_hint(smem_u32(sa),
                               A_tiled + ((size_t)(unit_m0(lu) / GM_BM) * k_tiles + x / GM_BK) * (GM_A_BYTES / 2),
                               GM_A_BYTES, full(s), pol_key);
                tma_load_2d(smem_u32(sa + GM_A_BYTES), &tmB, x, unit_n0(lu), full(s));
                issued = kt + 1;
            }
            // loads still in flight land in shared memory: wait (bounded) for every issued stage
            for (int kt = issued - GM_STAGES < 0 ? 0 : issued - GM_STAGES; kt < issued; kt++)
                mbar_wait(full(kt % GM_STAGES), (kt / GM_STAGES) & 1, err, 5, sched.spin_limit);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            bool ok = true;
            for (int c = 0; c < chunks && ok; c++) {
                int a = c & 1;
                u32 use = (u32)(c >> 1);
                if (!mbar_wait(acc_empty(a), (use & 1) ^ 1, err, 2, sched.spin_limit)) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const u32 d_tmem = tmem + (u32)(a * GM_BN);
                for (int t = 0; t < GM_CHUNK_TILES; t++) {
                    int kt = c * GM_CHUNK_TILES + t;
                    int s = kt % GM_STAGES;
                    if (!mbar_wait(full(s), (kt / GM_STAGES) & 1, err, 3, sched.spin_limit)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    u32 sa = smem_u32(smem + s * GM_STAGE_BYTES);
                    u64 adesc = umma_desc_sw128(sa), bdesc = umma_desc_sw128(sa + GM_A_BYTES);
#pragma unroll
                    for (int k = 0; k < GM_BK / 16; k++) {
                        u32 acc = (t > 0 || k > 0) ? 1u : 0u;
                        // advance 16 bf16 = 32 bytes along K inside the swizzled rows
                        u64 ad = adesc + (u64)((k * 32) >> 4), bd = bdesc + (u64)((k * 32) >> 4);
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                            "l"(ad), "l"(bd), "r"(GM_IDESC), "r"(acc));
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                        empty(s)));
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    acc_full(a)));
            }
            // every MMA this thread issued has completed before TMEM can be released
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mma_done));
            mbar_wait(mma_done, 0, err, 6, sched.spin_limit);
        }
    } else {
        // epilogue: int32 totals of one TMEM row (lane) x 64 columns in registers
        const int quarter = warp & 3;
        const int half = (warp - 2) >> 2;  // 64-column group 0..3
        const int row = quarter * 32 + lane;
        constexpr int COLS = 64;
        int acc[COLS];
#pragma unroll
        for (int q = 0; q < COLS; q++) acc[q] = 0;
        bool ok = true;
        for (int c = 0; c < chunks && ok; c++) {
            int a = c & 1;
            u32 use = (u32)(c >> 1);
            if (!mbar_wait(acc_full(a), use & 1, err, 4, sched.spin_limit)) {
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int cb = 0; cb < COLS; cb += 16) {
                u32 v[16];
                u32 taddr = tmem + ((u32)(quarter * 32) << 16) + (u32)(a * GM_BN + half * COLS + cb);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int e = 0; e < 16; e++) acc[cb + e] += __float2int_rn(__uint_as_float(v[e]));
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            mbar_arrive(acc_empty(a));
            // the tile's last unit of this CTA: its sums go to this CTA's slot of the tile
            const long long t = unit_tile(c);
            if (c + 1 == chunks || unit_tile(c + 1) != t) {
                const int k = (int)blockIdx.x - gm_cta_of(sched, t * sched.chunks);
                int* dst = S + (((size_t)t * sched.slots + k) * GM_BM + row) * GM_BN + half * COLS;
#pragma unroll
                for (int q = 0; q < COLS; q += 4) {
                    *reinterpret_cast<int4*>(dst + q) = make_int4(acc[q], acc[q + 1], acc[q + 2], acc[q + 3]);
                    acc[q] = acc[q + 1] = acc[q + 2] = acc[q + 3] = 0;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// ---------------------------------------------------------------------------
// The same GEMM on CTA pairs (clusters of 2, `tcgen05.mma.cta_group::2`): an M tile is 256 key
// rows, rows 0..127 in the even CTA's shared memory and 128..255 in the odd one's, and the 256
// witnesses of the N tile are split the same way, 0..127 and 128..255.  One thread of the even
// CTA issues M = 256 MMAs; each CTA's TMEM receives its 128 rows x all 256 witnesses.  So each
// SM loads half of the witness tile (the batch's witness digits are read from L2 once per 256
// key rows instead of once per 128) and a stage is 32 KB, six in flight.
//   Both CTAs: warp 0 loads the CTA's halves into its stages; warps 2..17 drain the CTA's TMEM
//   exactly as ajtai_gemm_kernel does and arrive on the even CTA's accumulator-empty barriers.
//   Even CTA, warp 1: the MMA issuer; it waits for its own stage and for the odd CTA's relay,
//   and its commits arrive on the stage-empty and accumulator-full barriers of both CTAs.
//   Odd CTA, warp 1: the relay; each of the CTA's stages, once loaded, is passed on as one
//   arrival on the even CTA's pair-full barrier of that stage.
// The arrivals on the other CTA's barriers are relaxed: each is made only after the arriving
// thread's own wait has seen what it reports complete (the stage's bytes landed, or the TMEM
// reads done with tcgen05.wait::ld), and shared memory has no cache to publish.  A release arrival
// per stage (a cluster-scope fence in the relay) held the pair to 0.44 ms per 256-witness batch
// against 0.29 ms relaxed.  The issuer's wait on the relay is what keeps the odd CTA's stage
// phases in step with the MMAs: it is not optional.
// Every wait is bounded.  Every thread of both CTAs passes the same two cluster barriers at the
// start and one at the end (none returns early), both CTAs allocate and free TMEM together, and
// each CTA waits for the arrivals the other still owes it before the last barrier.
// ---------------------------------------------------------------------------
constexpr int GP_BN_HALF = GM_BN / 2;               // witnesses of one CTA
constexpr int GP_B_BYTES = GP_BN_HALF * GM_BK * 2;  // 16 KB
// Stage shape per key layout.  HANKEL = false: one ring column (K = 64) per stage, the Toeplitz
// expansion's 16 KB swizzled tile, then the witness half.  HANKEL = true: two ring columns per
// stage (half the waits and commits per MMA), their two 3840-byte windows (ajtai_window_kernel,
// adjacent in memory: one copy) in an 8 KB slot, then the two witness halves, each at a
// 1024-byte boundary (their 128-byte swizzle needs one).
template <bool HANKEL>
struct GpShape {
    static constexpr int COLS = HANKEL ? 2 : 1;  // ring columns (64-deep K tiles) per stage
    static constexpr int STAGES = HANKEL ? 5 : 6;
    static constexpr int A_BYTES = HANKEL ? GW_A_BYTES : GM_A_BYTES;  // one column's key operand
    static constexpr int B_OFF = HANKEL ? 8192 : GM_A_BYTES;
    static constexpr int STAGE_BYTES = B_OFF + COLS * GP_B_BYTES;
    static constexpr int TX_BYTES = COLS * (A_BYTES + GP_B_BYTES);  // what one stage's copies deliver
    static constexpr int NBAR = 3 * STAGES + 5;  // full, empty, pair-full, accumulators x 4, mma_done
    static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 /*align*/ + 512 /*barriers*/;
    static_assert(NBAR * 8 + 8 <= 512, "barrier area");
    static_assert(COLS * A_BYTES <= B_OFF && B_OFF % 1024 == 0 && STAGE_BYTES % 1024 == 0, "stage layout");
    static_assert(GM_CHUNK_TILES % COLS == 0, "whole stages per 1024-deep chunk");
};
// instruction descriptor: D f32, A/B bf16, both K-major, M = 256 (the pair), N = 256
constexpr u32 GP_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((u32)(GM_BN >> 3) << 17) | ((u32)(256 >> 4) << 24);

__device__ __forceinline__ u32 cluster_rank() {
    u32 r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// the shared::cluster address of the same shared-memory offset in CTA `cta` of the cluster
__device__ __forceinline__ u32 peer_addr(u32 local, u32 cta) {
    u32 r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(cta));
    return r;
}
// relaxed arrival on a barrier of the other CTA of the pair (see the ordering note above)
__device__ __forceinline__ void mbar_arrive_remote(u32 cluster_addr) {
    asm volatile("mbarrier.arrive.relaxed.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait_cluster(u32 bar, u32 parity) {
    u32 ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait on a barrier that the other CTA of the pair arrives on
__device__ __forceinline__ bool mbar_wait_cluster(u32 bar, u32 parity, int* err, int code, unsigned long long limit) {
    for (unsigned long long it = 0; it < limit; it++) {
        if (mbar_try_wait_cluster(bar, parity)) return true;
        if ((it & 1023) == 1023 && *(volatile int*)err) return false;
    }
    atomicCAS(err, 0, code);
    return false;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

template <bool HANKEL>
__global__ void __launch_bounds__(GM_THREADS, 1) ajtai_gemm_pair_kernel(const uint8_t* __restrict__ A_tiles,
                                                                        const __grid_constant__ CUtensorMap tmB,
                                                                        int k_tiles, GmSched sched,
                                                                        int* __restrict__ S, int* __restrict__ err) {
    using SH = GpShape<HANKEL>;
    constexpr int GP_STAGES = SH::STAGES;
    constexpr int SPC = GM_CHUNK_TILES / SH::COLS;  // stages per 1024-deep chunk
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t* bars = (uint64_t*)(smem + GP_STAGES * SH::STAGE_BYTES);
    u32* tmem_slot = (u32*)(bars + SH::NBAR);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const u32 rank = cluster_rank();  // 0: the even CTA (the MMA issuer's), 1: the odd one
    const int pair_id = (int)(blockIdx.x >> 1);
    const long long u0 = gm_unit_begin(sched, pair_id);
    const int chunks = (int)(gm_unit_begin(sched, pair_id + 1) - u0);
    auto unit_tile = [&](int lu) { return (u0 + lu) / sched.chunks; };
    // this CTA's 128-row key tile of the unit's 256-row tile, its witness half, its first K tile
    auto unit_m128 = [&](int lu) { return (int)(unit_tile(lu) % sched.tiles_m) * 2 + (int)rank; };
    auto unit_n0 = [&](int lu) { return (int)(unit_tile(lu) / sched.tiles_m) * GM_BN + (int)rank * GP_BN_HALF; };
    auto unit_k0 = [&](int lu) { return (int)((u0 + lu) % sched.chunks) * GM_CHUNK_TILES; };

    auto full = [&](int s) { return smem_u32(bars + s); };
    auto empty = [&](int s) { return smem_u32(bars + GP_STAGES + s); };
    auto pfull = [&](int s) { return smem_u32(bars + 2 * GP_STAGES + s); };  // even CTA: the odd CTA's stage is in
    auto acc_full = [&](int a) { return smem_u32(bars + 3 * GP_STAGES + a); };
    auto acc_empty = [&](int a) { return smem_u32(bars + 3 * GP_STAGES + 2 + a); };  // even CTA: both drained
    const u32 mma_done = smem_u32(bars + 3 * GP_STAGES + 4);

    if (threadIdx.x == 0) {
        for (int s = 0; s < GP_STAGES; s++) {
            mbar_init(full(s), 1);
            mbar_init(empty(s), 1);
            mbar_init(pfull(s), 1);
        }
        for (int a = 0; a < 2; a++) {
            mbar_init(acc_full(a), 1);
            mbar_init(acc_empty(a), 2 * GM_EPI_WARPS);  // one arrival per epilogue warp of each CTA
        }
        mbar_init(mma_done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    cluster_sync_all();  // both CTAs resident, every barrier initialised before any remote arrival
    if (warp == 1) {  // TMEM, allocated by one warp of each CTA together: two 256-column accumulators
        __syncwarp();
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    cluster_sync_all();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const u32 tmem = *(volatile u32*)tmem_slot;
    u32 tmem_peer;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(tmem_peer) : "r"(peer_addr(smem_u32(tmem_slot), rank ^ 1u)));
    // the MMAs address both CTAs' TMEM through one address: a pair that got different ones does no work
    const bool bad = tmem != tmem_peer;
    if (bad && threadIdx.x == 0) atomicCAS(err, 0, 7);
    const int my_tiles = (bad || sched.starve) ? 0 : chunks * SPC;  // this CTA's stages
    const int my_chunks = bad ? 0 : chunks;

    if (warp == 0) {
        if (lane == 0) {
            const u64 pol_key = l2_evict_first();  // the key expansion is read once (as in ajtai_gemm_kernel)
            int issued = 0;
            for (int kt = 0; kt < my_tiles; kt++) {
                const int s = kt % GP_STAGES;
                const u32 ph = (kt / GP_STAGES) & 1;
                if (!mbar_wait(empty(s), ph ^ 1, err, 1, sched.spin_limit)) break;
                mbar_expect_tx(full(s), SH::TX_BYTES);
                uint8_t* sa = smem + s * SH::STAGE_BYTES;
                const int lu = kt / SPC, x = (unit_k0(lu) + (kt % SPC) * SH::COLS) * GM_BK;
                // the key tiles (or windows) of (m128, x / 64 ..) are COLS x A_BYTES contiguous,
                // in their smem layout
                bulk_load_hint(smem_u32(sa), A_tiles + ((size_t)unit_m128(lu) * k_tiles + x / GM_BK) * SH::A_BYTES,
                               SH::COLS * SH::A_BYTES, full(s), pol_key);
#pragma unroll
                for (int col = 0; col < SH::COLS; col++)
                    tma_load_2d(smem_u32(sa + SH::B_OFF + col * GP_B_BYTES), &tmB, x + col * GM_BK, unit_n0(lu), full(s));
                issued = kt + 1;
            }
            // the loads still in flight land, then the issuer's last commits for this CTA's stages
            // arrive here, before the CTA may leave
            const int first = issued - GP_STAGES < 0 ? 0 : issued - GP_STAGES;
            for (int kt = first; kt < issued; kt++)
                mbar_wait(full(kt % GP_STAGES), (kt / GP_STAGES) & 1, err, 5, sched.spin_limit);
            for (int kt = first; kt < issued; kt++)
                mbar_wait(empty(kt % GP_STAGES), (kt / GP_STAGES) & 1, err, 9, sched.spin_limit);
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 1) {
            // relay: each loaded stage of this CTA becomes one arrival on the even CTA's pair-full
            for (int kt = 0; kt < my_tiles; kt++) {
                const int s = kt % GP_STAGES;
                if (!mbar_wait(full(s), (kt / GP_STAGES) & 1, err, 8, sched.spin_limit)) break;
                mbar_arrive_remote(peer_addr(pfull(s), 0));
            }
        } else if (lane == 0 && rank == 0) {
            bool ok = true;
            int used = 0;  // accumulators handed out, for the final wait on their drains
            for (int c = 0; c < my_chunks && ok; c++) {
                const int a = c & 1;
                const u32 use = (u32)(c >> 1);
                if (!mbar_wait_cluster(acc_empty(a), (use & 1) ^ 1, err, 2, sched.spin_limit)) break;
                asm volatile("tcgen05.fence::after_thread_sync;");
                const u32 d_tmem = tmem + (u32)(a * GM_BN);
                for (int t = 0; t < SPC; t++) {
                    const int kt = c * SPC + t;
                    const int s = kt % GP_STAGES;
                    const u32 ph = (kt / GP_STAGES) & 1;
                    if (!mbar_wait(full(s), ph, err, 3, sched.spin_limit) ||
                        !mbar_wait(pfull(s), ph, err, 10, sched.spin_limit)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const u32 sa = smem_u32(smem + s * SH::STAGE_BYTES);
#pragma unroll
                    for (int col = 0; col < SH::COLS; col++) {
                        const u32 a_col = sa + col * SH::A_BYTES;
                        const u64 adesc = HANKEL ? umma_desc_hankel(a_col) : umma_desc_sw128(a_col);
                        const u64 bdesc = umma_desc_sw128(sa + SH::B_OFF + col * GP_B_BYTES);
#pragma unroll
                        for (int k = 0; k < GM_BK / 16; k++) {
                            const u32 acc = (t > 0 || col > 0 || k > 0) ? 1u : 0u;
                            // K step k: 16 columns = 32 bytes inside the swizzled rows, or two core
                            // matrices (2 x 256 bytes) along K in the window
                            const u64 ad = adesc + (u64)((HANKEL ? k * 512 : k * 32) >> 4);
                            const u64 bd = bdesc + (u64)((k * 32) >> 4);
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                                "l"(ad), "l"(bd), "r"(GP_IDESC), "r"(acc));
                        }
                    }
                    // the stage is free again in both CTAs once these MMAs have read it
                    asm volatile(
                        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
                        "[%0], %1;" ::"r"(empty(s)),
                        "h"((unsigned short)3));
                }
                if (!ok) break;
                asm volatile(
                    "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
                    "[%0], %1;" ::"r"(acc_full(a)),
                    "h"((unsigned short)3));
                used = c + 1;
            }
            asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mma_done));
            mbar_wait(mma_done, 0, err, 6, sched.spin_limit);
            // the odd CTA's epilogue arrives here after each drain: wait for the last ones
            for (int c = used - 2 < 0 ? 0 : used - 2; c < used; c++)
                mbar_wait_cluster(acc_empty(c & 1), (u32)(c >> 1) & 1, err, 11, sched.spin_limit);
        }
    } else {
        // epilogue: int32 totals of one TMEM row (lane) x 64 columns in registers
        const int quarter = warp & 3;
        const int half = (warp - 2) >> 2;
        const int row = quarter * 32 + lane;
        constexpr int COLS = 64;
        int acc[COLS];
#pragma unroll
        for (int q = 0; q < COLS; q++) acc[q] = 0;
        for (int c = 0; c < my_chunks; c++) {
            const int a = c & 1;
            const u32 use = (u32)(c >> 1);
            if (!mbar_wait(acc_full(a), use & 1, err, 4, sched.spin_limit)) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
            for (int cb = 0; cb < COLS; cb += 16) {
                u32 v[16];
                const u32 taddr = tmem + ((u32)(quarter * 32) << 16) + (u32)(a * GM_BN + half * COLS + cb);
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                    "%13, %14, %15}, [%16];"
                    : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                      "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                      "=r"(v[15])
                    : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int e = 0; e < 16; e++) acc[cb + e] += __float2int_rn(__uint_as_float(v[e]));
            }
            // every lane's TMEM reads have completed (wait::ld): one arrival for the warp, on the
            // even CTA's barrier
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) {
                if (rank == 0)
                    mbar_arrive(acc_empty(a));
                else
                    mbar_arrive_remote(peer_addr(acc_empty(a), 0));
            }
            // the tile's last unit of this pair: its sums go to this pair's slot of the CTA's half
            const long long t = unit_tile(c);
            if (c + 1 == chunks || unit_tile(c + 1) != t) {
                const int k = pair_id - gm_cta_of(sched, t * sched.chunks);
                // the window's row group 2 a' + beta is group a' of the tile's 64-row half beta
                const int srow = HANKEL ? ((row >> 3) & 1) * 64 + (row >> 4) * 8 + (row & 7) : row;
                int* dst = S + ((((size_t)t * 2 + rank) * sched.slots + k) * GM_BM + srow) * GM_BN + half * COLS;
#pragma unroll
                for (int q = 0; q < COLS; q += 4) {
                    *reinterpret_cast<int4*>(dst + q) = make_int4(acc[q], acc[q + 1], acc[q + 2], acc[q + 3]);
                    acc[q] = acc[q + 1] = acc[q + 2] = acc[q + 3] = 0;
                }
            }
        }
    }
    // neither CTA leaves (or frees TMEM) while the other may still use its shared memory or TMEM
    asm volatile("tcgen05.fence::before_thread_sync;");
    cluster_sync_all();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 1) {
        __syncwarp();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, 512;" ::"r"(tmem));
    }
}

// ---------------------------------------------------------------------------
// Witness-circulant tcgen05 GEMM.  The negacyclic structure moves to the witness side:
//   c_i[r] = sum_j sum_k M_ij[k] s'(r,k) z_j[(r-k) mod 64],   s' = -1 when k > r,
// so the key operand is the plain digit planes: A rows m = 16 p + (i mod 16) (digit plane p, ring
// row i; 128 rows per 16 ring rows), K = (j, kappa) with kappa = 63 - k reversed inside each ring
// column, 16 MB for 16 rows x 1024 columns, read through L2.  Witness z contributes, per ring
// column j, the 64 x 64 circulant
//   W[r][kappa] = G[r + kappa - 63],   G[t] = z'[t] (t >= 0), -z'[t + 64] (t < 0),   z' = z - 128.
// In the K-major no-swizzle layout the 8 x 8 core matrix (rows 8a.., columns 8b..) of W depends
// only on a + b: its row rho is G[8(a + b) + rho - 63 .. +7].  So W has 15 distinct core matrices,
// stored 128 bytes apart, and the MMA reads them in place through a descriptor whose leading- and
// stride-dimension offsets are both 128 bytes: one witness is one N = 64 MMA per K step, 1920
// bytes of shared memory per ring column instead of 8 KB.  A CTA's N tile is 4 witnesses (256
// TMEM columns), the accumulator pair fills TMEM.  Exactness as in ajtai_gemm_kernel:
// |d_p| <= 128, |G| <= 128, fp32 chunks 1024 deep, int32 totals.
//   warp 0: bulk-copy producer (the stage's key tile; each unit's witness bytes, 1 KB per witness)
//   warps 1 and 18: MMA issuers (one thread each), witnesses 0-1 and 2-3 of the tile.  An N = 64
//     MMA costs its issuing thread about 100 cycles, three times its tensor work, so two issuers
//     (measured: 0.35 against 0.44 ms for 256 witnesses; four: 0.33 ms, with register spills)
//   warps 2..17: build each stage's circulants (one 16-byte core-matrix row per thread) and drain
//     the accumulators (warp w: TMEM lanes 32 (w % 4) .. +31, the 64 columns of witness (w - 2) / 4)
// ---------------------------------------------------------------------------
constexpr int WC_WIT = 4;                  // witnesses per N tile
constexpr int WC_BN = WC_WIT * AJ_D;       // accumulator columns (witness, r)
constexpr int WC_STAGES = 8;
constexpr int WC_LAG = 4;                  // a chunk is drained this many stages into the next one
static_assert(WC_LAG % 4 == 0 && WC_LAG + 3 < 16, "each build group drains at one of its own stages");
constexpr int WC_A_BYTES = GM_BM * GM_BK * 2;            // 16 KB key tile
constexpr int WC_WIN_BYTES = 2048;                       // one circulant: 15 core matrices (1920 B)
constexpr int WC_ROWS_W = 120;                           // 16-byte core-matrix rows of one circulant
constexpr int WC_STAGE_BYTES = WC_A_BYTES + WC_WIT * WC_WIN_BYTES;  // 24 KB
constexpr int WC_ZUNIT = WC_WIT * GM_CHUNK_TILES * AJ_D;  // a unit's witness bytes: 4 KB
constexpr int WC_BUILDERS = 512;
constexpr int WC_ISSUERS = 2;  // MMA-issuing warps (1 and 18), two witnesses each
constexpr int WC_THREADS = 64 + WC_BUILDERS + 32 * (WC_ISSUERS - 1);
constexpr int WC_NBAR = 3 * WC_STAGES + 8 + WC_ISSUERS;
constexpr int WC_SMEM = WC_STAGES * WC_STAGE_BYTES + 2 * WC_ZUNIT + 1024 /*align*/ + 512 /*barriers*/;
static_assert(WC_WIT * WC_ROWS_W <= 4 * 128, "four core-matrix rows per thread of a build group");
// instruction descriptor: D f32, A/B bf16, both K-major, M = 128, N = 64
constexpr u32 WC_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((u32)(AJ_D >> 3) << 17) | ((u32)(GM_BM >> 4) << 24);

// shared-memory descriptor of a circulant: K-major, no swizzle, core matrices 128 bytes apart along
// both K (leading dimension) and N (stride dimension)
__device__ __forceinline__ u64 umma_desc_circ(u32 saddr) {
    u64 d = (u64)((saddr & 0x3FFFF) >> 4);
    d |= (u64)(128 >> 4) << 16;
    d |= (u64)(128 >> 4) << 32;
    d |= (u64)1 << 46;  // descriptor version for tcgen05; layout 0 = no swizzle
    return d;
}

__device__ __forceinline__ u32 bf16x2_of(int lo, int hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn((float)lo, (float)hi);  // |lo|, |hi| <= 128: exact
    return *reinterpret_cast<u32*>(&v);
}

__global__ void __launch_bounds__(WC_THREADS, 1) ajtai_gemm_wc_kernel(const __nv_bfloat16* __restrict__ A_tiled,
                                                                      const uint8_t* __restrict__ z, int B, u64 n_ring,
                                                                      int k_tiles, GmSched sched, int* __restrict__ S,
                                                                      int* __restrict__ err) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t* zs = smem + WC_STAGES * WC_STAGE_BYTES;  // two units' witness bytes
    uint64_t* bars = (uint64_t*)(zs + 2 * WC_ZUNIT);
    // bars: full[S] (key tile landed), ready[S] (circulants built), empty[S] (MMAs done with the
    // stage, one arrival per issuer), zfull[2], zempty[2], acc_full[2] (one arrival per issuer),
    // acc_empty[2], mma_done[issuers]; TMEM base address after them
    u32* tmem_slot = (u32*)(bars + WC_NBAR);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long u0 = gm_unit_begin(sched, blockIdx.x);
    const int chunks = (int)(gm_unit_begin(sched, blockIdx.x + 1) - u0);
    const int T = chunks * GM_CHUNK_TILES;  // this CTA's stages, one ring column each
    auto unit_tile = [&](int lu) { return (u0 + lu) / sched.chunks; };
    auto unit_mt = [&](int lu) { return (int)(unit_tile(lu) % sched.tiles_m); };
    auto unit_b0 = [&](int lu) { return (int)(unit_tile(lu) / sched.tiles_m) * WC_WIT; };
    auto unit_j0 = [&](int lu) { return (u64)((u0 + lu) % sched.chunks) * GM_CHUNK_TILES; };
    auto full = [&](int s) { return smem_u32(bars + s); };
    auto ready = [&](int s) { return smem_u32(bars + WC_STAGES + s); };
    auto empty = [&](int s) { return smem_u32(bars + 2 * WC_STAGES + s); };
    auto zfull = [&](int b) { return smem_u32(bars + 3 * WC_STAGES + b); };
    auto zempty = [&](int b) { return smem_u32(bars + 3 * WC_STAGES + 2 + b); };
    auto acc_full = [&](int a) { return smem_u32(bars + 3 * WC_STAGES + 4 + a); };
    auto acc_empty = [&](int a) { return smem_u32(bars + 3 * WC_STAGES + 6 + a); };
    auto mma_done = [&](int q) { return smem_u32(bars + 3 * WC_STAGES + 8 + q); };
    const unsigned long long lim = sched.spin_limit;

    if (threadIdx.x == 0) {
        for (int s = 0; s < WC_STAGES; s++) {
            mbar_init(full(s), 1);
            mbar_init(ready(s), 4);  // the four warps of the stage's build group
            mbar_init(empty(s), WC_ISSUERS);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(zfull(b), 1);
            mbar_init(zempty(b), WC_BUILDERS / 32);  // one arrival per warp
            mbar_init(acc_full(b), WC_ISSUERS);
            mbar_init(acc_empty(b), WC_BUILDERS / 32);
        }
        for (int q = 0; q < WC_ISSUERS; q++) mbar_init(mma_done(q), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tmem_slot)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    const u32 tmem = *(volatile u32*)tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            const int my_tiles = sched.starve ? 0 : T;
            int issued = 0, zissued = 0;
            size_t a_tile = 0;  // the unit's first key tile
            for (int kt = 0; kt < my_tiles; kt++) {
                const int lu = kt / GM_CHUNK_TILES, jl = kt % GM_CHUNK_TILES;
                if (jl == 0) {  // the unit's witness bytes: 16 ring columns of each valid witness
                    const int zb = lu & 1;
                    if (!mbar_wait(zempty(zb), ((lu >> 1) & 1) ^ 1, err, 1, lim)) break;
                    const int b0 = unit_b0(lu);
                    const u64 j0 = unit_j0(lu);
                    a_tile = (size_t)unit_mt(lu) * k_tiles + j0;
                    const u32 nb = (u32)(min((u64)GM_CHUNK_TILES, n_ring - j0) * AJ_D);
                    const int nw = min(WC_WIT, B - b0);
                    mbar_expect_tx(zfull(zb), nb * (u32)nw);
                    for (int w = 0; w < nw; w++)
                        bulk_load(smem_u32(zs + zb * WC_ZUNIT + w * (GM_CHUNK_TILES * AJ_D)),
                                  z + (size_t)(b0 + w) * (n_ring * AJ_D) + j0 * AJ_D, nb, zfull(zb));
                    zissued = lu + 1;
                }
                const int s = kt % WC_STAGES;
                if (!mbar_wait(empty(s), ((kt / WC_STAGES) & 1) ^ 1, err, 1, lim)) break;
                mbar_expect_tx(full(s), WC_A_BYTES);
                bulk_load(smem_u32(smem + s * WC_STAGE_BYTES),
                          A_tiled + (a_tile + jl) * (WC_A_BYTES / 2), WC_A_BYTES,
                          full(s));
                issued = kt + 1;
            }
            // copies still in flight land in shared memory before the CTA exits
            for (int kt = issued - WC_STAGES < 0 ? 0 : issued - WC_STAGES; kt < issued; kt++)
                mbar_wait(full(kt % WC_STAGES), (kt / WC_STAGES) & 1, err, 5, lim);
            for (int lu = zissued - 2 < 0 ? 0 : zissued - 2; lu < zissued; lu++)
                mbar_wait(zfull(lu & 1), (lu >> 1) & 1, err, 5, lim);
        }
    } else if (warp == 1 || warp == 18) {
        const int iss = warp == 1 ? 0 : 1;  // issues the MMAs of witnesses 2 iss, 2 iss + 1
        if (lane == 0) {
            bool ok = true;
            for (int c = 0; c < chunks && ok; c++) {
                const int a = c & 1;
                if (!mbar_wait(acc_empty(a), ((c >> 1) & 1) ^ 1, err, 2, lim)) break;
                // this issuer's witnesses of the tile: [w_lo, w_hi), possibly none in the last tile
                const int w_lo = 2 * iss, w_hi = min(min(WC_WIT, B - unit_b0(c)), w_lo + 2);
                asm volatile("tcgen05.fence::after_thread_sync;");
                for (int t = 0; t < GM_CHUNK_TILES; t++) {
                    const int kt = c * GM_CHUNK_TILES + t, s = kt % WC_STAGES;
                    const u32 ph = (kt / WC_STAGES) & 1;
                    if (!mbar_wait(full(s), ph, err, 3, lim) || !mbar_wait(ready(s), ph, err, 3, lim)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;");
                    const u32 sa = smem_u32(smem + s * WC_STAGE_BYTES);
                    const u64 adesc = umma_desc_sw128(sa);
                    // K step k, witness w: 32 bytes along the swizzled key rows, two core matrices
                    // (256 bytes) along the circulant
                    auto mma = [&](int k, int w) {
                        const u32 acc = (t > 0 || k > 0) ? 1u : 0u;
                        const u64 ad = adesc + (u64)((k * 32) >> 4);
                        const u64 bd = umma_desc_circ(sa + WC_A_BYTES + w * WC_WIN_BYTES + k * 256);
                        asm volatile(
                            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(
                                tmem + (u32)(a * WC_BN + w * AJ_D)),
                            "l"(ad), "l"(bd), "r"(WC_IDESC), "r"(acc));
                    };
                    if (w_hi == w_lo + 2) {  // both witnesses: the issue sequence fully unrolled
#pragma unroll
                        for (int k = 0; k < GM_BK / 16; k++) {
                            mma(k, w_lo);
                            mma(k, w_lo + 1);
                        }
                    } else if (w_hi > w_lo) {
#pragma unroll
                        for (int k = 0; k < GM_BK / 16; k++) mma(k, w_lo);
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                        empty(s)));
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    acc_full(a)));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                mma_done(iss)));
            mbar_wait(mma_done(iss), 0, err, 6, lim);
        }
    } else {
        // Group g = (warp - 2) / 4 of four warps (one per TMEM lane quarter) builds the stages
        // kt = g (mod 4), so that four stages are built at once; every warp also drains its
        // (lane quarter, witness g) block of the accumulators.
        const int quarter = warp & 3, g = (warp - 2) >> 2, row = quarter * 32 + lane;
        // build tasks of this thread: core-matrix rows row + 128 q (q < 4) of the stage's 480; row
        // crow of witness bw holds entries u .. u + 7 (u = crow + 1) of
        //   Gs[x] = 128 - z[x] (x < 64),  z[x - 64] - 128 (x >= 64):
        // bytes z[(u + e) mod 64], the first nneg of them negated.
        int acc[AJ_D];
#pragma unroll
        for (int q = 0; q < AJ_D; q++) acc[q] = 0;
        auto drain = [&](int c) -> bool {
            const int a = c & 1;
            if (!mbar_wait(acc_full(a), (c >> 1) & 1, err, 4, lim)) return false;
            asm volatile("tcgen05.fence::after_thread_sync;");
            const bool live = g < B - unit_b0(c);  // this warp's witness is in the batch (warp-uniform)
#pragma unroll
            for (int cb = 0; cb < AJ_D; cb += 8) {
                if (!live) break;
                u32 v[8];
                const u32 taddr = tmem + ((u32)(quarter * 32) << 16) + (u32)(a * WC_BN + g * AJ_D + cb);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                             : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                               "=r"(v[7])
                             : "r"(taddr));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int e = 0; e < 8; e++) acc[cb + e] += __float2int_rn(__uint_as_float(v[e]));
            }
            asm volatile("tcgen05.fence::before_thread_sync;");
            __syncwarp();
            if (lane == 0) mbar_arrive(acc_empty(a));
            const long long t = unit_tile(c);
            if (c + 1 == chunks || unit_tile(c + 1) != t) {  // this CTA's last unit of the tile
                const int k = (int)blockIdx.x - gm_cta_of(sched, t * sched.chunks);
                int* dst = S + (((size_t)t * sched.slots + k) * GM_BM + row) * WC_BN + g * AJ_D;
#pragma unroll
                for (int q = 0; q < AJ_D; q += 4) {
                    *reinterpret_cast<int4*>(dst + q) = make_int4(acc[q], acc[q + 1], acc[q + 2], acc[q + 3]);
                    acc[q] = acc[q + 1] = acc[q + 2] = acc[q + 3] = 0;
                }
            }
            return true;
        };
        bool ok = true;
        int ntask = 0;  // core-matrix rows to build per stage in the current unit
        for (int kt = g; kt < T && ok; kt += 4) {
            const int lu = kt / GM_CHUNK_TILES, jl = kt % GM_CHUNK_TILES, s = kt % WC_STAGES;
            if (jl == g) {  // this group's first stage of the unit
                if (!mbar_wait(zfull(lu & 1), (lu >> 1) & 1, err, 4, lim)) break;
                ntask = min(WC_WIT, B - unit_b0(lu)) * WC_ROWS_W;  // the tile's witnesses only
            }
            // the MMAs of this stage's previous use are done with its circulants
            if (!mbar_wait(empty(s), ((kt / WC_STAGES) & 1) ^ 1, err, 4, lim)) break;
            const uint8_t* zu = zs + (lu & 1) * WC_ZUNIT + jl * AJ_D;
            uint8_t* bst = smem + s * WC_STAGE_BYTES + WC_A_BYTES;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int task = row + 128 * q;
                if (task >= ntask) continue;
                const int bw = task / WC_ROWS_W, crow = task - bw * WC_ROWS_W, u = crow + 1;
                const int w0 = (u >> 3) & 7, nneg = min(8, max(0, 64 - u)), sh = (u & 7) * 8;
                const uint8_t* zw = zu + bw * (GM_CHUNK_TILES * AJ_D);
                const u64 lo = *reinterpret_cast<const u64*>(zw + 8 * w0);
                const u64 hi = *reinterpret_cast<const u64*>(zw + 8 * ((w0 + 1) & 7));
                const u64 x = sh ? (lo >> sh) | (hi << (64 - sh)) : lo;
                u32 pk[4];
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    const int b0 = (int)((x >> (16 * e)) & 255), b1 = (int)((x >> (16 * e + 8)) & 255);
                    pk[e] = bf16x2_of(2 * e < nneg ? 128 - b0 : b0 - 128, 2 * e + 1 < nneg ? 128 - b1 : b1 - 128);
                }
                asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(smem_u32(bst + bw * WC_WIN_BYTES + crow * 16)), "r"(pk[0]),
                             "r"(pk[1]), "r"(pk[2]), "r"(pk[3])
                             : "memory");
            }
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the tensor core
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(ready(s));
                if (jl >= GM_CHUNK_TILES - 4) mbar_arrive(zempty(lu & 1));  // the group's last stage of the unit
            }
            if (jl == WC_LAG + g && lu >= 1 && !drain(lu - 1)) ok = false;
        }
        if (ok && chunks > 0) drain(chunks - 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// c[b][i][r] = sum_p 256^p S[16 p + (i mod 16)][(b mod 4) 64 + r] + 128 rowsum[i][r]  mod q,
// canonical; S summed over the slots of tile (b / 4, i / 16).  A block takes 32 consecutive
// outputs (consecutive r): warp p sums digit plane p over the slots (coalesced along r, four loads
// in flight), and warp 0 combines the planes.  A small batch spreads one tile's K chunks over
// many CTAs (64 slots for one witness), so the slot sums are the combine's work.
__global__ void __launch_bounds__(256) ajtai_combine_wc_kernel(const int* __restrict__ S, GmSched sched, int rows,
                                                               int B, const u64* __restrict__ RS,
                                                               u64* __restrict__ out) {
    __shared__ long long part[8][32];
    const int IR = rows * AJ_D;
    const int p = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t o = (size_t)blockIdx.x * 32 + lane;  // output b IR + ir
    const bool valid = o < (size_t)B * IR;
    const int b = valid ? (int)(o / IR) : 0, ir = valid ? (int)(o % IR) : 0, i = ir / AJ_D, r = ir % AJ_D;
    long long sum = 0;
    if (valid) {
        const long long tile = (long long)(b / WC_WIT) * sched.tiles_m + i / 16;
        const int ns = gm_cta_of(sched, (tile + 1) * sched.chunks - 1) - gm_cta_of(sched, tile * sched.chunks) + 1;
        const int* base = S + ((size_t)tile * sched.slots * GM_BM + 16 * p + (i & 15)) * WC_BN + (b % WC_WIT) * AJ_D + r;
        const size_t stride = (size_t)GM_BM * WC_BN;  // one slot
        long long s0 = 0, s1 = 0, s2 = 0, s3 = 0;  // |total over the slots| <= 2^30
        int k = 0;
        for (; k + 4 <= ns; k += 4) {
            s0 += __ldg(base + (size_t)k * stride);
            s1 += __ldg(base + (size_t)(k + 1) * stride);
            s2 += __ldg(base + (size_t)(k + 2) * stride);
            s3 += __ldg(base + (size_t)(k + 3) * stride);
        }
        for (; k < ns; k++) s0 += __ldg(base + (size_t)k * stride);
        sum = s0 + s1 + s2 + s3;
    }
    part[p][lane] = sum;
    __syncthreads();
    if (p == 0 && valid) {
        __int128 acc = 0;
#pragma unroll
        for (int q = 7; q >= 0; q--) acc = acc * 256 + (__int128)part[q][lane];
        const u64 rs128 = agl_mul(__ldg(RS + ir), 128);
        out[o] = agl_canon(agl_add(agl_from_i128(acc), agl_canon(rs128)));
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// The driver's tensor-map encoder, resolved at run time so that loading the library
// needs no driver (CPU-only hosts load it to check its exports).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// 2D bf16 tensor map, inner dimension contiguous, 64 x box_rows boxes with 128-byte swizzle
static int make_map(CUtensorMap* map, void* base, u64 inner, u64 outer, u32 box_rows) {
    static const EncodeTiledFn encode = [] {  // resolved once (thread-safe static init)
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess)
            fn = nullptr;
        return (EncodeTiledFn)fn;
    }();
    if (!encode) {
        set_error_msg("cuTensorMapEncodeTiled is not available from the driver");
        return GB_ECUDA;
    }
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * 2};
    cuuint32_t box[2] = {GM_BK, box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error_msg("cuTensorMapEncodeTiled failed");
        return GB_ECUDA;
    }
    return GB_OK;
}

// Key-dependent operand: digit-expanded Toeplitz matrix and row sums.
struct AjtaiKey {
    u32 seed[8];
    int row_lo = 0, rows = 0;
    u64 N = 0;        // ring columns
    size_t K = 0, Kp = 0;
    u64* d_M = nullptr;              // [rows][N][64]
    __nv_bfloat16* d_T = nullptr;    // 8 * rows * 64 x Kp, tile by tile (ajtai_expand_kernel); built
                                     // by the first batch that takes the key-Toeplitz form
    __nv_bfloat16* d_A = nullptr;    // ceil(rows / 16) * 128 x Kp, tile by tile (ajtai_planes_kernel)
    uint8_t* d_W = nullptr;          // the Hankel windows, 3840 B per (128-row tile, ring column)
                                     // (ajtai_window_kernel); built by the first batch that needs them
    u64* d_RS = nullptr;             // [rows][64]
    std::once_flag t_once;           // the expansion's one build (any thread may commit)
    int t_rc = GB_OK;                // its outcome
    std::string t_err;
    std::once_flag w_once;           // the windows' one build
    int w_rc = GB_OK;
    std::string w_err;
};

static size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

static int key_create(const u32* h_seed, int row_lo, int rows, u64 N, AjtaiKey* k) {
    if (rows < 1 || N < 1 || N > (1ull << 24)) return GB_EINVAL;
    cudaStream_t s = stream();
    for (int q = 0; q < 8; q++) k->seed[q] = h_seed[q];
    k->row_lo = row_lo;
    k->rows = rows;
    k->N = N;
    k->K = (size_t)N * AJ_D;
    k->Kp = round_up(k->K, (size_t)GM_BK * GM_CHUNK_TILES);
    u32* d_key = nullptr;
    GB_CUDA_TRY(cudaMalloc(&k->d_M, (size_t)rows * N * AJ_D * 8));
    GB_CUDA_TRY(cudaMalloc(&k->d_RS, (size_t)rows * AJ_D * 8));
    GB_CUDA_TRY(cudaMallocAsync(&d_key, 32, s));
    GB_CUDA_TRY(cudaMemcpyAsync(d_key, h_seed, 32, cudaMemcpyHostToDevice, s));
    size_t tasks = (size_t)rows * N * 8;
    ajtai_prg_kernel<<<grid_for(tasks, 256), 256, 0, s>>>(d_key, row_lo, rows, 0, N, k->d_M);
    GB_LAUNCH_CHECK("ajtai_prg_kernel");
    dim3 g((unsigned)N, (unsigned)rows);
    {
        const size_t tiles_m = (size_t)(rows + 15) / 16;
        GB_CUDA_TRY(cudaMalloc(&k->d_A, tiles_m * GM_BM * k->Kp * 2));
        GB_CUDA_TRY(cudaMemsetAsync(k->d_A, 0, tiles_m * GM_BM * k->Kp * 2, s));
        ajtai_planes_kernel<<<g, 64, 0, s>>>(k->d_M, N, k->Kp / GM_BK, k->d_A);
        GB_LAUNCH_CHECK("ajtai_planes_kernel");
    }
    ajtai_rowsum_kernel<<<rows, 256, 0, s>>>(k->d_M, N, k->d_RS);
    GB_LAUNCH_CHECK("ajtai_rowsum_kernel");
    cudaFreeAsync(d_key, s);
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
}

// The key-Toeplitz form's operand: the digit-expanded Toeplitz matrix of the key's rows, 1.07 GB
// for 16 rows x 1024 ring columns.  Built once, on the calling thread's stream, by the first batch
// that needs it; later calls (from any thread) wait for that build and reuse it.
static int key_expand(AjtaiKey* k) {
    std::call_once(k->t_once, [k] {
        cudaStream_t s = stream();
        const size_t bytes = (size_t)8 * k->rows * AJ_D * k->Kp * 2;
        int rc = GB_OK;
        cudaError_t e = cudaMalloc(&k->d_T, bytes);
        if (e == cudaSuccess && k->Kp > k->K) e = cudaMemsetAsync(k->d_T, 0, bytes, s);  // the padding tiles
        if (e == cudaSuccess) {
            dim3 g((unsigned)k->N, (unsigned)k->rows);
            ajtai_expand_kernel<<<g, 64, 0, s>>>(k->d_M, k->rows, k->N, k->Kp / GM_BK, k->d_T);
            rc = check_launch("ajtai_expand_kernel");
            if (!rc) e = cudaStreamSynchronize(s);
        }
        if (e != cudaSuccess) {
            set_error("ajtai key expansion", e);
            rc = GB_ECUDA;
        }
        k->t_rc = rc;
        if (rc) k->t_err = gb_last_error();
    });
    if (k->t_rc) set_error_msg(k->t_err);
    return k->t_rc;
}

// The Hankel form's operand: the key's windows, 252 MB for 16 rows x 1024 ring columns (a quarter
// of the expansion).  Built once, like the expansion, by the first batch that needs it.
static int key_window(AjtaiKey* k) {
    std::call_once(k->w_once, [k] {
        cudaStream_t s = stream();
        const size_t KT = k->Kp / GM_BK;
        const size_t bytes = (size_t)4 * k->rows * KT * GW_A_BYTES;  // 8 rows x 64 / 128 tiles per ring row
        int rc = GB_OK;
        cudaError_t e = cudaMalloc(&k->d_W, bytes);
        if (e == cudaSuccess && k->Kp > k->K) e = cudaMemsetAsync(k->d_W, 0, bytes, s);  // the padding columns
        if (e == cudaSuccess) {
            dim3 g((unsigned)k->N, (unsigned)k->rows);
            ajtai_window_kernel<<<g, 128, 0, s>>>(k->d_M, k->rows, k->N, KT, k->d_W);
            rc = check_launch("ajtai_window_kernel");
            if (!rc) e = cudaStreamSynchronize(s);
        }
        if (e != cudaSuccess) {
            set_error("ajtai key windows", e);
            rc = GB_ECUDA;
        }
        k->w_rc = rc;
        if (rc) k->w_err = gb_last_error();
    });
    if (k->w_rc) set_error_msg(k->w_err);
    return k->w_rc;
}

static void key_free(AjtaiKey* k) {
    if (k->d_M) cudaFree(k->d_M);
    if (k->d_W) cudaFree(k->d_W);
    if (k->d_T) cudaFree(k->d_T);
    if (k->d_A) cudaFree(k->d_A);
    if (k->d_RS) cudaFree(k->d_RS);
    k->d_M = nullptr;
    k->d_T = nullptr;
    k->d_W = nullptr;
    k->d_A = nullptr;
    k->d_RS = nullptr;
}

// Test switch of the calling thread: the next GEMMs run starved (no operand loads, short wait
// limits), so that their bounded waits run out and the call reports it; see gb_ajtai_test_starve.
static thread_local int t_starve = 0;

// Waits for the calling thread's stream and reads the device word at d (the GEMMs' wait-error
// flag) through the thread's pinned staging, a plain DMA (a pageable destination would add a
// staged copy to every call).
static int read_flag(const int* d, int* out) {
    cudaStream_t s = stream();
    u64* pin = thread_pinned(2, 1);
    if (!pin) {
        set_error_msg("ajtai: no pinned staging for the error flag");
        return GB_ECUDA;
    }
    *reinterpret_cast<volatile int*>(pin) = 0;
    if (cudaMemcpyAsync(pin, d, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        return GB_ECUDA;
    *out = *reinterpret_cast<volatile int*>(pin);
    return GB_OK;
}

// Witness-circulant GEMM: one persistent launch over the (tile, 1024-deep chunk) units, tile =
// (4 witnesses, 16 ring rows), then the combine.
static int commit_batch_wc(AjtaiKey* k, const uint8_t* d_z, int B, u64* d_out) {
    cudaStream_t s = stream();
    GmSched sched;
    sched.tiles_m = (k->rows + 15) / 16;
    sched.chunks = (int)(k->Kp / ((size_t)GM_BK * GM_CHUNK_TILES));
    const long long tiles = (long long)sched.tiles_m * ((B + WC_WIT - 1) / WC_WIT);
    sched.units = tiles * sched.chunks;
    sched.ctas = (int)std::min<long long>(num_sms(), sched.units);
    sched.slots = 1;
    sched.starve = t_starve;
    sched.spin_limit = t_starve ? GM_SPIN_LIMIT_TEST : GM_SPIN_LIMIT;
    for (long long t = 0; t < tiles; t++)
        sched.slots = std::max(sched.slots, gm_cta_of(sched, (t + 1) * sched.chunks - 1) -
                                                gm_cta_of(sched, t * sched.chunks) + 1);
    const size_t s_ints = (size_t)tiles * sched.slots * GM_BM * WC_BN;
    uint8_t* zal = nullptr;
    int* S = nullptr;
    int* err = nullptr;
    if ((uintptr_t)d_z & 15) {  // the bulk copies read 16-byte aligned rows: realign the batch once
        GB_CUDA_TRY(cudaMallocAsync(&zal, (size_t)B * k->K, s));
        GB_CUDA_TRY(cudaMemcpyAsync(zal, d_z, (size_t)B * k->K, cudaMemcpyDeviceToDevice, s));
        d_z = zal;
    }
    GB_CUDA_TRY(cudaMallocAsync(&S, s_ints * 4, s));
    GB_CUDA_TRY(cudaMallocAsync(&err, 4, s));
    GB_CUDA_TRY(cudaMemsetAsync(err, 0, 4, s));
    // set on every call: idempotent, per device, and free of shared state between threads
    cudaFuncSetAttribute(ajtai_gemm_wc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, WC_SMEM);
    ajtai_gemm_wc_kernel<<<sched.ctas, WC_THREADS, WC_SMEM, s>>>(k->d_A, d_z, B, k->N, (int)(k->Kp / GM_BK), sched,
                                                                S, err);
    int rc = check_launch("ajtai_gemm_wc_kernel");
    if (!rc) {
        ajtai_combine_wc_kernel<<<grid_for((size_t)B * k->rows * AJ_D, 32), 256, 0, s>>>(S, sched, k->rows, B,
                                                                                      k->d_RS, d_out);
        rc = check_launch("ajtai_combine_wc_kernel");
    }
    int h_err = 0;
    if (!rc) rc = read_flag(err, &h_err);
    if (zal) cudaFreeAsync(zal, s);
    cudaFreeAsync(S, s);
    cudaFreeAsync(err, s);
    if (!rc && h_err) {
        set_error_msg("ajtai_gemm_wc_kernel: pipeline wait timed out (code " + std::to_string(h_err) + ")");
        rc = GB_ECUDA;
    }
    return rc;
}

// Form of the calling thread's batched commitments (gb_ajtai_set_batch_form): 0 by batch size,
// 1 the witness-circulant GEMM, 2 the key-Toeplitz GEMM, 3 the key-Toeplitz GEMM on CTA pairs,
// 4 the same pair GEMM reading the key's Hankel windows (a quarter of the expansion's bytes).
// Results never depend on it.
static thread_local int t_batch_form = 0;
// Largest batch that the automatic choice gives the witness-circulant GEMM.  Its work grows with
// the batch (one N = 64 MMA per witness and K step), while the pair GEMM streams the key's
// operand (its Hankel windows) whatever the batch; larger batches take the CTA-pair GEMM on
// the windows.  The two measured level near 105 witnesses (16 rows x 1024 ring columns: 0.169
// against 0.179 ms at 96, 0.185 against 0.180 ms at 112).
constexpr int AJ_WC_MAX_AUTO = 104;

// Launch shape of the pair GEMM: a cluster of 2 CTAs, GpShape<HANKEL>::SMEM bytes each.
template <bool HANKEL>
static cudaLaunchConfig_t pair_config(int clusters, cudaStream_t s, cudaLaunchAttribute* attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(2 * clusters));
    cfg.blockDim = dim3(GM_THREADS);
    cfg.dynamicSmemBytes = GpShape<HANKEL>::SMEM;
    cfg.stream = s;
    attr->id = cudaLaunchAttributeClusterDimension;
    attr->val.clusterDim.x = 2;
    attr->val.clusterDim.y = 1;
    attr->val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

// CTA pairs that the device runs at once (0 when clusters of two cannot run the pair GEMM).  The
// shared-memory attribute is set on every call (idempotent, per device); the occupancy answer
// depends only on the device and is kept per device (a race only recomputes the same value).
template <bool HANKEL>
static int pair_clusters() {
    if (cudaFuncSetAttribute(ajtai_gemm_pair_kernel<HANKEL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             GpShape<HANKEL>::SMEM) != cudaSuccess)
        return 0;
    constexpr int MAX_DEVICES = 64;
    static std::atomic<int> known[MAX_DEVICES];  // 0: not yet asked, else clusters + 1
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (dev >= 0 && dev < MAX_DEVICES) {
        const int k = known[dev].load(std::memory_order_relaxed);
        if (k > 0) return k - 1;
    }
    cudaLaunchAttribute attr;
    cudaLaunchConfig_t cfg = pair_config<HANKEL>(1, stream(), &attr);
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, ajtai_gemm_pair_kernel<HANKEL>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;  // not kept: a later call asks again
    }
    if (dev >= 0 && dev < MAX_DEVICES) known[dev].store(n + 1, std::memory_order_relaxed);
    return n;
}

static int commit_batch(AjtaiKey* k, const uint8_t* d_z, int B, u64* d_out) {
    if (B < 1) return GB_EINVAL;
    int form = t_batch_form ? t_batch_form : (B <= AJ_WC_MAX_AUTO ? 1 : 4);
    if (form == 1) return commit_batch_wc(k, d_z, B, d_out);
    // forms 3 and 4: CTA pairs, 256-row tiles; the device must run clusters of two at this size
    // (the automatic choice falls back to the one-CTA form when it cannot)
    const int clusters = form == 3 ? pair_clusters<false>() : form == 4 ? pair_clusters<true>() : 0;
    if (form >= 3 && clusters < 1 && t_batch_form == 0) form = 2;
    if (form >= 3 && clusters < 1) {
        set_error_msg("ajtai pair GEMM: the device runs no cluster of two CTAs of this size");
        return GB_ECUDA;
    }
    const bool hankel = form == 4;
    if (int rc = hankel ? key_window(k) : key_expand(k)) return rc;
    cudaStream_t s = stream();
    const int Bp = (int)round_up((size_t)B, GM_BN);
    const size_t Mrows = (size_t)8 * k->rows * AJ_D;
    const int pair = form >= 3 ? 1 : 0;
    // persistent schedule: one CTA (pair) per SM (pair), or per unit when there are fewer, equal unit ranges
    GmSched sched;
    sched.pair = pair;
    sched.tiles_m = (int)(Mrows / (GM_BM << pair));
    sched.chunks = (int)(k->Kp / ((size_t)GM_BK * GM_CHUNK_TILES));
    const long long tiles = (long long)sched.tiles_m * (Bp / GM_BN);
    sched.units = tiles * sched.chunks;
    sched.ctas = (int)std::min<long long>(pair ? clusters : num_sms(), sched.units);
    sched.slots = 1;
    sched.starve = t_starve;
    sched.spin_limit = t_starve ? GM_SPIN_LIMIT_TEST : GM_SPIN_LIMIT;
    for (long long t = 0; t < tiles; t++)
        sched.slots = std::max(sched.slots, gm_cta_of(sched, (t + 1) * sched.chunks - 1) -
                                                gm_cta_of(sched, t * sched.chunks) + 1);
    const size_t s_ints = ((size_t)tiles << pair) * sched.slots * GM_BM * GM_BN;
    __nv_bfloat16* zc = nullptr;
    int* S = nullptr;
    int* err = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&zc, (size_t)Bp * k->Kp * 2, s));
    GB_CUDA_TRY(cudaMallocAsync(&S, s_ints * 4, s));
    GB_CUDA_TRY(cudaMallocAsync(&err, 4, s));
    GB_CUDA_TRY(cudaMemsetAsync(err, 0, 4, s));
    // the Hankel form reads the witnesses with K reversed inside each ring column
    const unsigned g8 = grid_for((size_t)Bp * (k->Kp / 8), 256), g1 = grid_for((size_t)Bp * k->Kp, 256);
    if (((uintptr_t)d_z & 7) == 0) {
        if (hankel)
            ajtai_zprep_kernel<true><<<g8, 256, 0, s>>>(d_z, B, k->K, Bp, k->Kp, zc);
        else
            ajtai_zprep_kernel<false><<<g8, 256, 0, s>>>(d_z, B, k->K, Bp, k->Kp, zc);
    } else {
        if (hankel)
            ajtai_zprep_scalar_kernel<true><<<g1, 256, 0, s>>>(d_z, B, k->K, Bp, k->Kp, zc);
        else
            ajtai_zprep_scalar_kernel<false><<<g1, 256, 0, s>>>(d_z, B, k->K, Bp, k->Kp, zc);
    }
    int rc = check_launch("ajtai_zprep_kernel");
    CUtensorMap mapB;
    if (!rc) rc = make_map(&mapB, zc, k->Kp, (u64)Bp, pair ? GP_BN_HALF : GM_BN);
    const int k_tiles = (int)(k->Kp / GM_BK);
    if (!rc && pair) {
        cudaLaunchAttribute attr;
        cudaError_t e;
        if (hankel) {
            cudaLaunchConfig_t cfg = pair_config<true>(sched.ctas, s, &attr);
            e = cudaLaunchKernelEx(&cfg, ajtai_gemm_pair_kernel<true>, (const uint8_t*)k->d_W, mapB, k_tiles, sched, S,
                                   err);
        } else {
            cudaLaunchConfig_t cfg = pair_config<false>(sched.ctas, s, &attr);
            e = cudaLaunchKernelEx(&cfg, ajtai_gemm_pair_kernel<false>, (const uint8_t*)k->d_T, mapB, k_tiles, sched, S,
                                   err);
        }
        rc = check_launch("ajtai_gemm_pair_kernel");
        if (!rc && e != cudaSuccess) {
            set_error("ajtai_gemm_pair_kernel", e);
            rc = GB_ECUDA;
        }
    } else if (!rc) {
        // set on every call: idempotent, per device, and free of shared state between threads
        cudaFuncSetAttribute(ajtai_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, GM_SMEM);
        ajtai_gemm_kernel<<<sched.ctas, GM_THREADS, GM_SMEM, s>>>(k->d_T, mapB, k_tiles, sched, S, err);
        rc = check_launch("ajtai_gemm_kernel");
    }
    if (!rc) {
        dim3 cg((unsigned)((B + AJ_CB - 1) / AJ_CB), (unsigned)((k->rows * AJ_D + AJ_CR - 1) / AJ_CR));
        ajtai_combine_kernel<<<cg, 256, 0, s>>>(S, sched, k->rows, B, k->d_RS, d_out);
        rc = check_launch("ajtai_combine_kernel");
    }
    int h_err = 0;
    if (!rc) rc = read_flag(err, &h_err);
    cudaFreeAsync(zc, s);
    cudaFreeAsync(S, s);
    cudaFreeAsync(err, s);
    if (!rc && h_err) {
        set_error_msg(std::string(pair ? "ajtai_gemm_pair_kernel" : "ajtai_gemm_kernel") +
                      ": pipeline wait timed out (code " + std::to_string(h_err) + ")");
        rc = GB_ECUDA;
    }
    return rc;
}

// ---------------------------------------------------------------------------
// full-width commitment on the CUDA cores (reference ABI):
// thread (i, r) of column chunk accumulates sum_j sum_l s(r,l) M[i][j][(r-l) mod 64] z_j[l].
// One block per (chunk, row tile of 8 rows); the block generates the matrix columns it
// needs into shared memory, as the reference kernel does, then every thread runs the
// negacyclic dot product with modular multiplications.
// ---------------------------------------------------------------------------
constexpr int WIDE_ROWS = 8;
constexpr int WIDE_CHUNK = 16;  // columns per block

__global__ void __launch_bounds__(WIDE_ROWS * AJ_D) ajtai_wide_kernel(const u32* __restrict__ key,
                                                                    const u64* __restrict__ z, u64 N, u64 col_offset,
                                                                    u64* __restrict__ partial, int nchunks) {
    __shared__ u64 Msh[WIDE_ROWS * AJ_D];
    __shared__ u64 zsh[AJ_D];
    __shared__ u32 ksh[8];
    const int t = threadIdx.x, il = t / AJ_D, r = t % AJ_D;
    const int chunk = blockIdx.x, tile = blockIdx.y;
    const int row = tile * WIDE_ROWS + il;
    if (t < 8) ksh[t] = key[t];
    __syncthreads();
    u64 acc = 0;
    u64 j0 = (u64)chunk * WIDE_CHUNK, j1 = j0 + WIDE_CHUNK < N ? j0 + WIDE_CHUNK : N;
    for (u64 j = j0; j < j1; j++) {
        if (t < AJ_D) zsh[t] = z[j * AJ_D + t];
        if (t < WIDE_ROWS * 8) {
            int rl = t / 8, blk = t % 8;
            int rr = tile * WIDE_ROWS + rl;
            u64 out[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (rr < AJ_KAPPA) ajtai_prg_block(ksh, (u32)rr, j + col_offset, (u32)blk, out);
#pragma unroll
            for (int q = 0; q < 8; q++) Msh[rl * AJ_D + blk * 8 + q] = out[q];
        }
        __syncthreads();
        if (row < AJ_KAPPA) {
            const u64* m = Msh + il * AJ_D;
            for (int l = 0; l <= r; l++) acc = agl_add(acc, agl_mul(m[r - l], zsh[l]));
            for (int l = r + 1; l < AJ_D; l++) acc = agl_sub(acc, agl_mul(m[r - l + AJ_D], zsh[l]));
        }
        __syncthreads();
    }
    if (row < AJ_KAPPA) partial[((size_t)chunk * AJ_KAPPA + row) * AJ_D + r] = acc;
}

__global__ void ajtai_wide_reduce_kernel(const u64* __restrict__ partial, int nchunks, u64* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= AJ_KAPPA * AJ_D) return;
    u64 acc = 0;
    for (int c = 0; c < nchunks; c++) acc = agl_add(acc, partial[(size_t)c * AJ_KAPPA * AJ_D + t]);
    out[t] = agl_canon(acc);
}

// ---------------------------------------------------------------------------
// Set-bit commitments of small-coefficient witnesses (reference ABI): binary batches
// (commit_dense_batched_kernel, ajtai.cuh:82-162), ternary pos/neg bitmasks and sparse
// position lists (commit_sparse_partial_kernel, ajtai.cuh:382-440).  Same tiling as the
// wide kernel (8 matrix rows x 64 coefficients per block, the rows' column generated into
// shared memory); each set coefficient l of column j adds s(r, l) M[i][j][(r - l) mod 64].
// ---------------------------------------------------------------------------
constexpr int BITS_MAX_B = 16;

__device__ __forceinline__ void wide_fill_rows(const u32* ksh, int tile, u64 j, u64* Msh, int t) {
    if (t < WIDE_ROWS * 8) {
        int rl = t / 8, blk = t % 8;
        int rr = tile * WIDE_ROWS + rl;
        u64 out[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (rr < AJ_KAPPA) ajtai_prg_block(ksh, (u32)rr, j, (u32)blk, out);
#pragma unroll
        for (int q = 0; q < 8; q++) Msh[rl * AJ_D + blk * 8 + q] = out[q];
    }
}

// pos/neg: [B][N] bitmasks (neg may be null); partial [chunk][B][KAPPA][D].  With Mg (a
// materialized matrix [N][KAPPA][64], ajtai_materialize_m_ffi) the rows are read from it
// instead of being generated.
__global__ void __launch_bounds__(WIDE_ROWS * AJ_D) ajtai_bits_kernel(const u32* __restrict__ key,
                                                                    const u64* __restrict__ pos,
                                                                    const u64* __restrict__ neg, u64 N, int B,
                                                                    u64 col_offset, u64* __restrict__ partial,
                                                                    const u64* __restrict__ Mg) {
    __shared__ u64 Msh[WIDE_ROWS * AJ_D];
    __shared__ u64 psh[BITS_MAX_B], nsh[BITS_MAX_B];
    __shared__ u32 ksh[8];
    const int t = threadIdx.x, il = t / AJ_D, r = t % AJ_D;
    const int chunk = blockIdx.x, tile = blockIdx.y, row = tile * WIDE_ROWS + il;
    if (t < 8 && !Mg) ksh[t] = key[t];
    u64 acc[BITS_MAX_B];
#pragma unroll
    for (int b = 0; b < BITS_MAX_B; b++) acc[b] = 0;
    __syncthreads();
    const u64 j0 = (u64)chunk * WIDE_CHUNK, j1 = j0 + WIDE_CHUNK < N ? j0 + WIDE_CHUNK : N;
    for (u64 j = j0; j < j1; j++) {
        if (t < B) {
            psh[t] = pos[(u64)t * N + j];
            nsh[t] = neg ? neg[(u64)t * N + j] : 0;
        }
        if (Mg) {
            const int rr = tile * WIDE_ROWS + il;
            Msh[t] = rr < AJ_KAPPA ? Mg[((j + col_offset) * AJ_KAPPA + rr) * AJ_D + r] : 0;
        } else {
            wide_fill_rows(ksh, tile, j + col_offset, Msh, t);
        }
        __syncthreads();
        const u64* m = Msh + il * AJ_D;
#pragma unroll
        for (int b = 0; b < BITS_MAX_B; b++) {
            if (b >= B) break;
            u64 mask = psh[b];
            while (mask) {
                int l = __ffsll((long long)mask) - 1;
                mask &= mask - 1;
                acc[b] = l <= r ? agl_add(acc[b], m[r - l]) : agl_sub(acc[b], m[r - l + AJ_D]);
            }
            mask = nsh[b];
            while (mask) {
                int l = __ffsll((long long)mask) - 1;
                mask &= mask - 1;
                acc[b] = l <= r ? agl_sub(acc[b], m[r - l]) : agl_add(acc[b], m[r - l + AJ_D]);
            }
        }
        __syncthreads();
    }
    if (row < AJ_KAPPA)
#pragma unroll
        for (int b = 0; b < BITS_MAX_B; b++) {
            if (b >= B) break;
            partial[(((size_t)chunk * B + b) * AJ_KAPPA + row) * AJ_D + r] = acc[b];
        }
}

// positions: K global coefficient indices p = 64 j + l of a binary witness (a repeated index
// counts twice); partial [chunk][KAPPA][D] over WIDE_CHUNK * 16 positions per chunk
constexpr int SPARSE_CHUNK = WIDE_CHUNK * 16;
__global__ void __launch_bounds__(WIDE_ROWS * AJ_D) ajtai_sparse_kernel(const u32* __restrict__ key,
                                                                      const u64* __restrict__ positions, u64 K,
                                                                      u64* __restrict__ partial) {
    __shared__ u64 Msh[WIDE_ROWS * AJ_D];
    __shared__ u32 ksh[8];
    const int t = threadIdx.x, il = t / AJ_D, r = t % AJ_D;
    const int chunk = blockIdx.x, tile = blockIdx.y, row = tile * WIDE_ROWS + il;
    if (t < 8) ksh[t] = key[t];
    __syncthreads();
    u64 acc = 0;
    u64 prev = ~(u64)0;
    const u64 k0 = (u64)chunk * SPARSE_CHUNK, k1 = k0 + SPARSE_CHUNK < K ? k0 + SPARSE_CHUNK : K;
    for (u64 k = k0; k < k1; k++) {
        const u64 p = positions[k], j = p >> 6;
        const int l = (int)(p & 63);
        if (j != prev) {  // the same for the whole block
            __syncthreads();
            wide_fill_rows(ksh, tile, j, Msh, t);
            __syncthreads();
            prev = j;
        }
        const u64* m = Msh + il * AJ_D;
        acc = l <= r ? agl_add(acc, m[r - l]) : agl_sub(acc, m[r - l + AJ_D]);
    }
    if (row < AJ_KAPPA) partial[((size_t)chunk * AJ_KAPPA + row) * AJ_D + r] = acc;
}

// out[b][i][r] = sum over chunks of partial[chunk][b][i][r], canonical
__global__ void ajtai_reduce_b_kernel(const u64* __restrict__ partial, int nchunks, int B, u64* __restrict__ out) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= B * AJ_KAPPA * AJ_D) return;
    u64 acc = 0;
    for (int c = 0; c < nchunks; c++) acc = agl_add(acc, partial[(size_t)c * B * AJ_KAPPA * AJ_D + t]);
    out[t] = agl_canon(acc);
}

static bool chunk_ok(int chunk) {
    return chunk == 64 || chunk == 128 || chunk == 256 || chunk == 1024 || chunk == 4096;
}

static int commit_bits(const u32* d_key, const u64* d_pos, const u64* d_neg, u64 N, int B, u64 col_offset,
                       u64* d_out, const char* name, const u64* d_M = nullptr) {
    if (N == 0 || B < 1 || B > BITS_MAX_B || !(d_key || d_M) || !d_pos || !d_out) return GB_EINVAL;
    cudaStream_t s = stream();
    const int nchunks = (int)((N + WIDE_CHUNK - 1) / WIDE_CHUNK);
    u64* partial = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&partial, (size_t)nchunks * B * AJ_KAPPA * AJ_D * 8, s));
    dim3 g((unsigned)nchunks, (unsigned)((AJ_KAPPA + WIDE_ROWS - 1) / WIDE_ROWS));
    ajtai_bits_kernel<<<g, WIDE_ROWS * AJ_D, 0, s>>>(d_key, d_pos, d_neg, N, B, col_offset, partial, d_M);
    int rc = check_launch(name);
    if (!rc) {
        ajtai_reduce_b_kernel<<<grid_for((size_t)B * AJ_KAPPA * AJ_D, 256), 256, 0, s>>>(partial, nchunks, B, d_out);
        rc = check_launch("ajtai_reduce_b_kernel");
    }
    cudaFreeAsync(partial, s);
    return rc ? rc : sync_stream(name);
}

}  // namespace gb

using namespace gb;

extern "C" {

int almost_goldilocks_cuda_init(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return -1;
    return cudaSetDevice(0) == cudaSuccess ? 0 : -1;
}

int ajtai_commit_wide_ffi(const uint32_t* d_key, const uint64_t* d_z_wide, uint64_t N, uint64_t col_offset, int chunk,
                          uint64_t* d_out) {
    // The reference accepts chunk sizes 64/128/256/1024/4096 (a tuning knob); any of them
    // gives the same commitment, so the value is validated and otherwise ignored.
    if (chunk != 64 && chunk != 128 && chunk != 256 && chunk != 1024 && chunk != 4096) return GB_EUNSUPPORTED;
    if (N == 0) return GB_EINVAL;
    cudaStream_t s = stream();
    int nchunks = (int)((N + WIDE_CHUNK - 1) / WIDE_CHUNK);
    u64* partial = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&partial, (size_t)nchunks * AJ_KAPPA * AJ_D * 8, s));
    dim3 g((unsigned)nchunks, (unsigned)((AJ_KAPPA + WIDE_ROWS - 1) / WIDE_ROWS));
    ajtai_wide_kernel<<<g, WIDE_ROWS * AJ_D, 0, s>>>(d_key, d_z_wide, N, col_offset, partial, nchunks);
    int rc = check_launch("ajtai_wide_kernel");
    if (!rc) {
        ajtai_wide_reduce_kernel<<<grid_for(AJ_KAPPA * AJ_D, 256), 256, 0, s>>>(partial, nchunks, d_out);
        rc = check_launch("ajtai_wide_reduce_kernel");
    }
    cudaFreeAsync(partial, s);
    if (rc) return rc;
    return sync_stream("ajtai_commit_wide_ffi");
}

}  // extern "C"

namespace gb {
// Scratch of ajtai_commit_wide_noalloc_ffi: the per-chunk partial commitments of at most
// AJ_NOALLOC_MAX_RING ring columns (256 chunks x 42 rows x 64 coefficients x 8 B = 5.25 MiB),
// in the module's static device memory so that the call allocates nothing.  Nothing in it has
// to start at zero: ajtai_wide_kernel writes every word that ajtai_wide_reduce_kernel reads.
constexpr u64 AJ_NOALLOC_MAX_RING = 4096;
constexpr int AJ_NOALLOC_MAX_CHUNKS = (int)(AJ_NOALLOC_MAX_RING / WIDE_CHUNK);
static __device__ __align__(256) u64 g_wide_noalloc_scratch[(size_t)AJ_NOALLOC_MAX_CHUNKS * AJ_KAPPA * AJ_D];

// Device address of the scratch on the current device.  It is looked up on every call (a host-side
// table lookup once the module is loaded), so no address outlives a context that a device reset
// tore down.
static int wide_noalloc_scratch(u64** out) {
    void* p = nullptr;
    GB_CUDA_TRY(cudaGetSymbolAddress(&p, g_wide_noalloc_scratch));
    *out = static_cast<u64*>(p);
    return GB_OK;
}
}  // namespace gb

extern "C" {

int ajtai_commit_wide_noalloc_ffi(const uint32_t* d_key, const uint64_t* d_z_wide, uint64_t N, uint64_t col_offset,
                                  int chunk, uint64_t* d_out) {
    if (chunk != 64 && chunk != 128 && chunk != 256 && chunk != 1024 && chunk != 4096) return GB_EUNSUPPORTED;
    if (N == 0) return GB_EINVAL;
    if (N > AJ_NOALLOC_MAX_RING) {
        set_error_msg("ajtai_commit_wide_noalloc_ffi: N = " + std::to_string(N) + " ring elements exceeds the " +
                      std::to_string(AJ_NOALLOC_MAX_RING) + " that its static scratch holds");
        return GB_EINVAL;
    }
    u64* partial = nullptr;
    int rc = wide_noalloc_scratch(&partial);
    if (rc) return rc;
    cudaStream_t s = stream();
    int nchunks = (int)((N + WIDE_CHUNK - 1) / WIDE_CHUNK);
    dim3 g((unsigned)nchunks, (unsigned)((AJ_KAPPA + WIDE_ROWS - 1) / WIDE_ROWS));
    ajtai_wide_kernel<<<g, WIDE_ROWS * AJ_D, 0, s>>>(d_key, d_z_wide, N, col_offset, partial, nchunks);
    GB_LAUNCH_CHECK("ajtai_wide_kernel");
    ajtai_wide_reduce_kernel<<<grid_for(AJ_KAPPA * AJ_D, 256), 256, 0, s>>>(partial, nchunks, d_out);
    GB_LAUNCH_CHECK("ajtai_wide_reduce_kernel");
    return sync_stream("ajtai_commit_wide_noalloc_ffi");
}

int ajtai_commit_dense_batched_at_ffi(const uint32_t* d_key, const uint64_t* d_z, uint64_t N, int B, int chunk,
                                      uint64_t col_offset, uint64_t* d_out) {
    if (!chunk_ok(chunk)) return GB_EUNSUPPORTED;
    return commit_bits(d_key, d_z, nullptr, N, B, col_offset, d_out, "ajtai_commit_dense_batched_ffi");
}

int ajtai_commit_dense_batched_ffi(const uint32_t* d_key, const uint64_t* d_z, uint64_t N, int B, int chunk,
                                   uint64_t* d_out) {
    return ajtai_commit_dense_batched_at_ffi(d_key, d_z, N, B, chunk, 0, d_out);
}

int ajtai_commit_ternary_ffi(const uint32_t* d_key, const uint64_t* d_pos, const uint64_t* d_neg, uint64_t N_ring,
                             int chunk, uint64_t* d_out) {
    if (!chunk_ok(chunk)) return GB_EUNSUPPORTED;
    if (!d_neg) return GB_EINVAL;
    return commit_bits(d_key, d_pos, d_neg, N_ring, AJ_SPLIT_K, 0, d_out, "ajtai_commit_ternary_ffi");
}

// M[j][i][0..63] = M_{i,j} for j < N, i < KAPPA (ajtai_premat.cuh:35-85)
__global__ void ajtai_materialize_kernel(const u32* __restrict__ key, u64 N, u64* __restrict__ M) {
    const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= (size_t)N * AJ_KAPPA * 8) return;
    u32 k[8];
#pragma unroll
    for (int q = 0; q < 8; q++) k[q] = __ldg(key + q);
    const u32 blk = (u32)(t & 7);
    const size_t ji = t >> 3;  // j * KAPPA + i
    const u64 j = ji / AJ_KAPPA;
    const int i = (int)(ji % AJ_KAPPA);
    u64 out[8];
    ajtai_prg_block(k, (u32)i, j, blk, out);
    u64* dst = M + ji * AJ_D + 8 * blk;
#pragma unroll
    for (int q = 0; q < 8; q++) dst[q] = out[q];
}

int ajtai_materialize_m_ffi(const uint32_t* d_chacha_key, uint64_t* d_M, uint64_t N) {
    if (!d_chacha_key || !d_M || N == 0) return GB_EINVAL;
    cudaStream_t s = stream();
    ajtai_materialize_kernel<<<grid_for((size_t)N * AJ_KAPPA * 8, 256), 256, 0, s>>>(d_chacha_key, N, d_M);
    return check_launch("ajtai_materialize_kernel");
}

int ajtai_commit_ternary_premat_ffi(const uint64_t* d_M, const uint64_t* d_pos, const uint64_t* d_neg, uint64_t N_ring,
                                    int chunk, uint64_t* d_out) {
    if (!chunk_ok(chunk)) return GB_EUNSUPPORTED;
    if (!d_neg || !d_M) return GB_EINVAL;
    return commit_bits(nullptr, d_pos, d_neg, N_ring, AJ_SPLIT_K, 0, d_out, "ajtai_commit_ternary_premat_ffi", d_M);
}

int ajtai_commit_sparse_ffi(const uint32_t* d_key, const uint64_t* d_positions, uint64_t K, int chunk,
                            uint64_t* d_out) {
    if (!chunk_ok(chunk)) return GB_EUNSUPPORTED;
    if (!d_key || !d_out || (K && !d_positions)) return GB_EINVAL;
    cudaStream_t s = stream();
    if (K == 0) {
        GB_CUDA_TRY(cudaMemsetAsync(d_out, 0, AJ_KAPPA * AJ_D * 8, s));
        return sync_stream("ajtai_commit_sparse_ffi");
    }
    const int nchunks = (int)((K + SPARSE_CHUNK - 1) / SPARSE_CHUNK);
    u64* partial = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&partial, (size_t)nchunks * AJ_KAPPA * AJ_D * 8, s));
    dim3 g((unsigned)nchunks, (unsigned)((AJ_KAPPA + WIDE_ROWS - 1) / WIDE_ROWS));
    ajtai_sparse_kernel<<<g, WIDE_ROWS * AJ_D, 0, s>>>(d_key, d_positions, K, partial);
    int rc = check_launch("ajtai_sparse_kernel");
    if (!rc) {
        ajtai_reduce_b_kernel<<<grid_for(AJ_KAPPA * AJ_D, 256), 256, 0, s>>>(partial, nchunks, 1, d_out);
        rc = check_launch("ajtai_reduce_b_kernel");
    }
    cudaFreeAsync(partial, s);
    return rc ? rc : sync_stream("ajtai_commit_sparse_ffi");
}

int gb_ajtai_key_create(const uint32_t* h_seed, int row_lo, int rows, uint64_t n_ring, void** handle) {
    if (!h_seed || !handle) return GB_EINVAL;
    AjtaiKey* k = new AjtaiKey();
    int rc = key_create(h_seed, row_lo, rows, n_ring, k);
    if (rc) {
        key_free(k);
        delete k;
        return rc;
    }
    *handle = k;
    return GB_OK;
}

int gb_ajtai_key_destroy(void* handle) {
    AjtaiKey* k = (AjtaiKey*)handle;
    if (!k) return GB_OK;
    key_free(k);
    delete k;
    return GB_OK;
}

int gb_ajtai_key_info(void* handle, int* row_lo, int* rows, uint64_t* n_ring) {
    AjtaiKey* k = (AjtaiKey*)handle;
    if (!k) return GB_EINVAL;
    if (row_lo) *row_lo = k->row_lo;
    if (rows) *rows = k->rows;
    if (n_ring) *n_ring = k->N;
    return GB_OK;
}

int gb_ajtai_commit_u8_batched(void* handle, const uint8_t* d_z, int num_witnesses, uint64_t* d_out) {
    AjtaiKey* k = (AjtaiKey*)handle;
    if (!k || !d_z || !d_out) return GB_EINVAL;
    return commit_batch(k, d_z, num_witnesses, d_out);
}

int gb_ajtai_set_batch_form(int form) {
    if (form < 0 || form > 4) {
        set_error_msg("gb_ajtai_set_batch_form: form must be 0 (by batch size), 1, 2, 3 or 4");
        return GB_EINVAL;
    }
    const int old = t_batch_form;
    t_batch_form = form;
    return old;
}

int gb_ajtai_test_starve(int on) {
    int old = t_starve;
    t_starve = on ? 1 : 0;
    return old;
}

}  // extern "C"
