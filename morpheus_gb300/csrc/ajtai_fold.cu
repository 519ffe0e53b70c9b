// Ajtai fold-tree operations of zk-torch-4 over R_q = F_q[X]/(X^64 + 1), q = 2^64 - 2^32 - 31
// (almost-goldilocks-cuda-rs/src/ffi.rs:435-500, :601-648; cuda/wrapper.cu:1468-1620, :1717-1740;
// cuda_almost_goldilocks/ajtai.cuh:700-1260):
//
//   fold_witness          out[j] = z1[j] + r . z2[j]                (binary z1, z2; F_q out)
//   multifold_witness     out[j] = sum_i r_i . z_i[j]               (binary z_i; i16 out)
//   multifold_mixed       out[j] = sum_b r_b . bin_b[j] + sum_t r_t . (pos_t[j] - neg_t[j])
//   split_witness         v = sum_{i<13} 2^i (pos_i - neg_i) per coefficient of an i16 witness
//   fold / multifold commitment   c = c1 + r . c2,  c = sum_i r_i . c_i   (F_q rows)
//
// where a . b is the negacyclic product: (a . b)[k] = sum_l s(k, l) a[(k - l) mod 64] b[l],
// s = -1 when l > k.  The challenges r have small integer coefficients (int8).
//
// Witness folds.  For a binary z and one coefficient plane A of r (the positions where r has
// sign s and magnitude bit p set), the contribution to coefficient k is
//     s 2^p (popc(z & S & low_k) - popc(z & S & ~low_k)),   S = rotl(brev(A), k + 1),
// low_k = bits 0..k: bit l of S is set iff (k - l) mod 64 is in A, and l > k is the wrap.
// So one instance costs a few AND/POPC per nonzero plane (three for r in {-1, 0, 1, 2})
// instead of a loop over the set bits of z.  One thread per (ring element, coefficient).
#include <algorithm>
#include <vector>

#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "agl.cuh"
#include "common.cuh"

namespace gb {

constexpr int AF_D = 64;
constexpr int AF_KAPPA = 42;
constexpr int AF_SPLIT_K = 13;
constexpr int AF_MAX_PLANES = 16;  // magnitude bits 0..7 x sign

struct AfPlane {
    u64 rmask;  // brev of the positions of this plane
    int w;      // signed weight s 2^p
};

// The nonzero planes of challenge r (64 int8 coefficients), brev'ed: at most 16.
__device__ __forceinline__ int af_planes(const int8_t* r, AfPlane* out) {
    u64 m[AF_MAX_PLANES];
#pragma unroll
    for (int q = 0; q < AF_MAX_PLANES; q++) m[q] = 0;
    for (int l = 0; l < AF_D; l++) {
        const int v = r[l];
        const int a = v < 0 ? -v : v, sg = v < 0 ? 1 : 0;
#pragma unroll
        for (int p = 0; p < 8; p++)
            if ((a >> p) & 1) m[2 * p + sg] |= 1ull << l;
    }
    int n = 0;
#pragma unroll
    for (int q = 0; q < AF_MAX_PLANES; q++)
        if (m[q]) {
            out[n].rmask = __brevll(m[q]);
            out[n].w = (q & 1 ? -1 : 1) * (1 << (q >> 1));
            n++;
        }
    return n;
}

__device__ __forceinline__ u64 rotl64(u64 x, int s) { return s ? (x << s) | (x >> (64 - s)) : x; }

// sum over the planes of z's contribution to coefficient k
__device__ __forceinline__ int af_contrib(u64 z, const AfPlane* pl, int np, int k) {
    const u64 low = k == 63 ? ~0ull : ((2ull << k) - 1);
    int acc = 0;
    for (int q = 0; q < np; q++) {
        const u64 S = rotl64(pl[q].rmask, (k + 1) & 63) & z;
        acc += pl[q].w * (__popcll(S & low) - __popcll(S & ~low));
    }
    return acc;
}

// Per-block challenge planes in shared memory: planes[i * 16 + q], counts np[i].
// Block: 256 threads = 4 ring elements x 64 coefficients; ring elements grid-stride.
// out16 (i16) or out64 (canonical F_q, with z1 added as bit k).
__global__ void __launch_bounds__(256) af_multifold_kernel(const u64* __restrict__ zb, int nb,
                                                           const u64* __restrict__ pos, const u64* __restrict__ neg,
                                                           int nt, const int8_t* __restrict__ r_all, u64 N,
                                                           const u64* __restrict__ z1, int16_t* __restrict__ out16,
                                                           u64* __restrict__ out64) {
    extern __shared__ unsigned char af_sm[];
    const int M = nb + nt;
    AfPlane* planes = reinterpret_cast<AfPlane*>(af_sm);
    int* np = reinterpret_cast<int*>(planes + (size_t)M * AF_MAX_PLANES);
    u64* zsh = reinterpret_cast<u64*>(np + ((M + 1) & ~1));  // [4][nb + 2 nt]
    for (int i = threadIdx.x; i < M; i += blockDim.x) np[i] = af_planes(r_all + (size_t)i * AF_D, planes + (size_t)i * AF_MAX_PLANES);
    __syncthreads();
    const int sub = threadIdx.x >> 6, k = threadIdx.x & 63;
    const int W = nb + 2 * nt;
    for (u64 j0 = (u64)blockIdx.x * 4; j0 < N; j0 += (u64)gridDim.x * 4) {
        for (int t = threadIdx.x; t < 4 * W; t += blockDim.x) {
            const int s = t / W, w = t % W;
            const u64 j = j0 + s;
            u64 v = 0;
            if (j < N) v = w < nb ? zb[(u64)w * N + j] : w < nb + nt ? pos[(u64)(w - nb) * N + j] : neg[(u64)(w - nb - nt) * N + j];
            zsh[t] = v;
        }
        __syncthreads();
        const u64 j = j0 + sub;
        if (j < N) {
            const u64* zz = zsh + sub * W;
            int acc = 0;
            for (int i = 0; i < nb; i++) acc += af_contrib(zz[i], planes + (size_t)i * AF_MAX_PLANES, np[i], k);
            for (int t = 0; t < nt; t++) {
                const AfPlane* pl = planes + (size_t)(nb + t) * AF_MAX_PLANES;
                acc += af_contrib(zz[nb + t], pl, np[nb + t], k) - af_contrib(zz[nb + nt + t], pl, np[nb + t], k);
            }
            if (out64) {
                acc += (int)((z1[j] >> k) & 1);
                out64[j * AF_D + k] = acc >= 0 ? (u64)acc : AGL_Q - (u64)(-acc);
            } else {
                out16[j * AF_D + k] = (int16_t)acc;
            }
        }
        __syncthreads();
    }
}

static int multifold(const u64* zb, int nb, const u64* pos, const u64* neg, int nt, const int8_t* r_all, u64 N,
                     const u64* z1, int16_t* out16, u64* out64, const char* name) {
    const int M = nb + nt;
    if (M < 1 || nb < 0 || nt < 0 || N == 0 || !r_all || (nb && !zb) || (nt && (!pos || !neg)) || !(out16 || out64))
        return GB_EINVAL;
    cudaStream_t s = stream();
    const size_t smem = (size_t)M * AF_MAX_PLANES * sizeof(AfPlane) + (size_t)((M + 1) & ~1) * sizeof(int) +
                        (size_t)4 * (nb + 2 * nt) * 8;
    if (smem > 200 * 1024) return GB_EINVAL;
    if (smem > 48 * 1024) GB_CUDA_TRY(cudaFuncSetAttribute(af_multifold_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned g = (unsigned)std::min<u64>((N + 3) / 4, (u64)num_sms() * 8);
    af_multifold_kernel<<<g, 256, smem, s>>>(zb, nb, pos, neg, nt, r_all, N, z1, out16, out64);
    return check_launch(name);
}

// c = sum_i r_i . c_i (+ c_first with weight 1): one block per row, one thread per coefficient
__global__ void af_commit_fold_kernel(const u64* __restrict__ c_first, const u64* __restrict__ c_all,
                                      const int8_t* __restrict__ r_all, int M, u64* __restrict__ out) {
    __shared__ u64 csh[AF_D];
    __shared__ int8_t rsh[AF_D];
    const int row = blockIdx.x, k = threadIdx.x;
    u64 acc = c_first ? c_first[row * AF_D + k] : 0;
    for (int i = 0; i < M; i++) {
        __syncthreads();
        csh[k] = c_all[((size_t)i * AF_KAPPA + row) * AF_D + k];
        rsh[k] = r_all[(size_t)i * AF_D + k];
        __syncthreads();
        for (int l = 0; l < AF_D; l++) {
            const int rv = rsh[l];
            if (!rv) continue;
            const int idx = k - l;
            const u64 c = csh[idx < 0 ? idx + AF_D : idx];
            const int sv = idx < 0 ? -rv : rv;
            const u64 a = sv < 0 ? (u64)(-sv) : (u64)sv;
            const u64 t = agl_mul(c, a);
            acc = sv < 0 ? agl_sub(acc, t) : agl_add(acc, t);
        }
    }
    out[row * AF_D + k] = agl_canon(acc);
}

// split of an i16 witness into 13 ternary chunks (pos, neg bitmasks), a warp per ring element:
// lane l holds coefficients l and l + 32; each chunk's masks are two ballots
__global__ void af_split_kernel(const int16_t* __restrict__ z, u64* __restrict__ pos, u64* __restrict__ neg, u64 N) {
    const int lane = threadIdx.x & 31;
    const u64 w0 = (blockIdx.x * (u64)blockDim.x + threadIdx.x) >> 5, nw = ((u64)gridDim.x * blockDim.x) >> 5;
    for (u64 j = w0; j < N; j += nw) {
        const int a = z[j * AF_D + lane], b = z[j * AF_D + 32 + lane];
        const int aa = a < 0 ? -a : a, bb = b < 0 ? -b : b;
        u64 mine = 0;
#pragma unroll
        for (int i = 0; i < AF_SPLIT_K; i++) {
            const unsigned pa = __ballot_sync(0xffffffffu, a > 0 && ((aa >> i) & 1));
            const unsigned pb = __ballot_sync(0xffffffffu, b > 0 && ((bb >> i) & 1));
            const unsigned na = __ballot_sync(0xffffffffu, a < 0 && ((aa >> i) & 1));
            const unsigned nbm = __ballot_sync(0xffffffffu, b < 0 && ((bb >> i) & 1));
            if (lane == i) mine = (u64)pa | ((u64)pb << 32);
            if (lane == AF_SPLIT_K + i) mine = (u64)na | ((u64)nbm << 32);
        }
        if (lane < AF_SPLIT_K) pos[(u64)lane * N + j] = mine;
        else if (lane < 2 * AF_SPLIT_K) neg[(u64)(lane - AF_SPLIT_K) * N + j] = mine;
    }
}

static bool af_chunk_ok(int chunk) {
    return chunk == 64 || chunk == 128 || chunk == 256 || chunk == 1024 || chunk == 4096;
}

}  // namespace gb

using namespace gb;

extern "C" {

int ajtai_fold_witness_ffi(const uint64_t* d_z1, const uint64_t* d_z2, const int8_t* r_coeffs, uint64_t N_ring,
                           int chunk, uint64_t* d_out) {
    if (!af_chunk_ok(chunk)) return GB_EUNSUPPORTED;
    if (!d_z1 || !d_z2 || !r_coeffs) return GB_EINVAL;
    cudaStream_t s = stream();
    int8_t* d_r = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&d_r, AF_D, s));
    int rc = cudaMemcpyAsync(d_r, r_coeffs, AF_D, cudaMemcpyHostToDevice, s) == cudaSuccess ? GB_OK : GB_ECUDA;
    if (!rc) rc = multifold(d_z2, 1, nullptr, nullptr, 0, d_r, N_ring, d_z1, nullptr, d_out, "ajtai_fold_witness_ffi");
    cudaFreeAsync(d_r, s);
    return rc;
}

int ajtai_multifold_witness_ffi(const uint64_t* d_z_packed, const int8_t* d_r_all, int16_t* d_out, int num_instances,
                                uint64_t N_ring, uint64_t chunk_size) {
    if (chunk_size == 0) return GB_EINVAL;
    return multifold(d_z_packed, num_instances, nullptr, nullptr, 0, d_r_all, N_ring, nullptr, d_out, nullptr,
                     "ajtai_multifold_witness_ffi");
}

int ajtai_multifold_mixed_witness_ffi(const uint64_t* d_z_bin_packed, const uint64_t* d_pos_packed,
                                      const uint64_t* d_neg_packed, const int8_t* d_r_all, int16_t* d_out,
                                      int num_binary, int num_ternary, uint64_t N_ring, uint64_t chunk_size) {
    if (chunk_size == 0) return GB_EINVAL;
    return multifold(d_z_bin_packed, num_binary, d_pos_packed, d_neg_packed, num_ternary, d_r_all, N_ring, nullptr,
                     d_out, nullptr, "ajtai_multifold_mixed_witness_ffi");
}

int ajtai_multifold_mixed_witness_tc_ffi(const uint64_t* d_z_bin_packed, const uint64_t* d_pos_packed,
                                         const uint64_t* d_neg_packed, const int8_t* d_r_all, int16_t* d_out,
                                         int num_binary, int num_ternary, uint64_t N_ring) {
    return multifold(d_z_bin_packed, num_binary, d_pos_packed, d_neg_packed, num_ternary, d_r_all, N_ring, nullptr,
                     d_out, nullptr, "ajtai_multifold_mixed_witness_tc_ffi");
}

int ajtai_multifold_mixed_witness_tc_fused_ffi(const uint64_t* d_z_bin_packed, const uint64_t* d_pos_packed,
                                               const uint64_t* d_neg_packed, const int8_t* d_r_all, int16_t* d_out,
                                               int num_binary, int num_ternary, uint64_t N_ring) {
    return multifold(d_z_bin_packed, num_binary, d_pos_packed, d_neg_packed, num_ternary, d_r_all, N_ring, nullptr,
                     d_out, nullptr, "ajtai_multifold_mixed_witness_tc_fused_ffi");
}

int ajtai_split_witness_ffi(const int16_t* d_z_wide, uint64_t* d_pos_chunks, uint64_t* d_neg_chunks, uint64_t N_ring) {
    if (!d_z_wide || !d_pos_chunks || !d_neg_chunks || N_ring == 0) return GB_EINVAL;
    cudaStream_t s = stream();
    const unsigned g = (unsigned)std::min<u64>((N_ring + 7) / 8, (u64)num_sms() * 16);
    af_split_kernel<<<g, 256, 0, s>>>(d_z_wide, d_pos_chunks, d_neg_chunks, N_ring);
    return check_launch("af_split_kernel");
}

int ajtai_multifold_commitment_ffi(const uint64_t* d_c_packed, const int8_t* d_r_all, int num_instances,
                                   uint64_t* d_out) {
    if (!d_c_packed || !d_r_all || !d_out || num_instances < 1) return GB_EINVAL;
    af_commit_fold_kernel<<<AF_KAPPA, AF_D, 0, stream()>>>(nullptr, d_c_packed, d_r_all, num_instances, d_out);
    return check_launch("af_commit_fold_kernel");
}

int ajtai_fold_commitment_ffi(const uint64_t* d_c1, const uint64_t* d_c2, const int8_t* r_coeffs, uint64_t* d_out) {
    if (!d_c1 || !d_c2 || !r_coeffs || !d_out) return GB_EINVAL;
    cudaStream_t s = stream();
    int8_t* d_r = nullptr;
    GB_CUDA_TRY(cudaMallocAsync(&d_r, AF_D, s));
    int rc = cudaMemcpyAsync(d_r, r_coeffs, AF_D, cudaMemcpyHostToDevice, s) == cudaSuccess ? GB_OK : GB_ECUDA;
    if (!rc) {
        af_commit_fold_kernel<<<AF_KAPPA, AF_D, 0, s>>>(d_c1, d_c2, d_r, 1, d_out);
        rc = check_launch("af_commit_fold_kernel");
    }
    cudaFreeAsync(d_r, s);
    return rc;
}

}  // extern "C"
