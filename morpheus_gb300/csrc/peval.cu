// Partial evaluation, bit permutation and the fused permute + partial evaluation of the einsum
// input preparation, for Goldilocks (goldilocks-cuda-rs/src/ffi.rs:377-390, :650-669;
// wrapper.cu:1164-1210, :1824-1885 over cuda/partial_eval.cuh and cuda/fused_permute_peval.cuh)
// and almost-Goldilocks (almost-goldilocks-cuda-rs/src/ffi.rs:113-119, :198-226; wrapper.cu:713-805,
// :1061-1085).
//
//   partial eval:  fix the low m variables at r, LSB first: out[j] = in[2j] + r_i (in[2j+1] - in[2j])
//                  per level.  Folding K levels is the dot product of each group of 2^K inputs with
//                  the eq table of those K challenges, so a pass fixes up to 10 variables reading the
//                  input once, at two lazy products per input (base x Ext2).
//   bit permute:   out[new] = in[old(new)], old bit inv_perm[k] <- new bit k.  One block per tile
//                  whose new-index bits cover new bits 0..4 and the new positions of old bits 0..4:
//                  the tile is read in old order (coalesced), staged in shared memory, written in
//                  new order (coalesced), whatever the permutation.
//   fused:         out[j] = sum_b evals[old(j 2^m + b)] eq[b], old() from the caller's split LUTs.
//                  The 32 lanes of a warp take the new positions of old bits 0..4, so every warp
//                  load is 256 contiguous bytes; lanes whose bits fall in the summed range b are
//                  combined by shuffles at the end, and large sums are split over warps with a
//                  second, tiny reduction launch.
#include <algorithm>
#include <vector>

#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "../../include/goldilocks_cuda_wrapper.h"
#include "agl.cuh"
#include "common.cuh"
#include "gl.cuh"

namespace gb {

// ---------------------------------------------------------------- field traits
struct FGl {
    using E = e2;
    static constexpr u64 W = 7;
    static __device__ __forceinline__ u64 add(u64 a, u64 b) { return gl_add(a, b); }
    static __device__ __forceinline__ u64 sub(u64 a, u64 b) { return gl_sub(a, b); }
    static __device__ __forceinline__ u64 mul(u64 a, u64 b) { return gl_mul(a, b); }
    static __device__ __forceinline__ u64 canon(u64 a) { return gl_canon(a); }
    static __device__ __forceinline__ E emake(u64 a, u64 b) { return e2_make(a, b); }
    static __device__ __forceinline__ E eadd(E a, E b) { return e2_add(a, b); }
    static __device__ __forceinline__ E esub(E a, E b) { return e2_sub(a, b); }
    static __device__ __forceinline__ E emul(E a, E b) { return e2_mul(a, b); }
    // lazy sum of base x Ext2 products
    struct Acc {
        gl3 a0, a1;
        __device__ __forceinline__ void zero() { a0 = a1 = gl3_zero(); }
        __device__ __forceinline__ void add(u64 v, u64 e0, u64 e1) {
            gl3_add_prod(a0, v, e0);
            gl3_add_prod(a1, v, e1);
        }
        __device__ __forceinline__ void add1(u64 v, u64 e) { gl3_add_prod(a0, v, e); }
        // (v0 + v1 X)(e0 + e1 X), X^2 = 7: e1w = 7 e1
        __device__ __forceinline__ void add2(u64 v0, u64 v1, u64 e0, u64 e1, u64 e1w) {
            gl3_add_prod(a0, v0, e0);
            gl3_add_prod(a0, v1, e1w);
            gl3_add_prod(a1, v0, e1);
            gl3_add_prod(a1, v1, e0);
        }
        __device__ __forceinline__ void get(u64& c0, u64& c1) const {
            c0 = gl_canon(gl3_reduce(a0));
            c1 = gl_canon(gl3_reduce(a1));
        }
    };
};
struct FAgl {
    using E = ae2;
    static constexpr u64 W = 3;
    static __device__ __forceinline__ u64 add(u64 a, u64 b) { return agl_add(a, b); }
    static __device__ __forceinline__ u64 sub(u64 a, u64 b) { return agl_sub(a, b); }
    static __device__ __forceinline__ u64 mul(u64 a, u64 b) { return agl_mul(a, b); }
    static __device__ __forceinline__ u64 canon(u64 a) { return agl_canon(a); }
    static __device__ __forceinline__ E emake(u64 a, u64 b) { return ae2_make(a, b); }
    static __device__ __forceinline__ E eadd(E a, E b) { return ae2_add(a, b); }
    static __device__ __forceinline__ E esub(E a, E b) { return ae2_sub(a, b); }
    static __device__ __forceinline__ E emul(E a, E b) { return ae2_mul(a, b); }
    struct Acc {
        u64 a0, a1;
        __device__ __forceinline__ void zero() { a0 = a1 = 0; }
        __device__ __forceinline__ void add(u64 v, u64 e0, u64 e1) {
            a0 = agl_add(a0, agl_mul(v, e0));
            a1 = agl_add(a1, agl_mul(v, e1));
        }
        __device__ __forceinline__ void add1(u64 v, u64 e) { a0 = agl_add(a0, agl_mul(v, e)); }
        __device__ __forceinline__ void add2(u64 v0, u64 v1, u64 e0, u64 e1, u64 e1w) {
            a0 = agl_add(a0, agl_add(agl_mul(v0, e0), agl_mul(v1, e1w)));
            a1 = agl_add(a1, agl_add(agl_mul(v0, e1), agl_mul(v1, e0)));
        }
        __device__ __forceinline__ void get(u64& c0, u64& c1) const {
            c0 = agl_canon(a0);
            c1 = agl_canon(a1);
        }
    };
};

// ---------------------------------------------------------------- partial evaluation passes
// Fixing K variables is a dot product with their eq table: out[o] = sum_{b < 2^K} in[o 2^K + b] E[b],
// E[b] = prod_l (b_l ? r_l : 1 - r_l) (variable l <-> bit l, as the LSB-first folds).  The block
// builds E in shared memory by doubling; lanes read 32 consecutive inputs (coalesced) and
// accumulate lazily; lanes of one output are combined by shuffles.
// MODE 0: base in, base r.  1: base in, Ext2 r.  2: Ext2 in, Ext2 r.  Outputs canonical.
constexpr int PE_BATCH = 8;

template <class F, int MODE, bool FULL>
__global__ void __launch_bounds__(256) pe_dot_kernel(const u64* __restrict__ in, u64* __restrict__ out,
                                                     const u64* __restrict__ r, int lvl0, int K, size_t outs) {
    // E in shared memory as separate arrays: e0[2^K], and for Ext2 r e1[2^K], e1w[2^K] = W e1
    extern __shared__ u64 se[];
    const int S = 1 << K;
    u64* e0 = se;
    u64* e1 = se + S;
    u64* e1w = se + 2 * S;
    if (threadIdx.x == 0) {
        e0[0] = 1;
        if (MODE) e1[0] = 0;
    }
    __syncthreads();
    for (int l = 0; l < K; l++) {
        const int h = 1 << l;
        for (int b = threadIdx.x; b < h; b += blockDim.x) {
            if (MODE == 0) {
                const u64 rl = __ldg(r + lvl0 + l), v = e0[b];
                e0[b + h] = F::mul(v, rl);
                e0[b] = F::mul(v, F::sub(1, rl));
            } else {
                const typename F::E rl = F::emake(__ldg(r + 2 * (lvl0 + l)), __ldg(r + 2 * (lvl0 + l) + 1));
                const typename F::E v = F::emake(e0[b], e1[b]);
                const typename F::E hi = F::emul(v, rl), lo = F::esub(v, hi);  // v (1 - r) = v - v r
                e0[b + h] = hi.c0;
                e1[b + h] = hi.c1;
                e0[b] = lo.c0;
                e1[b] = lo.c1;
            }
        }
        __syncthreads();
    }
    for (int b = threadIdx.x; b < S; b += blockDim.x) {
        e0[b] = F::canon(e0[b]);
        if (MODE) {
            e1[b] = F::canon(e1[b]);
            e1w[b] = F::canon(F::mul(F::W, e1[b]));
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const size_t warp0 = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
    const size_t nwarps = ((size_t)gridDim.x * blockDim.x) >> 5;
    // FULL (2^K >= 32): a warp task is one output, 2^K / 32 steps of 32 consecutive inputs;
    // else a task is 32 consecutive inputs covering 32 / 2^K outputs
    const int steps = FULL ? S / 32 : 1;
    const size_t tasks = FULL ? outs : (outs * S + 31) / 32;
    const size_t total = outs * (size_t)S;
    for (size_t task = warp0; task < tasks; task += nwarps) {
        const size_t base = task * 32 * (size_t)steps;
        typename F::Acc acc;
        acc.zero();
        int i = 0;
        if (FULL) {
            // PE_BATCH independent loads in flight per lane before they are multiplied in
            for (; i + PE_BATCH <= steps; i += PE_BATCH) {
                u64 v0[PE_BATCH], v1[PE_BATCH];
#pragma unroll
                for (int u = 0; u < PE_BATCH; u++) {
                    const size_t e = base + (size_t)(i + u) * 32 + lane;
                    if (MODE == 2) {
                        const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(in) + e);
                        v0[u] = v.x;
                        v1[u] = v.y;
                    } else {
                        v0[u] = __ldg(in + e);
                    }
                }
#pragma unroll
                for (int u = 0; u < PE_BATCH; u++) {
                    const int b = (i + u) * 32 + lane;
                    if (MODE == 0) acc.add1(v0[u], e0[b]);
                    else if (MODE == 1) acc.add(v0[u], e0[b], e1[b]);
                    else acc.add2(v0[u], v1[u], e0[b], e1[b], e1w[b]);
                }
            }
        }
        for (; i < steps; i++) {
            const int b = FULL ? i * 32 + lane : (lane & (S - 1));
            const size_t e = base + (size_t)i * 32 + lane;
            if (FULL || e < total) {
                if (MODE == 0) {
                    acc.add1(__ldg(in + e), e0[b]);
                } else if (MODE == 1) {
                    acc.add(__ldg(in + e), e0[b], e1[b]);
                } else {
                    const ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(in) + e);
                    acc.add2(v.x, v.y, e0[b], e1[b], e1w[b]);
                }
            }
        }
        u64 c0, c1;
        acc.get(c0, c1);
        const int red = FULL ? 5 : K;  // lane bits inside one output
        for (int k = 0; k < red; k++) {
            c0 = F::add(c0, __shfl_xor_sync(0xffffffffu, c0, 1 << k));
            if (MODE) c1 = F::add(c1, __shfl_xor_sync(0xffffffffu, c1, 1 << k));
        }
        if ((lane & ((1 << red) - 1)) == 0) {
            const size_t o = (base + lane) >> K;
            if (FULL || o < outs) {
                if (MODE == 0) out[o] = F::canon(c0);
                else {
                    out[2 * o] = F::canon(c0);
                    out[2 * o + 1] = F::canon(c1);
                }
            }
        }
    }
}

template <class F, int MODE>
static int pe_pass(const u64* in, u64* out, const u64* r, int lvl0, int K, size_t outs, cudaStream_t s) {
    const size_t smem = ((size_t)1 << K) * (MODE == 0 ? 8 : 24);
    const size_t tasks = K >= 5 ? outs : ((outs << K) + 31) / 32;
    const unsigned g = (unsigned)std::max<size_t>(1, std::min<size_t>((tasks + 7) / 8, (size_t)num_sms() * 8));
    if (K >= 5) pe_dot_kernel<F, MODE, true><<<g, 256, smem, s>>>(in, out, r, lvl0, K, outs);
    else pe_dot_kernel<F, MODE, false><<<g, 256, smem, s>>>(in, out, r, lvl0, K, outs);
    return check_launch("pe_dot_kernel");
}

constexpr int PE_MAX_K = 10;

// Fix the low m of log_n variables.  EXT: Ext2 r (base input, Ext2 output).  The m variables
// are split into passes of at most PE_MAX_K, the first the largest; passes 1..P-1 write the two scratch
// halves alternately and pass P writes dst; with one pass and dst == src the result goes
// through scratch and is copied back.
template <class F, bool EXT>
static int partial_eval(const u64* src, u64* dst, const u64* r, int log_n, int m) {
    if (!src || !dst || !r || log_n < 0 || log_n > 40 || m < 0 || m > log_n) return GB_EINVAL;
    if (m == 0) return GB_OK;
    cudaStream_t s = stream();
    const int w = EXT ? 2 : 1;  // words per output element
    // the first pass reads the whole input: give it the most variables (a longer sum per output)
    std::vector<int> ks;
    for (int left = m; left > 0; left -= std::min(left, PE_MAX_K)) ks.push_back(std::min(left, PE_MAX_K));
    const int P = (int)ks.size();
    const bool copy_back = (P == 1 && src == dst);
    size_t s0 = 0, s1 = 0;
    if (P > 1 || copy_back) {
        s0 = ((size_t)1 << (log_n - ks[0])) * w;
        s1 = P > 2 ? ((size_t)1 << (log_n - ks[0] - ks[1])) * w : 0;
    }
    u64* scratch = nullptr;
    if (s0 + s1) GB_CUDA_TRY(cudaMallocAsync(&scratch, (s0 + s1) * 8, s));
    int rc = GB_OK;
    const u64* cur = src;
    int lvl = 0, left = log_n;
    for (int i = 0; i < P && !rc; i++) {
        const int K = ks[i];
        const size_t outs = (size_t)1 << (left - K);
        u64* o = (i == P - 1 && !copy_back) ? dst : (i % 2 == 0 ? scratch : scratch + s0);
        if (!EXT) rc = pe_pass<F, 0>(cur, o, r, lvl, K, outs, s);
        else if (i == 0) rc = pe_pass<F, 1>(cur, o, r, lvl, K, outs, s);
        else rc = pe_pass<F, 2>(cur, o, r, lvl, K, outs, s);
        cur = o;
        lvl += K;
        left -= K;
    }
    if (!rc && copy_back && cudaMemcpyAsync(dst, cur, ((size_t)1 << left) * w * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        rc = GB_ECUDA;
    if (scratch) cudaFreeAsync(scratch, s);
    return rc;
}

// ---------------------------------------------------------------- bit permutation
struct PermTile {
    int n, tb;        // index bits, tile bits
    int ord_old[10];  // tile bits in load order: new positions of old bits 0..c-1, then the rest
    int ord_new[10];  // tile bits in store order: new bits 0..c-1, then the rest
    int old_of_ord_old[10];
    unsigned rest_mask;  // new bits outside the tile
    int inv[32];         // inv[new bit] = old bit
};

__device__ __forceinline__ size_t pdep64(size_t v, unsigned mask) {
    size_t r = 0;
    for (int k = 0; mask; k++) {
        const int b = __ffs(mask) - 1;
        mask &= mask - 1;
        r |= ((v >> k) & 1) << b;
    }
    return r;
}

__global__ void __launch_bounds__(256) bit_permute_tile_kernel(const u64* __restrict__ in, u64* __restrict__ out,
                                                              PermTile pt, size_t tiles) {
    __shared__ u64 sm[1024];
    const int T = 1 << pt.tb;
    for (size_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const size_t base_new = pdep64(tile, pt.rest_mask);
        size_t base_old = 0;
        for (int k = 0; k < pt.n; k++)
            if ((base_new >> k) & 1) base_old |= (size_t)1 << pt.inv[k];
        for (int u = threadIdx.x; u < T; u += blockDim.x) {
            size_t o = base_old;
            unsigned nl = 0;
            for (int i = 0; i < pt.tb; i++)
                if ((u >> i) & 1) {
                    o |= (size_t)1 << pt.old_of_ord_old[i];
                    nl |= 1u << pt.ord_old[i];
                }
            // smem slot: the store-order index of this new-local index
            int v = 0;
            for (int i = 0; i < pt.tb; i++) v |= ((nl >> pt.ord_new[i]) & 1) << i;
            sm[v] = __ldg(in + o);
        }
        __syncthreads();
        for (int v = threadIdx.x; v < T; v += blockDim.x) {
            size_t nw = base_new;
            for (int i = 0; i < pt.tb; i++)
                if ((v >> i) & 1) nw |= (size_t)1 << pt.ord_new[i];
            out[nw] = sm[v];
        }
        __syncthreads();
    }
}

// inv_perm[new bit] = old bit (the reference's d_perm_map argument), read from the device.
static int bit_permute(const u64* in, u64* out, const int* d_inv_perm, int n_bits, long long total) {
    if (!in || !out || !d_inv_perm || n_bits < 0 || n_bits > 31 || total != (1ll << n_bits)) return GB_EINVAL;
    cudaStream_t s = stream();
    int inv[32] = {0};
    GB_CUDA_TRY(cudaMemcpyAsync(inv, d_inv_perm, sizeof(int) * n_bits, cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned seen = 0;
    for (int k = 0; k < n_bits; k++) {
        if (inv[k] < 0 || inv[k] >= n_bits || ((seen >> inv[k]) & 1)) return GB_EINVAL;
        seen |= 1u << inv[k];
    }
    PermTile pt{};
    pt.n = n_bits;
    for (int k = 0; k < n_bits; k++) pt.inv[k] = inv[k];
    int pm[32];
    for (int k = 0; k < n_bits; k++) pm[inv[k]] = k;
    const int c = std::min(5, n_bits);
    unsigned tmask = 0;
    int nb = 0;
    for (int o = 0; o < c; o++) {  // load order: new positions of old bits 0..c-1 first
        pt.ord_old[nb] = pm[o];
        pt.old_of_ord_old[nb] = o;
        tmask |= 1u << pm[o];
        nb++;
    }
    for (int k = 0; k < c; k++)
        if (!((tmask >> k) & 1)) {
            pt.ord_old[nb] = k;
            pt.old_of_ord_old[nb] = inv[k];
            tmask |= 1u << k;
            nb++;
        }
    pt.tb = nb;
    int ns = 0;
    for (int k = 0; k < c; k++) pt.ord_new[ns++] = k;  // store order: new bits 0..c-1 first
    for (int i = 0; i < nb; i++)
        if (pt.ord_old[i] >= c) pt.ord_new[ns++] = pt.ord_old[i];
    pt.rest_mask = (n_bits >= 32 ? 0xFFFFFFFFu : ((1u << n_bits) - 1)) & ~tmask;
    const size_t tiles = (size_t)1 << (n_bits - nb);
    const unsigned g = (unsigned)std::min<size_t>(tiles, (size_t)num_sms() * 8);
    bit_permute_tile_kernel<<<g, 256, 0, s>>>(in, out, pt, tiles);
    return check_launch("bit_permute_tile_kernel");
}

// ---------------------------------------------------------------- fused permute + partial evaluation
struct FpeGeom {
    int c;             // lane bits (old bits 0..c-1)
    int pm[5];         // new positions of old bits 0..c-1
    unsigned lmask;    // those positions
    unsigned it_mask;  // summed-range bits not carried by lanes
    unsigned wj_mask;  // output-range bits not carried by lanes
    int cb;            // lane bits inside the summed range
};

// the new position of each old bit 0..c-1, read from the split LUTs (entry 1 << p of the LUT
// holding new bit p is the single old bit of p)
// (lanes cover the old bits 0..c-1 that the LUTs place; a malformed LUT only narrows the lanes)
__device__ __forceinline__ void fpe_geometry(const uint32_t* lo, const uint32_t* hi, int n, int m, int half,
                                             FpeGeom& g) {
    const int cmax = n < 5 ? n : 5;
    unsigned found = 0;
    for (int k = 0; k < 5; k++) g.pm[k] = 0;
    for (int p = 0; p < n; p++) {
        const uint32_t ob = p < half ? lo[1u << p] : hi[1u << (p - half)];
        const int o = __ffs(ob) - 1;
        if (o >= 0 && o < cmax && !((found >> o) & 1)) {
            g.pm[o] = p;
            found |= 1u << o;
        }
    }
    g.c = 0;
    while (g.c < cmax && ((found >> g.c) & 1)) g.c++;
    g.lmask = 0;
    for (int k = 0; k < g.c; k++) g.lmask |= 1u << g.pm[k];
    const unsigned all = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1);
    const unsigned bm = m >= 32 ? 0xFFFFFFFFu : ((1u << m) - 1);
    g.it_mask = bm & ~g.lmask;
    g.wj_mask = all & ~bm & ~g.lmask;
    g.cb = __popc(g.lmask & bm);
}

constexpr int FPE_U = 8;

template <class F>
__global__ void __launch_bounds__(256) fpe_kernel(const u64* __restrict__ evals, u64* __restrict__ out,
                                                  const u64* __restrict__ eq, const uint32_t* __restrict__ lo,
                                                  const uint32_t* __restrict__ hi, int n, int m, int half,
                                                  long long outs, int s_host) {
    __shared__ FpeGeom sg;
    if (threadIdx.x == 0) fpe_geometry(lo, hi, n, m, half, sg);
    __syncthreads();
    const FpeGeom g = sg;
    const int lane = threadIdx.x & 31;
    const bool active = lane < (1 << g.c);
    unsigned lane_new = 0;
    for (int k = 0; k < g.c; k++)
        if ((lane >> k) & 1) lane_new |= 1u << g.pm[k];
    const unsigned bm = m >= 32 ? 0xFFFFFFFFu : ((1u << m) - 1);
    const unsigned lane_b = lane_new & bm;
    const unsigned lo_mask = half >= 32 ? 0xFFFFFFFFu : ((1u << half) - 1);
    const int iter_bits = m - g.cb;
    const long long s_eff = std::min<long long>(s_host, 1ll << iter_bits);
    const int per_bits = iter_bits - (31 - __clz((int)s_eff));  // per = 2^iter_bits / s_eff
    const long long wj_count = 1ll << __popc(g.wj_mask);
    const long long tasks = wj_count * s_eff;
    const long long warp0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long task = warp0; task < tasks; task += nwarps) {
        const long long wj = task / s_eff, chunk = task % s_eff;
        const unsigned warp_new = (unsigned)pdep64((size_t)wj, g.wj_mask);
        const unsigned base_old = (lo[warp_new & lo_mask] | hi[warp_new >> half]) | (unsigned)lane;
        unsigned x = (unsigned)pdep64((size_t)chunk << per_bits, g.it_mask);
        typename F::Acc acc;
        acc.zero();
        if (active) {
            const long long iters = 1ll << per_bits;
            const size_t nmax = (size_t)1 << n;
            long long it = 0;
            // FPE_U independent gathers in flight per lane (the LUT loads are warp-uniform)
            for (; it + FPE_U <= iters; it += FPE_U) {
                unsigned xs[FPE_U];
                u64 v[FPE_U];
                ulonglong2 e[FPE_U];
#pragma unroll
                for (int k = 0; k < FPE_U; k++) {
                    xs[k] = x;
                    x = ((x | ~g.it_mask) + 1) & g.it_mask;
                }
#pragma unroll
                for (int k = 0; k < FPE_U; k++) {
                    const size_t idx = base_old | lo[xs[k] & lo_mask] | hi[xs[k] >> half];
                    v[k] = idx < nmax ? __ldg(evals + idx) : 0;  // malformed LUT entries read nothing
                    e[k] = __ldg(reinterpret_cast<const ulonglong2*>(eq) + (lane_b | xs[k]));
                }
#pragma unroll
                for (int k = 0; k < FPE_U; k++) acc.add(v[k], e[k].x, e[k].y);
            }
            for (; it < iters; it++) {
                const size_t idx = base_old | lo[x & lo_mask] | hi[x >> half];
                const u64 v = idx < nmax ? __ldg(evals + idx) : 0;
                const ulonglong2 e = __ldg(reinterpret_cast<const ulonglong2*>(eq) + (lane_b | x));
                acc.add(v, e.x, e.y);
                x = ((x | ~g.it_mask) + 1) & g.it_mask;
            }
        }
        u64 c0, c1;
        acc.get(c0, c1);
        if (!active) c0 = c1 = 0;
        for (int k = 0; k < g.c; k++)
            if (g.pm[k] < m) {
                c0 = F::add(c0, __shfl_xor_sync(0xffffffffu, c0, 1 << k));
                c1 = F::add(c1, __shfl_xor_sync(0xffffffffu, c1, 1 << k));
            }
        if (active && lane_b == 0) {
            const long long j = (long long)((lane_new | warp_new) >> m);
            if (j < outs) {
                u64* o = out + 2 * ((s_host > 1 ? chunk * outs : 0) + j);
                o[0] = F::canon(c0);
                o[1] = F::canon(c1);
            }
        }
    }
}

// out[j] = sum over the s_eff chunk partials
template <class F>
__global__ void fpe_reduce_kernel(const u64* __restrict__ part, u64* __restrict__ out, const uint32_t* __restrict__ lo,
                                  const uint32_t* __restrict__ hi, int n, int m, int half, long long outs, int s_host) {
    __shared__ FpeGeom sg;
    if (threadIdx.x == 0) fpe_geometry(lo, hi, n, m, half, sg);
    __syncthreads();
    const long long s_eff = std::min<long long>(s_host, 1ll << (m - sg.cb));
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < outs; j += (long long)gridDim.x * blockDim.x) {
        u64 c0 = 0, c1 = 0;
        for (long long c = 0; c < s_eff; c++) {
            c0 = F::add(c0, part[2 * (c * outs + j)]);
            c1 = F::add(c1, part[2 * (c * outs + j) + 1]);
        }
        out[2 * j] = F::canon(c0);
        out[2 * j + 1] = F::canon(c1);
    }
}

template <class F>
static int fused_permute_peval(const u64* evals, u64* out, const u64* eq, const uint32_t* lo, const uint32_t* hi, int n,
                               int m, int half, int output_size) {
    if (!evals || !out || !eq || !lo || !hi || n < 0 || n > 31 || m < 0 || m > n || half < 0 || half > n ||
        output_size <= 0 || (long long)output_size > (1ll << (n - m)))
        return GB_EINVAL;
    cudaStream_t s = stream();
    const unsigned grid = (unsigned)num_sms() * 4;
    const long long warps = (long long)grid * 8;
    // the output range has at least 2^(n-m-5) warp tasks; split the sum until there are about
    // four tasks per warp of the grid (a short tail), keeping chunks of at least 64 terms
    const long long min_tasks = std::max(1ll, 1ll << std::max(0, n - m - 5));
    long long sh = 1;
    while (sh * min_tasks < 4 * warps && sh * 64 < (1ll << m)) sh <<= 1;
    u64* part = nullptr;
    if (sh > 1) GB_CUDA_TRY(cudaMallocAsync(&part, (size_t)sh * output_size * 16, s));
    fpe_kernel<F><<<grid, 256, 0, s>>>(evals, sh > 1 ? part : out, eq, lo, hi, n, m, half, output_size, (int)sh);
    int rc = check_launch("fpe_kernel");
    if (!rc && sh > 1) {
        fpe_reduce_kernel<F><<<grid_for((size_t)output_size, 256), 256, 0, s>>>(part, out, lo, hi, n, m, half,
                                                                               output_size, (int)sh);
        rc = check_launch("fpe_reduce_kernel");
    }
    if (part) cudaFreeAsync(part, s);
    return rc;
}

}  // namespace gb

using namespace gb;

extern "C" {

int partial_eval_gl_ffi(uint64_t* d_data, const uint64_t* d_r, int log_n, int m) {
    if (m <= 0) return GB_OK;
    return partial_eval<FGl, false>(d_data, d_data, d_r, log_n, m);
}

int partial_eval_ext2_from_gl_ffi(const uint64_t* d_input, uint64_t* d_output, const uint64_t* d_r, int log_n, int m) {
    if (m <= 0) return GB_OK;
    return partial_eval<FGl, true>(d_input, d_output, d_r, log_n, m);
}

int bit_permute_gl_ffi(const uint64_t* d_input, uint64_t* d_output, const int* d_perm_map, int n_bits, int total) {
    return bit_permute(d_input, d_output, d_perm_map, n_bits, total);
}

int fused_permute_partial_eval_ffi(const uint64_t* d_evals, uint64_t* d_output, const uint64_t* d_eq_table,
                                   const uint32_t* d_lo_lut, const uint32_t* d_hi_lut, int n, int m, int half,
                                   int output_size, int smem_bytes) {
    (void)smem_bytes;  // the LUTs are read through the cache (warp-uniform loads), not staged
    return fused_permute_peval<FGl>(d_evals, d_output, d_eq_table, d_lo_lut, d_hi_lut, n, m, half, output_size);
}

int agl_partial_eval_ffi(uint64_t* d_data, const uint64_t* d_r, int log_n, int m) {
    if (m <= 0) return GB_OK;
    return partial_eval<FAgl, false>(d_data, d_data, d_r, log_n, m);
}

int agl_partial_eval_ext2_from_base_ffi(const uint64_t* d_input, uint64_t* d_output, const uint64_t* d_r, int log_n,
                                        int m) {
    if (m <= 0) return GB_OK;
    return partial_eval<FAgl, true>(d_input, d_output, d_r, log_n, m);
}

int agl_bit_permute_ffi(const uint64_t* d_input, uint64_t* d_output, const int* d_perm_map, int n_bits, int total) {
    return bit_permute(d_input, d_output, d_perm_map, n_bits, total);
}

int agl_fused_permute_partial_eval_ffi(const uint64_t* d_evals, uint64_t* d_output, const uint64_t* d_eq_table,
                                       const uint32_t* d_lo_lut, const uint32_t* d_hi_lut, int n, int m, int half,
                                       int output_size, int smem_bytes) {
    (void)smem_bytes;
    return fused_permute_peval<FAgl>(d_evals, d_output, d_eq_table, d_lo_lut, d_hi_lut, n, m, half, output_size);
}

}  // extern "C"
