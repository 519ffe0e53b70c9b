// Round-synchronous batch prover: many instances (gb_instance, the protocol of batch.cu) with
// their Basefold openings run in lockstep, so that every step of a round is ONE launch over
// all polynomials (ragged segment tables) instead of one launch per polynomial:
//   1. commits in lockstep (transform passes, codewords, leaf hashes, layers), then the product
//      sumchecks in lockstep: for round k, one launch per degree over every instance still in
//      its protocol, one reduce launch for all the messages and one host round trip in which
//      every instance's transcript advances; every commitment stays resident;
//   2. openings: for round r = 0, 1, ... on the calling thread's stream, one launch each for
//      the eq/bh fold + oracle partials, their per-polynomial reduction, the codeword fold +
//      leaf hash, every Merkle layer, the roots and the final folds of all polynomials still
//      in round r; then one copy of all round records to the host, where each polynomial's
//      own transcript advances exactly as in open_ext2 (basefold.rs:578-870);
//   3. queries: one gather launch for all polynomials.
// Work that does not fit the HBM budget runs in several waves (largest instances first).
// Every proof is bit-identical to gb_prove_instance's.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/goldilocks_cuda_wrapper.h"
#include "basefold.cuh"
#include "bf_device.cuh"
#include "host_field.hpp"
#include "merkle.cuh"
#include "open_engine.cuh"
#include "reduce.cuh"
#include "sc_device.cuh"

namespace gb {

constexpr int LS_RED_THREADS = RED_THREADS;  // 256
constexpr int LS_ITEMS = 4;                  // items per thread in the reduction kernels
constexpr int LS_THREADS = 128;              // per-item kernels
constexpr int LS_REC = 16;                   // record words per polynomial: oracle 0..5, root 8..11, final 12..15

#define LS_RC(x)           \
    do {                   \
        int _r = (x);      \
        if (_r) return _r; \
    } while (0)

// One polynomial's part of one launch.
struct LsSeg {
    const u64* a;
    const u64* b;
    u64* c;
    u64* d;
    u64 c0, c1;
    u64 items;
    u64 block0;
};

__device__ __forceinline__ int ls_find(const LsSeg* __restrict__ segs, int nseg, u64 block) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (segs[mid].block0 <= block) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

#define LS_SEG_PROLOGUE                                       \
    __shared__ int s_seg;                                     \
    if (threadIdx.x == 0) s_seg = ls_find(segs, nseg, blockIdx.x); \
    __syncthreads();                                          \
    const LsSeg sg = segs[s_seg];

// CTA size of a segmented Poseidon2 launch, and each segment's first block for it: the wide
// shape (P2_BOUNDS) when the launch is large and its segments average at least one wide CTA.
static int ls_p2_assign(LsSeg* hs, int cnt, u64& nb) {
    u64 total = 0;
    for (int k = 0; k < cnt; k++) total += hs[k].items;
    const int T = (p2_wide(total) && total >= (u64)cnt * P2_WIDE) ? P2_WIDE : P2_NARROW;
    nb = 0;
    for (int k = 0; k < cnt; k++) {
        hs[k].block0 = nb;
        nb += hs[k].items ? (hs[k].items + T - 1) / T : 1;
    }
    return T;
}

// round 0 oracle partials: a = bh (base), b = eq (Ext2), items = pairs
__global__ void __launch_bounds__(LS_RED_THREADS) ls_round0_kernel(const LsSeg* __restrict__ segs, int nseg,
                                                                   u64* __restrict__ partials) {
    LS_SEG_PROLOGUE
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    const u64 base = (blockIdx.x - sg.block0) * (u64)blockDim.x * LS_ITEMS;
#pragma unroll
    for (int k = 0; k < LS_ITEMS; k++) {
        u64 i = base + (u64)k * blockDim.x + threadIdx.x;
        if (i < sg.items) open_round0_item(sg.a, sg.b, i, acc);
    }
    block_reduce<6>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int w = 0; w < 6; w++) partials[(size_t)blockIdx.x * 6 + w] = acc[w];
}

// round r >= 1 oracle partials with the eq/bh folds: a = eq_in, b = bh_in, c = eq_out, d = bh_out
template <bool BH_BASE>
__global__ void __launch_bounds__(LS_RED_THREADS) ls_open_round_kernel(const LsSeg* __restrict__ segs, int nseg,
                                                                       u64* __restrict__ partials) {
    LS_SEG_PROLOGUE
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    const e2 ch = e2_make(sg.c0, sg.c1);
    const u64 base = (blockIdx.x - sg.block0) * (u64)blockDim.x * LS_ITEMS;
#pragma unroll
    for (int k = 0; k < LS_ITEMS; k++) {
        u64 y = base + (u64)k * blockDim.x + threadIdx.x;
        if (y < sg.items) open_round_item<BH_BASE>(sg.a, sg.b, sg.c, sg.d, y, ch, acc);
    }
    block_reduce<6>(acc);
    if (threadIdx.x == 0)
#pragma unroll
        for (int w = 0; w < 6; w++) partials[(size_t)blockIdx.x * 6 + w] = acc[w];
}

// per polynomial: sum its blocks' partials into recs[seg][0..5] (canonical); one warp each
__global__ void ls_reduce_kernel(const LsSeg* __restrict__ segs, int nseg, const u64* __restrict__ partials,
                                 u64* __restrict__ recs) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nseg) return;
    const u64 per_block = (u64)LS_RED_THREADS * LS_ITEMS;
    const u64 nb = (segs[w].items + per_block - 1) / per_block;
    u64 acc[6] = {0, 0, 0, 0, 0, 0};
    for (u64 b = lane; b < nb; b += 32)
#pragma unroll
        for (int k = 0; k < 6; k++) acc[k] = gl_add(acc[k], partials[(segs[w].block0 + b) * 6 + k]);
#pragma unroll
    for (int k = 0; k < 6; k++) {
        u64 v = gl_warp_sum(acc[k]);
        if (lane == 0) recs[(size_t)w * LS_REC + k] = gl_canon(v);
    }
}

// codeword fold + leaf hash: a = codeword in, b = table level, c = folded out, d = tree leaves
template <bool BASE_IN, int T>
__global__ void P2_SEG_BOUNDS(T) ls_fold_hash_kernel(const LsSeg* __restrict__ segs, int nseg) {
    LS_SEG_PROLOGUE
    const u64 i = (blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x;
    if (i >= sg.items) return;
    e2 f0, f1;
    fold_leaf_item<BASE_IN>(sg.a, sg.b, i, sg.c0, sg.c1, f0, f1);
    e2_st(sg.c + 4 * i, f0);
    e2_st(sg.c + 4 * i + 2, f1);
    u64 s[8] = {f0.c0, f0.c1, f1.c0, f1.c1, 0, 0, 0, 0};
    p2_permute<4>(s);
    st_digest(sg.d + 4 * i, s);
}

// one Merkle layer: a = children, c = parents
template <int T>
__global__ void P2_SEG_BOUNDS(T) ls_merkle_level_kernel(const LsSeg* __restrict__ segs, int nseg) {
    LS_SEG_PROLOGUE
    const u64 j = (blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x;
    if (j >= sg.items) return;
    u64 s[8];
    ld_digest(sg.a + 8 * j, s);
    ld_digest(sg.a + 8 * j + 4, s + 4);
    p2_permute(s);
    st_digest(sg.c + 4 * j, s);
}

// one Merkle layer in the pair form (mid-size layers): lanes 2j, 2j + 1 of a segment's blocks make
// parent j, each holding half the state; a = children, c = parents.  Pairs past a segment's end
// compute parent 0 and store nothing (their warp takes part in the exchanges).
template <int T>
__global__ void P2_PAIR_BOUNDS(T) ls_merkle_level_pair_kernel(const LsSeg* __restrict__ segs, int nseg) {
    LS_SEG_PROLOGUE
    const u64 j = ((blockIdx.x - sg.block0) * (u64)T + threadIdx.x) >> 1;
    const int h = threadIdx.x & 1;
    const bool live = j < sg.items;
    u64 st[4];
    ld_digest(sg.a + 8 * (live ? j : 0) + 4 * h, st);
    p2_permute_pair(st, h);
    if (live && h == 0) st_digest(sg.c + 4 * j, st);
}

// one Merkle layer in the 8-lane form (latency-bound layers): group g of a segment's blocks makes
// parent g; a = children, c = parents.  Groups past a segment's end compute parent 0 and store
// nothing (their warp takes part in the shuffles).
constexpr int LS_COOP_THREADS = 128;
__global__ void __launch_bounds__(LS_COOP_THREADS) ls_merkle_level_coop_kernel(const LsSeg* __restrict__ segs,
                                                                               int nseg) {
    LS_SEG_PROLOGUE
    const u64 g = ((blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x) >> 3;
    const int l = threadIdx.x & 7;
    const bool live = g < sg.items;
    const P2Lane c = p2_lane_consts(l);
    const u64 x = p2_permute_coop(sg.a[8 * (live ? g : 0) + l], l, c);
    if (live && l < 4) sg.c[4 * g + l] = x;
}

// The form of one segmented Merkle layer, by its total parents, as the per-call trees choose
// (p2_form): the 8-lane form below `coop` (the layer cannot fill the GPU, and one thread's
// permutation is a long serial chain), the pair form below P2_ONE_FROM (two lanes per parent,
// 128- or 256-thread CTAs), else one permutation per thread in ls_p2_assign's CTA size.  The form
// is named, not read off the CTA size: several forms use 128 threads.
enum class LsLayerForm { Coop, Pair128, Pair256, Wide, Narrow };
static LsLayerForm ls_layer_assign(LsSeg* hs, int cnt, size_t coop, u64& nb) {
    u64 total = 0;
    for (int k = 0; k < cnt; k++) total += hs[k].items;
    auto blocks = [&](u64 threads_per_item, int T) {
        nb = 0;
        for (int k = 0; k < cnt; k++) {
            hs[k].block0 = nb;
            nb += (hs[k].items * threads_per_item + T - 1) / T;  // no block for an empty segment
        }
    };
    if (total < coop) {
        blocks(8, LS_COOP_THREADS);
        return LsLayerForm::Coop;
    }
    if (total < P2_ONE_FROM) {
        const int T = p2_pair_threads(total);
        blocks(2, T);
        return T == 256 ? LsLayerForm::Pair256 : LsLayerForm::Pair128;
    }
    return ls_p2_assign(hs, cnt, nb) == P2_WIDE ? LsLayerForm::Wide : LsLayerForm::Narrow;
}
static int ls_layer_launch(LsLayerForm form, u64 nb, const LsSeg* ds, int cnt, cudaStream_t s) {
    switch (form) {
        case LsLayerForm::Coop:
            ls_merkle_level_coop_kernel<<<(unsigned)nb, LS_COOP_THREADS, 0, s>>>(ds, cnt);
            break;
        case LsLayerForm::Pair128:
            ls_merkle_level_pair_kernel<128><<<(unsigned)nb, 128, 0, s>>>(ds, cnt);
            break;
        case LsLayerForm::Pair256:
            ls_merkle_level_pair_kernel<256><<<(unsigned)nb, 256, 0, s>>>(ds, cnt);
            break;
        case LsLayerForm::Wide:
            ls_merkle_level_kernel<P2_WIDE><<<(unsigned)nb, P2_WIDE, 0, s>>>(ds, cnt);
            break;
        case LsLayerForm::Narrow:
            ls_merkle_level_kernel<P2_NARROW><<<(unsigned)nb, P2_NARROW, 0, s>>>(ds, cnt);
            break;
    }
    return check_launch("ls_merkle_level_kernel");
}

// recs[seg][8..11] = root digest at a (canonical); one thread per polynomial
__global__ void ls_root_kernel(const LsSeg* __restrict__ segs, int nseg, u64* __restrict__ recs) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
#pragma unroll
    for (int k = 0; k < 4; k++) recs[(size_t)s * LS_REC + 8 + k] = gl_canon(segs[s].a[k]);
}

// last round's fold (Ext2 codeword, no tree): a = codeword in, b = table level, c = out,
// items = pairs (<= 2 for rate 1/2); also copied into recs[seg][12..]
__global__ void ls_fold_final_kernel(const LsSeg* __restrict__ segs, int nseg, u64* __restrict__ recs) {
    int s = blockIdx.x;
    if (s >= nseg) return;
    const LsSeg sg = segs[s];
    for (u64 i = threadIdx.x; i < sg.items; i += blockDim.x) {
        u64 o[2];
        fold_pair<2>(sg.a, i, sg.b[2 * i], sg.b[2 * i + 1], sg.c0, sg.c1, o);
        sg.c[2 * i] = gl_canon(o[0]);
        sg.c[2 * i + 1] = gl_canon(o[1]);
        if (2 * i + 1 < 4) {
            recs[(size_t)s * LS_REC + 12 + 2 * i] = gl_canon(o[0]);
            recs[(size_t)s * LS_REC + 13 + 2 * i] = gl_canon(o[1]);
        }
    }
}

// ---- commits (commit_device, basefold.cu) for all polynomials ----
// transform pass over bits [c0, c0 + K): a = in, c = out (may equal a), items = groups
template <int K>
__global__ void __launch_bounds__(LS_THREADS) ls_transform_pass_kernel(const LsSeg* __restrict__ segs, int nseg) {
    LS_SEG_PROLOGUE
    const u64 g = (blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x;
    if (g >= sg.items) return;
    bf_transform_group<0, K>(sg.a, sg.c, (int)sg.c0, g);
}

// codeword[j] = u[bitrev_n(j mod 2^n)]: a = u, c = codeword, items = L, c0 = n
__global__ void __launch_bounds__(LS_THREADS) ls_bitrev_replicate_kernel(const LsSeg* __restrict__ segs, int nseg) {
    LS_SEG_PROLOGUE
    const u64 j = (blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x;
    if (j >= sg.items) return;
    const int n = (int)sg.c0;
    sg.c[j] = __ldg(sg.a + bitrev_dev(j & (((u64)1 << n) - 1), n));
}

// leaf i = P2(cw[2i], cw[2i+1], 0, ...) for the first copy's leaves: a = codeword, d = tree
template <int T>
__global__ void P2_SEG_BOUNDS(T) ls_hash_leaves_kernel(const LsSeg* __restrict__ segs, int nseg) {
    LS_SEG_PROLOGUE
    const u64 i = (blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x;
    if (i >= sg.items) return;
    ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(sg.a) + i);
    u64 st[8] = {v.x, v.y, 0, 0, 0, 0, 0, 0};
    p2_permute<2>(st);
    st_digest(sg.d + 4 * i, st);
}

// copies of the first copy's subtree on every layer (replicate_layers_kernel, merkle.cu):
// c = tree, items = copied words, c0 = leaves of the full tree, c1 = leaves of one copy (2 copies)
__global__ void __launch_bounds__(LS_THREADS) ls_replicate_kernel(const LsSeg* __restrict__ segs, int nseg) {
    LS_SEG_PROLOGUE
    u64 t = (blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x;
    if (t >= sg.items) return;
    u64 off = 0, nodes = sg.c0, n = sg.c1;
    for (;;) {
        const u64 words = 4 * n;  // (copies - 1) = 1
        if (t < words) {
            u64* layer = sg.c + off;
            layer[4 * n + t] = layer[t % (4 * n)];
            return;
        }
        t -= words;
        off += 4 * nodes;
        nodes >>= 1;
        n >>= 1;
        if (n == 0) return;
    }
}

// all polynomials' queries: block (query k, polynomial p)
__global__ void ls_query_kernel(const QueryJob* __restrict__ jobs, const u64* __restrict__ idx, int q,
                                u64* const* __restrict__ outs, const u64* __restrict__ per_query) {
    const int k = blockIdx.x, p = blockIdx.y;
    query_gather_block(jobs[p], idx[(size_t)p * q + k], outs[p] + (size_t)k * per_query[p]);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static size_t align2(size_t w) { return (w + 1) & ~(size_t)1; }  // 16-byte multiples of words

// Host threads for the per-polynomial steps between rounds (each polynomial's transcript is its
// own, so they run in parallel).  The threads are started once and wait between jobs: a round
// trip of the engine should not pay for thread creation.  One job at a time (jobs are issued
// by the calling thread of a batch, and concurrent batches take turns).
class LsPool {
  public:
    static LsPool& get() {
        static LsPool pool;
        return pool;
    }
    // fn(i) for i in [0, count), split into ranges among the pool and the calling thread
    void run(size_t count, const std::function<void(size_t)>& fn) {
        const size_t nt = std::min<size_t>(workers_.size() + 1, (count + 63) / 64);
        if (nt <= 1) {
            for (size_t i = 0; i < count; i++) fn(i);
            return;
        }
        std::lock_guard<std::mutex> job_lock(job_);
        {
            std::lock_guard<std::mutex> l(m_);
            fn_ = &fn;
            count_ = count;
            parts_ = nt;
            next_part_ = 1;  // part 0 is the calling thread's
            done_ = 0;
            gen_++;
        }
        cv_.notify_all();
        part(0);
        std::unique_lock<std::mutex> l(m_);
        done_cv_.wait(l, [&] { return done_ == parts_ - 1; });
        fn_ = nullptr;
    }
    ~LsPool() {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
            gen_++;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }

  private:
    LsPool() {
        const size_t hw = std::max(1u, std::thread::hardware_concurrency());
        const size_t n = std::min<size_t>(hw, 16) - 1;
        for (size_t t = 0; t < n; t++) workers_.emplace_back([this] { loop(); });
    }
    void part(size_t k) {
        for (size_t i = k * count_ / parts_; i < (k + 1) * count_ / parts_; i++) (*fn_)(i);
    }
    void loop() {
        unsigned long long seen = 0;
        for (;;) {
            size_t k;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [&] { return stop_ || (gen_ != seen && next_part_ < parts_); });
                if (stop_) return;
                k = next_part_++;
                if (next_part_ >= parts_) seen = gen_;
            }
            part(k);
            {
                std::lock_guard<std::mutex> l(m_);
                done_++;
            }
            done_cv_.notify_one();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex job_, m_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(size_t)>* fn_ = nullptr;
    size_t count_ = 0, parts_ = 0, next_part_ = 0, done_ = 0;
    unsigned long long gen_ = 0;
    bool stop_ = false;
};

template <typename F>
static void ls_parallel(size_t count, F fn) {
    const std::function<void(size_t)> f = fn;
    LsPool::get().run(count, f);
}

struct LsPoly {
    int n = 0;
    size_t N = 0, L = 0;
    const BfCommitment* com = nullptr;
    const u64* point = nullptr;  // host, 2n canonical words (the instance's sumcheck challenges)
    gb_transcript t;
    u64* proof = nullptr;  // host, gb_basefold_proof_len(n, 1, q) words
    u64 *d_point = nullptr, *eq = nullptr, *bufs_eq[2] = {nullptr, nullptr}, *bufs_bh[2] = {nullptr, nullptr};
    std::vector<u64*> fcw, ftree;
    const u64* eq_cur = nullptr;
    const u64* bh_cur = nullptr;
    int pp = 0;
    size_t sc = 0;
};

// device words one polynomial's opening needs
static size_t ls_poly_words(int n, int lr) {
    size_t N = (size_t)1 << n, L = N << lr, w = 0;
    w += align2(2 * (size_t)n) + 2 * N + 4 * N;  // point, eq, eqA, eqB, bhA, bhB (N/2 Ext2 each)
    for (int r = 0; r < n; r++) w += align2(2 * (L >> (r + 1)));
    for (int r = 0; r + 1 < n; r++) w += 4 * (2 * ((L >> (r + 1)) / 2) - 1) + 2;
    return w;
}

// eq(r, x) tables of every polynomial of a runner at once (the values of eq_table, eq.cu):
// block 2k + h builds polynomial k's table over its low (h = 0) or high (h = 1) half of the
// variables by the doubling loop; then one launch multiplies them out, block -> polynomial by
// binary search over block0.
struct EqSeg {
    const u64* r;  // 2n words (Ext2 point)
    u64* lo;       // 2^k Ext2 scratch
    u64* hi;       // 2^(n-k) Ext2 scratch
    u64* out;      // 2^n Ext2
    u64 n, k, block0;
};

__global__ void __launch_bounds__(256) ls_eq_halves_kernel(const EqSeg* __restrict__ segs, int nseg) {
    const int k = blockIdx.x >> 1, h = blockIdx.x & 1;
    if (k >= nseg) return;
    const EqSeg sg = segs[k];
    u64* out = h ? sg.hi : sg.lo;
    const int v0 = h ? (int)sg.k : 0, v1 = h ? (int)sg.n : (int)sg.k;
    if (threadIdx.x == 0) {
        out[0] = 1;
        out[1] = 0;
    }
    __syncthreads();
    for (int v = v0; v < v1; v++) {
        const size_t half = (size_t)1 << (v - v0);
        const e2 rv = e2_make(sg.r[2 * v], sg.r[2 * v + 1]);
        for (size_t j = threadIdx.x; j < half; j += blockDim.x) {
            const e2 a = e2_make(out[2 * j], out[2 * j + 1]);
            const e2 ar = e2_mul(a, rv);
            const e2 lo_v = e2_sub(a, ar);
            out[2 * (j + half)] = ar.c0;
            out[2 * (j + half) + 1] = ar.c1;
            out[2 * j] = lo_v.c0;
            out[2 * j + 1] = lo_v.c1;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) ls_eq_expand_kernel(const EqSeg* __restrict__ segs, int nseg) {
    __shared__ int s_seg;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (segs[mid].block0 <= blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        s_seg = lo;
    }
    __syncthreads();
    const EqSeg sg = segs[s_seg];
    const u64 x = (blockIdx.x - sg.block0) * (u64)blockDim.x + threadIdx.x;
    if (x >= ((u64)1 << sg.n)) return;
    const u64 xl = x & (((u64)1 << sg.k) - 1), xh = x >> sg.k;
    e2_st(sg.out + 2 * x, e2_mul(e2_ld(sg.lo + 2 * xl), e2_ld(sg.hi + 2 * xh)));
}

class LsRunner {
  public:
    LsRunner(const BfTable* tab, int q, size_t coop) : tab_(tab), q_(q), coop_(coop) {}

    // openings of `polys` (transcripts already hold their "bf-open" preamble prefix)
    int open(std::vector<LsPoly>& P) {
        using namespace host;
        cudaStream_t s = stream();
        const int np = (int)P.size();
        const int lr = 1;
        size_t words = 0;
        for (auto& p : P) words += ls_poly_words(p.n, lr);
        int maxn = 0;
        for (auto& p : P) maxn = std::max(maxn, p.n);
        // workspace carving
        GB_CUDA_TRY(cudaMallocAsync(&ws_, std::max<size_t>(words, 2) * 8, s));
        {
            u64* cur = ws_;
            for (auto& p : P) {
                p.d_point = cur;
                cur += align2(2 * (size_t)p.n);
                p.eq = cur;
                cur += 2 * p.N;
                p.bufs_eq[0] = cur;
                cur += p.N;
                p.bufs_eq[1] = cur;
                cur += p.N;
                p.bufs_bh[0] = cur;
                cur += p.N;
                p.bufs_bh[1] = cur;
                cur += p.N;
                p.fcw.assign(p.n, nullptr);
                p.ftree.assign(p.n > 1 ? p.n - 1 : 0, nullptr);
                for (int r = 0; r < p.n; r++) {
                    p.fcw[r] = cur;
                    cur += align2(2 * (p.L >> (r + 1)));
                }
                for (int r = 0; r + 1 < p.n; r++) {
                    p.ftree[r] = cur;
                    cur += 4 * (2 * ((p.L >> (r + 1)) / 2) - 1) + 2;
                }
            }
        }
        // per-launch tables and records
        np_max_ = (size_t)np;
        seg_cap_ = (size_t)np * (maxn + 8);  // one round's launches (layers + 4) never need more slots
        GB_CUDA_TRY(cudaMallocAsync(&d_segs_, seg_cap_ * sizeof(LsSeg), s));
        GB_CUDA_TRY(cudaMallocHost(&h_segs_, seg_cap_ * sizeof(LsSeg)));
        GB_CUDA_TRY(cudaMallocHost(&h_recs_, (size_t)np * LS_REC * 8));
        {
            // the kernels write the records straight into the pinned array (its device address)
            void* d = nullptr;
            GB_CUDA_TRY(cudaHostGetDevicePointer(&d, h_recs_, 0));
            d_recs_ = (u64*)d;
        }
        size_t max_blocks = 0;
        for (auto& p : P) max_blocks += (p.N / 2 + LS_RED_THREADS * LS_ITEMS - 1) / (LS_RED_THREADS * LS_ITEMS) + 1;
        GB_CUDA_TRY(cudaMallocAsync(&d_partials_, max_blocks * 6 * 8, s));

        // preamble: root and point into each transcript; eq tables
        {
            std::vector<u64> pts;
            ls_parallel(P.size(), [&](size_t k) {
                LsPoly& p = P[k];
                for (int w = 0; w < 4; w++) tr_append_u64(&p.t, "", p.com->root[w]);
                for (int i = 0; i < p.n; i++) tr_append_ext2(&p.t, "", E2{canon(p.point[2 * i]), canon(p.point[2 * i + 1])});
            });
            // every point in one copy into one buffer, then every eq table in two launches
            std::vector<size_t> poff(np);
            size_t pwords = 0, scratch = 0;
            for (int k = 0; k < np; k++) {
                poff[k] = pwords;
                pwords += align2(2 * (size_t)P[k].n);
                scratch += 2 * (((size_t)1 << (P[k].n / 2)) + ((size_t)1 << (P[k].n - P[k].n / 2)));
            }
            pts.assign(pwords, 0);
            for (int k = 0; k < np; k++)
                for (int i = 0; i < 2 * P[k].n; i++) pts[poff[k] + i] = canon(P[k].point[i]);
            u64* d_pts = nullptr;
            GB_CUDA_TRY(cudaMallocAsync(&d_pts, pwords * 8, s));
            GB_CUDA_TRY(cudaMemcpyAsync(d_pts, pts.data(), pwords * 8, cudaMemcpyHostToDevice, s));
            u64* eqs = nullptr;
            EqSeg* d_eqsegs = nullptr;
            std::vector<EqSeg> eqsegs(np);
            GB_CUDA_TRY(cudaMallocAsync(&eqs, scratch * 8, s));
            GB_CUDA_TRY(cudaMallocAsync(&d_eqsegs, (size_t)np * sizeof(EqSeg), s));
            u64 nb = 0;
            u64* cur = eqs;
            for (int k = 0; k < np; k++) {
                LsPoly& p = P[k];
                EqSeg& g = eqsegs[k];
                g.r = d_pts + poff[k];
                g.n = (u64)p.n;
                g.k = (u64)(p.n / 2);
                g.lo = cur;
                cur += 2 * ((size_t)1 << g.k);
                g.hi = cur;
                cur += 2 * ((size_t)1 << (g.n - g.k));
                g.out = p.eq;
                g.block0 = nb;
                nb += ((u64)1 << p.n) / 256 + 1;
            }
            GB_CUDA_TRY(cudaMemcpyAsync(d_eqsegs, eqsegs.data(), (size_t)np * sizeof(EqSeg), cudaMemcpyHostToDevice, s));
            ls_eq_halves_kernel<<<(unsigned)(2 * np), 256, 0, s>>>(d_eqsegs, np);
            GB_LAUNCH_CHECK("ls_eq_halves_kernel");
            ls_eq_expand_kernel<<<(unsigned)nb, 256, 0, s>>>(d_eqsegs, np);
            GB_LAUNCH_CHECK("ls_eq_expand_kernel");
            cudaFreeAsync(eqs, s);
            cudaFreeAsync(d_eqsegs, s);
            cudaFreeAsync(d_pts, s);
            GB_CUDA_TRY(cudaStreamSynchronize(s));  // the host arrays above go out of scope
        }
        // round 0 oracle
        std::vector<int> all(np);
        std::iota(all.begin(), all.end(), 0);
        {
            u64 nb = 0;
            LsSeg* hs = next_slot(); if (!hs) return GB_EINVAL;
            for (int k = 0; k < np; k++) {
                LsPoly& p = P[k];
                hs[k] = LsSeg{p.com->d_evals, p.eq, nullptr, nullptr, 0, 0, p.N / 2, nb};
                nb += blocks_red(p.N / 2);
            }
            const LsSeg* ds = upload(hs, np);
            if (!ds) return GB_ECUDA;
            ls_round0_kernel<<<(unsigned)nb, LS_RED_THREADS, 0, s>>>(ds, np, d_partials_);
            GB_LAUNCH_CHECK("ls_round0_kernel");
            ls_reduce_kernel<<<(unsigned)((np * 32 + 255) / 256), 256, 0, s>>>(ds, np, d_partials_, d_recs_);
            GB_LAUNCH_CHECK("ls_reduce_kernel");
            LS_RC(read_recs(np));
            ls_parallel(np, [&](size_t k) {
                LsPoly& p = P[k];
                const u64* rec = h_recs_ + k * LS_REC;
                E2 c0{rec[0], rec[1]};
                E2 s1 = put_oracle(p, 0, rec);
                E2 ev = e2add(c0, s1);
                p.proof[0] = ev.c0;
                p.proof[1] = ev.c1;
                p.eq_cur = p.eq;
                p.bh_cur = p.com->d_evals;
                p.pp = 0;
                p.sc = p.N;
            });
        }
        // rounds
        std::vector<E2> ch(np);
        for (int rd = 0; rd < maxn; rd++) {
            std::vector<int> mid, last;  // still folding with a tree / final fold
            for (int k = 0; k < np; k++) {
                if (rd >= P[k].n) continue;
                (rd < P[k].n - 1 ? mid : last).push_back(k);
            }
            ls_parallel(np, [&](size_t k) {
                if (rd < P[k].n) ch[k] = tr_challenge_ext2(&P[k].t, "");
            });
            if (!mid.empty()) {
                // eq/bh folds + next oracle
                u64 nb = 0;
                LsSeg* hs = next_slot(); if (!hs) return GB_EINVAL;
                for (size_t m = 0; m < mid.size(); m++) {
                    LsPoly& p = P[mid[m]];
                    size_t quarter = p.sc / 4;
                    hs[m] = LsSeg{p.eq_cur, p.bh_cur, p.bufs_eq[p.pp], p.bufs_bh[p.pp], ch[mid[m]].c0, ch[mid[m]].c1,
                                  quarter, nb};
                    nb += blocks_red(quarter);
                }
                const LsSeg* ds = upload(hs, (int)mid.size());
                if (!ds) return GB_ECUDA;
                if (rd == 0)
                    ls_open_round_kernel<true><<<(unsigned)nb, LS_RED_THREADS, 0, s>>>(ds, (int)mid.size(), d_partials_);
                else
                    ls_open_round_kernel<false><<<(unsigned)nb, LS_RED_THREADS, 0, s>>>(ds, (int)mid.size(), d_partials_);
                GB_LAUNCH_CHECK("ls_open_round_kernel");
                // records of `mid` are written in mid order; the host reads them back by m
                ls_reduce_kernel<<<(unsigned)((mid.size() * 32 + 255) / 256), 256, 0, s>>>(ds, (int)mid.size(),
                                                                                           d_partials_, d_recs_);
                GB_LAUNCH_CHECK("ls_reduce_kernel");
                for (int k : mid) {
                    LsPoly& p = P[k];
                    p.eq_cur = p.bufs_eq[p.pp];
                    p.bh_cur = p.bufs_bh[p.pp];
                    p.pp ^= 1;
                    p.sc /= 2;
                }
                // codeword fold + leaf hash
                nb = 0;
                hs = next_slot(); if (!hs) return GB_EINVAL;
                for (size_t m = 0; m < mid.size(); m++) {
                    LsPoly& p = P[mid[m]];
                    size_t leaves = (p.L >> (rd + 1)) / 2;
                    const u64* cw_in = rd == 0 ? p.com->d_codeword : p.fcw[rd - 1];
                    hs[m] = LsSeg{cw_in, tab_->d_entries + 2 * tab_->level_offsets[rd], p.fcw[rd], p.ftree[rd],
                                  ch[mid[m]].c0, ch[mid[m]].c1, leaves, nb};
                    nb += blocks(leaves);
                }
                const int th = ls_p2_assign(hs, (int)mid.size(), nb);
                ds = upload(hs, (int)mid.size());
                if (!ds) return GB_ECUDA;
                if (th == P2_WIDE) {
                    if (rd == 0) ls_fold_hash_kernel<true, P2_WIDE><<<(unsigned)nb, th, 0, s>>>(ds, (int)mid.size());
                    else ls_fold_hash_kernel<false, P2_WIDE><<<(unsigned)nb, th, 0, s>>>(ds, (int)mid.size());
                } else {
                    if (rd == 0) ls_fold_hash_kernel<true, P2_NARROW><<<(unsigned)nb, th, 0, s>>>(ds, (int)mid.size());
                    else ls_fold_hash_kernel<false, P2_NARROW><<<(unsigned)nb, th, 0, s>>>(ds, (int)mid.size());
                }
                GB_LAUNCH_CHECK("ls_fold_hash_kernel");
                // Merkle layers, all trees at once
                for (int lvl = 0;; lvl++) {
                    int cnt = 0;
                    nb = 0;
                    hs = next_slot(); if (!hs) return GB_EINVAL;
                    for (size_t m = 0; m < mid.size(); m++) {
                        LsPoly& p = P[mid[m]];
                        size_t leaves = (p.L >> (rd + 1)) / 2;
                        size_t nodes = leaves >> lvl;
                        if (nodes < 2) continue;
                        size_t off = 0;
                        for (int l = 0; l < lvl; l++) off += leaves >> l;
                        u64* layer = p.ftree[rd] + 4 * off;
                        hs[cnt++] = LsSeg{layer, nullptr, layer + 4 * nodes, nullptr, 0, 0, nodes / 2, nb};
                        nb += blocks(nodes / 2);
                    }
                    if (!cnt) {
                        unslot();
                        break;
                    }
                    const LsLayerForm form = ls_layer_assign(hs, cnt, coop_, nb);
                    ds = upload(hs, cnt);
                    if (!ds) return GB_ECUDA;
                    LS_RC(ls_layer_launch(form, nb, ds, cnt, s));
                }
                hs = next_slot(); if (!hs) return GB_EINVAL;
                for (size_t m = 0; m < mid.size(); m++) {
                    LsPoly& p = P[mid[m]];
                    size_t leaves = (p.L >> (rd + 1)) / 2;
                    hs[m] = LsSeg{p.ftree[rd] + 4 * (2 * leaves - 2), nullptr, nullptr, nullptr, 0, 0, 0, 0};
                }
                ds = upload(hs, (int)mid.size());
                if (!ds) return GB_ECUDA;
                ls_root_kernel<<<(unsigned)((mid.size() + 127) / 128), 128, 0, s>>>(ds, (int)mid.size(), d_recs_);
                GB_LAUNCH_CHECK("ls_root_kernel");
                LS_RC(read_recs((int)mid.size()));
                ls_parallel(mid.size(), [&](size_t m) {
                    LsPoly& p = P[mid[m]];
                    const u64* rec = h_recs_ + m * LS_REC;
                    put_oracle(p, rd + 1, rec);
                    u64* root = p.proof + 2 + (size_t)p.n * 6 + (size_t)rd * 4;
                    for (int k = 0; k < 4; k++) {
                        root[k] = rec[8 + k];
                        tr_append_u64(&p.t, "", root[k]);
                    }
                });
            }
            if (!last.empty()) {
                LsSeg* hs = next_slot(); if (!hs) return GB_EINVAL;
                for (size_t m = 0; m < last.size(); m++) {
                    LsPoly& p = P[last[m]];
                    size_t pairs = p.L >> (rd + 1);
                    const u64* cw_in = rd == 0 ? p.com->d_codeword : p.fcw[rd - 1];
                    hs[m] = LsSeg{cw_in, tab_->d_entries + 2 * tab_->level_offsets[rd], p.fcw[rd], nullptr,
                                  ch[last[m]].c0, ch[last[m]].c1, pairs, 0};
                }
                const LsSeg* ds = upload(hs, (int)last.size());
                if (!ds) return GB_ECUDA;
                ls_fold_final_kernel<<<(unsigned)last.size(), 32, 0, s>>>(ds, (int)last.size(), d_recs_);
                GB_LAUNCH_CHECK("ls_fold_final_kernel");
                LS_RC(read_recs((int)last.size()));
                for (size_t m = 0; m < last.size(); m++) {
                    LsPoly& p = P[last[m]];
                    u64* fin = p.proof + 2 + (size_t)p.n * 6 + (size_t)(p.n - 1) * 4;
                    for (int k = 0; k < (2 << lr); k++) fin[k] = h_recs_[m * LS_REC + 12 + k];
                }
            }
        }
        // queries: indices from each transcript, one gather launch
        if (q_ > 0) {
            std::vector<QueryJob> jobs(np);
            std::vector<u64> idx((size_t)np * q_), per_q(np);
            std::vector<const u64*> ptrs;
            std::vector<size_t> out_off(np);
            size_t out_words = 0;
            ls_parallel(np, [&](size_t k) {
                LsPoly& p = P[k];
                for (int j = 0; j < q_; j++) idx[k * q_ + j] = tr_challenge(&p.t, "") % (u64)(p.L / 2);
            });
            for (int k = 0; k < np; k++) {
                LsPoly& p = P[k];
                size_t pw = 0;
                for (int r = 0; r < p.n; r++) pw += (size_t)(p.n + lr - 1 - r);
                per_q[k] = 1 + (size_t)p.n * 4 + pw * 4;
                out_off[k] = out_words;
                out_words += per_q[k] * q_;
            }
            // pointer tables: per polynomial fcw[0..n-2] then ftree[0..n-2]
            std::vector<size_t> ptr_off(np);
            for (int k = 0; k < np; k++) {
                ptr_off[k] = ptrs.size();
                for (int r = 0; r + 1 < P[k].n; r++) ptrs.push_back(P[k].fcw[r]);
                for (int r = 0; r + 1 < P[k].n; r++) ptrs.push_back(P[k].ftree[r]);
            }
            u64 *d_idx = nullptr, *d_perq = nullptr, *d_out = nullptr;
            const u64** d_ptrs = nullptr;
            QueryJob* d_jobs = nullptr;
            u64** d_outs = nullptr;
            GB_CUDA_TRY(cudaMallocAsync(&d_idx, idx.size() * 8, s));
            GB_CUDA_TRY(cudaMallocAsync(&d_perq, per_q.size() * 8, s));
            GB_CUDA_TRY(cudaMallocAsync(&d_out, std::max<size_t>(out_words, 1) * 8, s));
            GB_CUDA_TRY(cudaMallocAsync(&d_ptrs, std::max<size_t>(ptrs.size(), 1) * sizeof(u64*), s));
            GB_CUDA_TRY(cudaMallocAsync(&d_jobs, (size_t)np * sizeof(QueryJob), s));
            GB_CUDA_TRY(cudaMallocAsync(&d_outs, (size_t)np * sizeof(u64*), s));
            std::vector<u64*> outs(np);
            for (int k = 0; k < np; k++) {
                LsPoly& p = P[k];
                const u64* const* base = d_ptrs + ptr_off[k];
                jobs[k] = QueryJob{p.com->d_codeword, p.com->d_tree, base, base + (p.n - 1), p.n, lr, false};
                outs[k] = d_out + out_off[k];
            }
            GB_CUDA_TRY(cudaMemcpyAsync(d_idx, idx.data(), idx.size() * 8, cudaMemcpyHostToDevice, s));
            GB_CUDA_TRY(cudaMemcpyAsync(d_perq, per_q.data(), per_q.size() * 8, cudaMemcpyHostToDevice, s));
            if (!ptrs.empty())
                GB_CUDA_TRY(cudaMemcpyAsync(d_ptrs, ptrs.data(), ptrs.size() * sizeof(u64*), cudaMemcpyHostToDevice, s));
            GB_CUDA_TRY(cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(QueryJob), cudaMemcpyHostToDevice, s));
            GB_CUDA_TRY(cudaMemcpyAsync(d_outs, outs.data(), outs.size() * sizeof(u64*), cudaMemcpyHostToDevice, s));
            ls_query_kernel<<<dim3((unsigned)q_, (unsigned)np), 128, 0, s>>>(d_jobs, d_idx, q_, d_outs, d_perq);
            GB_LAUNCH_CHECK("ls_query_kernel");
            std::vector<u64> host_out(out_words);
            GB_CUDA_TRY(cudaMemcpyAsync(host_out.data(), d_out, out_words * 8, cudaMemcpyDeviceToHost, s));
            GB_CUDA_TRY(cudaStreamSynchronize(s));
            for (int k = 0; k < np; k++) {
                LsPoly& p = P[k];
                u64* dst = p.proof + 2 + (size_t)p.n * 6 + (size_t)(p.n - 1) * 4 + ((size_t)2 << lr);
                std::memcpy(dst, host_out.data() + out_off[k], per_q[k] * q_ * 8);
            }
            for (void* x : {(void*)d_idx, (void*)d_perq, (void*)d_out, (void*)d_ptrs, (void*)d_jobs, (void*)d_outs})
                cudaFreeAsync(x, s);
        }
        return GB_OK;
    }

    ~LsRunner() {
        cudaStream_t s = stream();
        if (ws_) cudaFreeAsync(ws_, s);
        if (d_segs_) cudaFreeAsync(d_segs_, s);
        if (d_partials_) cudaFreeAsync(d_partials_, s);
        cudaStreamSynchronize(s);
        if (h_segs_) cudaFreeHost(h_segs_);
        if (h_recs_) cudaFreeHost(h_recs_);
    }

  private:
    static u64 blocks_red(u64 items) {
        u64 per = (u64)LS_RED_THREADS * LS_ITEMS;
        return items ? (items + per - 1) / per : 1;
    }
    static u64 blocks(u64 items) { return items ? (items + LS_THREADS - 1) / LS_THREADS : 1; }
    // Descriptor slots: each launch takes a fresh slot of np entries; the slots are reused only
    // after read_recs, which waits for every launch before it.
    LsSeg* next_slot() {
        if (slot_ + 1 > seg_cap_ / np_max_) return nullptr;
        return h_segs_ + (slot_++) * np_max_;
    }
    void unslot() { slot_--; }
    const LsSeg* upload(const LsSeg* hs, int count) {
        if (!hs) return nullptr;
        size_t off = (size_t)(hs - h_segs_);
        if (cudaMemcpyAsync(d_segs_ + off, hs, (size_t)count * sizeof(LsSeg), cudaMemcpyHostToDevice, stream()) !=
            cudaSuccess)
            return nullptr;
        return d_segs_ + off;
    }
    int read_recs(int) {  // the records are in h_recs_ once the stream is idle
        GB_CUDA_TRY(cudaStreamSynchronize(stream()));
        slot_ = 0;
        return GB_OK;
    }
    // oracle r from a record (c0, s1, c2): c1 = s1 - c0 - c2; written to the proof and the transcript
    static host::E2 put_oracle(LsPoly& p, int r, const u64* rec) {
        using namespace host;
        E2 c0{rec[0], rec[1]}, s1{rec[2], rec[3]}, c2{rec[4], rec[5]};
        E2 c1 = e2sub(e2sub(s1, c0), c2);
        u64* o = p.proof + 2 + (size_t)r * 6;
        o[0] = c0.c0;
        o[1] = c0.c1;
        o[2] = c1.c0;
        o[3] = c1.c1;
        o[4] = c2.c0;
        o[5] = c2.c1;
        tr_append_ext2(&p.t, "", c0);
        tr_append_ext2(&p.t, "", c1);
        tr_append_ext2(&p.t, "", c2);
        return s1;
    }

    const BfTable* tab_;
    int q_;
    size_t coop_;  // layers below this many parents run in the 8-lane form
    u64* ws_ = nullptr;
    LsSeg* d_segs_ = nullptr;
    LsSeg* h_segs_ = nullptr;
    u64* d_recs_ = nullptr;  // device address of h_recs_ (mapped pinned memory)
    u64* h_recs_ = nullptr;
    u64* d_partials_ = nullptr;
    size_t seg_cap_ = 0, np_max_ = 1, slot_ = 0;
};

// Commits of a batch of polynomials (rate 1/2, two copies of one subtree), as commit_device:
// T-transform -> bit-reverse + replicate -> leaf hashes of one copy -> its layers -> copies ->
// top layer.  Each step is one launch for all polynomials.  The commitments' buffers are carved
// from `ws` (see ls_commit_words); d_evals points at the caller's evaluations.
struct LsCommitJob {
    int n = 0;
    const u64* evals = nullptr;
    BfCommitment com;
};

static size_t ls_commit_words(int n) {
    size_t N = (size_t)1 << n, L = 2 * N;
    return N /* transform scratch */ + L /* codeword */ + 4 * (2 * N - 1) + 2 /* tree */;
}

class LsCommitter {
  public:
    explicit LsCommitter(size_t coop) : coop_(coop) {}
    int commit(std::vector<LsCommitJob>& J, u64* ws) {
        cudaStream_t s = stream();
        const int nj = (int)J.size();
        if (!nj) return GB_OK;
        int maxn = 0;
        for (auto& j : J) maxn = std::max(maxn, j.n);
        std::vector<u64*> tmp(nj);
        {
            u64* cur = ws;
            for (int k = 0; k < nj; k++) {
                size_t N = (size_t)1 << J[k].n;
                tmp[k] = cur;
                cur += N;
                J[k].com.num_vars = J[k].n;
                J[k].com.log_rate = 1;
                J[k].com.d_evals = const_cast<u64*>(J[k].evals);
                J[k].com.d_codeword = cur;
                cur += 2 * N;
                J[k].com.d_tree = cur;
                cur += 4 * (2 * N - 1) + 2;
            }
        }
        const size_t cap = (size_t)nj * ((maxn + 3) / 4 * 4 + maxn + 8);
        GB_CUDA_TRY(cudaMallocAsync(&d_segs_, cap * sizeof(LsSeg), s));
        GB_CUDA_TRY(cudaMallocAsync(&d_recs_, (size_t)nj * LS_REC * 8, s));
        GB_CUDA_TRY(cudaMallocHost(&h_segs_, cap * sizeof(LsSeg)));
        GB_CUDA_TRY(cudaMallocHost(&h_recs_, (size_t)nj * LS_REC * 8));
        size_t used = 0;
        auto launch_t = [&](auto kernel, int count, u64 nb, int threads) -> int {
            LsSeg* hs = h_segs_ + used;
            GB_CUDA_TRY(cudaMemcpyAsync(d_segs_ + used, hs, (size_t)count * sizeof(LsSeg), cudaMemcpyHostToDevice, s));
            kernel<<<(unsigned)nb, threads, 0, s>>>(d_segs_ + used, count);
            used += count;
            return check_launch("ls_commit");
        };
        auto launch = [&](auto kernel, int count, u64 nb) -> int { return launch_t(kernel, count, nb, LS_THREADS); };
        // a Merkle layer over the segments at h_segs_ + used, in the form ls_layer_assign picks
        auto launch_layer = [&](int count) -> int {
            u64 nb = 0;
            LsSeg* hs = h_segs_ + used;
            const LsLayerForm form = ls_layer_assign(hs, count, coop_, nb);
            GB_CUDA_TRY(cudaMemcpyAsync(d_segs_ + used, hs, (size_t)count * sizeof(LsSeg), cudaMemcpyHostToDevice, s));
            const int rc = ls_layer_launch(form, nb, d_segs_ + used, count, s);
            used += count;
            return rc;
        };
        // a Poseidon2 kernel (template on its CTA size) over the segments at h_segs_ + used
        auto launch_p2 = [&](auto wide_kernel, auto narrow_kernel, int count) -> int {
            u64 nb = 0;
            const int th = ls_p2_assign(h_segs_ + used, count, nb);
            return th == P2_WIDE ? launch_t(wide_kernel, count, nb, th) : launch_t(narrow_kernel, count, nb, th);
        };
        // 1. transform passes: pass p covers bits [4p, 4p + K) with K = min(4, n - 4p)
        for (int b = 0; b < maxn; b += 4) {
            for (int K = 1; K <= 4; K++) {
                int cnt = 0;
                u64 nb = 0;
                LsSeg* hs = h_segs_ + used;
                for (int k = 0; k < nj; k++) {
                    const int n = J[k].n;
                    if (n <= b || std::min(4, n - b) != K) continue;
                    const u64 groups = ((u64)1 << n) >> K;
                    hs[cnt++] = LsSeg{b == 0 ? J[k].evals : tmp[k], nullptr, tmp[k], nullptr, (u64)b, 0, groups, nb};
                    nb += blocks(groups);
                }
                if (!cnt) continue;
                int rc = K == 4   ? launch(ls_transform_pass_kernel<4>, cnt, nb)
                         : K == 3 ? launch(ls_transform_pass_kernel<3>, cnt, nb)
                         : K == 2 ? launch(ls_transform_pass_kernel<2>, cnt, nb)
                                  : launch(ls_transform_pass_kernel<1>, cnt, nb);
                if (rc) return rc;
            }
        }
        // 2. codeword, 3. first copy's leaves
        {
            LsSeg* hs = h_segs_ + used;
            u64 nb = 0;
            for (int k = 0; k < nj; k++) {
                const u64 L = (u64)2 << J[k].n;
                hs[k] = LsSeg{tmp[k], nullptr, J[k].com.d_codeword, nullptr, (u64)J[k].n, 0, L, nb};
                nb += blocks(L);
            }
            LS_RC(launch(ls_bitrev_replicate_kernel, nj, nb));
            hs = h_segs_ + used;
            nb = 0;
            for (int k = 0; k < nj; k++) {
                const u64 sub = (u64)1 << (J[k].n - 1);
                hs[k] = LsSeg{J[k].com.d_codeword, nullptr, nullptr, J[k].com.d_tree, 0, 0, sub, nb};
                nb += blocks(sub);
            }
            LS_RC(launch_p2(ls_hash_leaves_kernel<P2_WIDE>, ls_hash_leaves_kernel<P2_NARROW>, nj));
        }
        // 4. the first copy's layers (full-tree offsets: layer l holds N >> l nodes)
        for (int l = 0;; l++) {
            int cnt = 0;
            u64 nb = 0;
            LsSeg* hs = h_segs_ + used;
            for (int k = 0; k < nj; k++) {
                const u64 N = (u64)1 << J[k].n, sub = N / 2;
                const u64 parents = sub >> (l + 1);
                if (!parents) continue;
                u64 off = 0;
                for (int t = 0; t < l; t++) off += N >> t;
                u64* layer = J[k].com.d_tree + 4 * off;
                hs[cnt++] = LsSeg{layer, nullptr, layer + 4 * (N >> l), nullptr, 0, 0, parents, nb};
                nb += blocks(parents);
            }
            if (!cnt) break;
            LS_RC(launch_layer(cnt));
        }
        // 5. the second copy on every layer
        {
            LsSeg* hs = h_segs_ + used;
            u64 nb = 0;
            for (int k = 0; k < nj; k++) {
                const u64 N = (u64)1 << J[k].n, sub = N / 2;
                u64 total = 0;
                for (u64 m = sub; m >= 1; m >>= 1) total += 4 * m;
                hs[k] = LsSeg{nullptr, nullptr, J[k].com.d_tree, nullptr, N, sub, total, nb};
                nb += blocks(total);
            }
            LS_RC(launch(ls_replicate_kernel, nj, nb));
        }
        // 6. the top layer: two copy roots -> the root
        {
            LsSeg* hs = h_segs_ + used;
            u64 nb = 0;
            for (int k = 0; k < nj; k++) {
                const int n = J[k].n;
                const u64 N = (u64)1 << n;
                u64 off = 0;
                for (int t = 0; t < n - 1; t++) off += N >> t;  // the layer of 2 nodes
                u64* layer = J[k].com.d_tree + 4 * off;
                hs[k] = LsSeg{layer, nullptr, layer + 8, nullptr, 0, 0, 1, nb};
                nb += 1;
            }
            LS_RC(launch_layer(nj));
            hs = h_segs_ + used;
            for (int k = 0; k < nj; k++) {
                const u64 N = (u64)1 << J[k].n;
                hs[k] = LsSeg{J[k].com.d_tree + 4 * (2 * N - 2), nullptr, nullptr, nullptr, 0, 0, 0, 0};
            }
            GB_CUDA_TRY(cudaMemcpyAsync(d_segs_ + used, hs, (size_t)nj * sizeof(LsSeg), cudaMemcpyHostToDevice, s));
            ls_root_kernel<<<(unsigned)((nj + 127) / 128), 128, 0, s>>>(d_segs_ + used, nj, d_recs_);
            GB_LAUNCH_CHECK("ls_root_kernel");
        }
        GB_CUDA_TRY(cudaMemcpyAsync(h_recs_, d_recs_, (size_t)nj * LS_REC * 8, cudaMemcpyDeviceToHost, s));
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        for (int k = 0; k < nj; k++)
            for (int w = 0; w < 4; w++) J[k].com.root[w] = h_recs_[(size_t)k * LS_REC + 8 + w];
        return GB_OK;
    }
    ~LsCommitter() {
        cudaStream_t s = stream();
        if (d_segs_) cudaFreeAsync(d_segs_, s);
        if (d_recs_) cudaFreeAsync(d_recs_, s);
        cudaStreamSynchronize(s);
        if (h_segs_) cudaFreeHost(h_segs_);
        if (h_recs_) cudaFreeHost(h_recs_);
    }

  private:
    size_t coop_;  // layers below this many parents run in the 8-lane form
    static u64 blocks(u64 items) { return items ? (items + LS_THREADS - 1) / LS_THREADS : 1; }
    LsSeg* d_segs_ = nullptr;
    LsSeg* h_segs_ = nullptr;
    u64* d_recs_ = nullptr;
    u64* h_recs_ = nullptr;
};

// ---------------------------------------------------------------------------
// Product sumchecks of a wave in lockstep.  Round k of every instance still in its protocol is
// one launch per degree (block -> instance by binary search over the segment table), then one
// reduce launch writes every instance's message into mapped pinned records, then one host round
// trip advances every instance's own transcript; the final folds are one launch.  Each instance's
// transcript steps and arithmetic are those of gb_sumcheck_prove_ext2 (sumcheck.cu), so its
// proof is identical to the per-call one.
// ---------------------------------------------------------------------------
constexpr int LSC_MAX_D = 8;
constexpr int LSC_W = 2 * (LSC_MAX_D + 1);  // message words of the largest degree (partials stride)
constexpr int LSC_FIN = 2 * LSC_MAX_D;      // final-value words per instance
constexpr int LSC_ITEMS = 2;                // pairs per thread

struct ScSeg {
    const u64* in;               // this round's input level (the base polynomials in rounds 0 and 1)
    u64* out;                    // the folded level (rounds >= 1)
    u64 in_stride, out_stride;   // elements per polynomial
    u64 r0, r1;                  // the previous round's challenge (rounds >= 1; the last one for the finals)
    u64 items;                   // pairs: input pairs in round 0, output pairs later
    u64 block0;                  // first block of this instance in its launch
    u64 pblock0;                 // its first row of the round's partials
    u64 rec;                     // record slot (position in the wave)
    u64 d;                       // degree
};

__device__ __forceinline__ int sc_find(const ScSeg* __restrict__ segs, int nseg, u64 block) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (segs[mid].block0 <= block) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// MODE 0: round 0 (base input, message only); 1: round 1 (fold the base input into Ext2, message);
// 2: rounds >= 2 (fold Ext2, message).  Same per-pair math as sc_round0_kernel<D, true> and
// sc_fold_round_e2_kernel<D, BASE_IN>.
template <int D, int MODE>
__global__ void __launch_bounds__(RED_THREADS) ls_sc_round_kernel(const ScSeg* __restrict__ segs, int nseg,
                                                                  u64* __restrict__ partials) {
    __shared__ int s_seg;
    if (threadIdx.x == 0) s_seg = sc_find(segs, nseg, blockIdx.x);
    __syncthreads();
    const ScSeg sg = segs[s_seg];
    constexpr int W = 2 * (D + 1);
    u64 acc[W];
#pragma unroll
    for (int w = 0; w < W; w++) acc[w] = 0;
    const bool vec = aligned16(sg.in);
    const e2 r = e2_make(sg.r0, sg.r1);
    const u64 base = (blockIdx.x - sg.block0) * (u64)RED_THREADS * LSC_ITEMS;
#pragma unroll
    for (int it = 0; it < LSC_ITEMS; it++) {
        const u64 y = base + (u64)it * RED_THREADS + threadIdx.x;
        if (y >= sg.items) continue;
        if constexpr (MODE == 0) {
            u64 e[D], dl[D];
#pragma unroll
            for (int i = 0; i < D; i++) {
                u64 a, b;
                ld_pair(sg.in + (size_t)i * sg.in_stride + 2 * y, vec, a, b);
                e[i] = a;
                dl[i] = gl_sub(b, a);
            }
            u64 bacc[D + 1];
#pragma unroll
            for (int c = 0; c <= D; c++) bacc[c] = 0;
            accum_base<D>(e, dl, bacc);
#pragma unroll
            for (int c = 0; c <= D; c++) acc[2 * c] = gl_add(acc[2 * c], bacc[c]);
        } else {
            e2 e[D], dl[D];
#pragma unroll
            for (int i = 0; i < D; i++) {
                e2 a, b;
                if constexpr (MODE == 1) {
                    const u64* p = sg.in + (size_t)i * sg.in_stride + 4 * y;
                    u64 x0, x1, x2, x3;
                    ld_pair(p, vec, x0, x1);
                    ld_pair(p + 2, vec, x2, x3);
                    const u64 d0 = gl_sub(x1, x0), d1 = gl_sub(x3, x2);
                    a = e2_make(gl_add(x0, gl_mul(sg.r0, d0)), gl_mul(sg.r1, d0));
                    b = e2_make(gl_add(x2, gl_mul(sg.r0, d1)), gl_mul(sg.r1, d1));
                } else {
                    const u64* p = sg.in + (size_t)i * 2 * sg.in_stride + 8 * y;
                    const e2 x0 = ld_e2(p, true), x1 = ld_e2(p + 2, true), x2 = ld_e2(p + 4, true),
                             x3 = ld_e2(p + 6, true);
                    a = e2_add(x0, e2_mul(r, e2_sub(x1, x0)));
                    b = e2_add(x2, e2_mul(r, e2_sub(x3, x2)));
                }
                u64* q = sg.out + (size_t)i * 2 * sg.out_stride + 4 * y;
                e2_st(q, a);
                e2_st(q + 2, b);
                e[i] = a;
                dl[i] = e2_sub(b, a);
            }
            accum_e2<D>(e, dl, acc);
        }
    }
    block_reduce<W>(acc);
    if (threadIdx.x == 0) {
        u64* dst = partials + (sg.pblock0 + (blockIdx.x - sg.block0)) * LSC_W;
#pragma unroll
        for (int w = 0; w < W; w++) dst[w] = acc[w];
    }
}

static u64 lsc_blocks(u64 items) {
    const u64 per = (u64)RED_THREADS * LSC_ITEMS;
    return items ? (items + per - 1) / per : 1;
}

// each instance's message: the sum of its blocks' partials, canonical; one warp per instance
__global__ void ls_sc_reduce_kernel(const ScSeg* __restrict__ segs, int nseg, const u64* __restrict__ partials,
                                    u64* __restrict__ recs) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= nseg) return;
    const ScSeg sg = segs[w];
    const u64 per = (u64)RED_THREADS * LSC_ITEMS;
    const u64 nb = sg.items ? (sg.items + per - 1) / per : 1;
    const int words = 2 * ((int)sg.d + 1);
    u64 acc[LSC_W];
#pragma unroll
    for (int k = 0; k < LSC_W; k++) acc[k] = 0;
    for (u64 b = lane; b < nb; b += 32)
#pragma unroll
        for (int k = 0; k < LSC_W; k++)
            if (k < words) acc[k] = gl_add(acc[k], partials[(sg.pblock0 + b) * LSC_W + k]);
#pragma unroll
    for (int k = 0; k < LSC_W; k++) {
        const u64 v = gl_warp_sum(acc[k]);
        if (lane == 0 && k < words) recs[sg.rec * LSC_W + k] = gl_canon(v);
    }
}

// each instance's final values: its last level (2 elements per polynomial) folded with its last
// challenge; one block per instance, thread i folds polynomial i (as sc_final_kernel<true, false>)
__global__ void ls_sc_final_kernel(const ScSeg* __restrict__ segs, int nseg, u64* __restrict__ fins) {
    if ((int)blockIdx.x >= nseg) return;
    const ScSeg sg = segs[blockIdx.x];
    const int i = threadIdx.x;
    if (i >= (int)sg.d) return;
    const u64* p = sg.in + (size_t)i * 2 * sg.in_stride;
    const e2 a = e2_make(p[0], p[1]), b = e2_make(p[2], p[3]);
    const e2 f = e2_canon(e2_add(a, e2_mul(e2_make(sg.r0, sg.r1), e2_sub(b, a))));
    fins[sg.rec * LSC_FIN + 2 * i] = f.c0;
    fins[sg.rec * LSC_FIN + 2 * i + 1] = f.c1;
}

template <int D>
static void lsc_launch(int mode, unsigned blocks, const ScSeg* segs, int nseg, u64* partials, cudaStream_t s) {
    if (mode == 0) ls_sc_round_kernel<D, 0><<<blocks, RED_THREADS, 0, s>>>(segs, nseg, partials);
    else if (mode == 1) ls_sc_round_kernel<D, 1><<<blocks, RED_THREADS, 0, s>>>(segs, nseg, partials);
    else ls_sc_round_kernel<D, 2><<<blocks, RED_THREADS, 0, s>>>(segs, nseg, partials);
}
static void lsc_launch_d(int d, int mode, unsigned blocks, const ScSeg* segs, int nseg, u64* partials, cudaStream_t s) {
    switch (d) {
        case 1: lsc_launch<1>(mode, blocks, segs, nseg, partials, s); break;
        case 2: lsc_launch<2>(mode, blocks, segs, nseg, partials, s); break;
        case 3: lsc_launch<3>(mode, blocks, segs, nseg, partials, s); break;
        case 4: lsc_launch<4>(mode, blocks, segs, nseg, partials, s); break;
        case 5: lsc_launch<5>(mode, blocks, segs, nseg, partials, s); break;
        case 6: lsc_launch<6>(mode, blocks, segs, nseg, partials, s); break;
        case 7: lsc_launch<7>(mode, blocks, segs, nseg, partials, s); break;
        default: lsc_launch<8>(mode, blocks, segs, nseg, partials, s); break;
    }
}

// The product sumchecks of the wave's instances (their roots already in their proofs), all
// rounds in lockstep.  polys[k]: instance wave[k]'s d base polynomials of 2^n values on the device.
static int ls_sumchecks(const u64 seed[2], const gb_instance* insts, const std::vector<int>& wave,
                        const std::vector<const u64*>& polys) {
    using namespace host;
    cudaStream_t s = stream();
    const int nw = (int)wave.size();
    if (!nw) return GB_OK;
    struct St {
        int n = 0, d = 0;
        u64 N = 0;
        u64* buf[2] = {nullptr, nullptr};
        const u64* cur = nullptr;
        u64 cur_stride = 0;
        int pp = 0;
        E2 r{0, 0};
        gb_transcript t;
    };
    std::vector<St> st(nw);
    size_t ws_words = 0, max_blocks = 1;
    int maxn = 0;
    for (int k = 0; k < nw; k++) {
        const gb_instance& in = insts[wave[k]];
        St& x = st[k];
        x.n = in.num_vars;
        x.d = in.degree;
        x.N = (u64)1 << x.n;
        maxn = std::max(maxn, x.n);
        ws_words += 2 * (size_t)x.d * x.N;  // two levels of d x N/2 Ext2 values
        max_blocks += lsc_blocks(x.N >> 1);
    }
    u64 *ws = nullptr, *partials = nullptr, *h_recs = nullptr, *d_recs = nullptr;
    ScSeg *h_segs = nullptr, *d_segs = nullptr;
    int rc = GB_OK;
    auto cleanup = [&] {
        if (ws) cudaFreeAsync(ws, s);
        if (partials) cudaFreeAsync(partials, s);
        if (d_segs) cudaFreeAsync(d_segs, s);
        cudaStreamSynchronize(s);
        if (h_recs) cudaFreeHost(h_recs);
        if (h_segs) cudaFreeHost(h_segs);
    };
    auto fail = [&](const char* where, cudaError_t e) {
        set_error(where, e);
        cleanup();
        return GB_ECUDA;
    };
    cudaError_t e = cudaMallocAsync(&ws, ws_words * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&partials, max_blocks * LSC_W * 8, s);
    if (e == cudaSuccess) e = cudaMallocAsync(&d_segs, (size_t)nw * sizeof(ScSeg), s);
    if (e == cudaSuccess) e = cudaMallocHost(&h_recs, (size_t)nw * (LSC_W + LSC_FIN) * 8);
    if (e == cudaSuccess) e = cudaMallocHost(&h_segs, (size_t)nw * sizeof(ScSeg));
    if (e == cudaSuccess) {
        void* d = nullptr;
        e = cudaHostGetDevicePointer(&d, h_recs, 0);
        d_recs = (u64*)d;
    }
    if (e != cudaSuccess) return fail("lockstep sumcheck workspace", e);
    u64* h_fins = h_recs + (size_t)nw * LSC_W;
    u64* d_fins = d_recs + (size_t)nw * LSC_W;
    {
        u64* cur = ws;
        for (int k = 0; k < nw; k++) {
            St& x = st[k];
            x.buf[0] = cur;
            cur += (size_t)x.d * x.N;
            x.buf[1] = cur;
            cur += (size_t)x.d * x.N;
            x.cur = polys[k];
            x.cur_stride = x.N;
        }
    }
    // each instance's transcript, up to its first round (ls_sumcheck, gb_sumcheck_prove_ext2)
    ls_parallel(nw, [&](size_t k) {
        const gb_instance& in = insts[wave[k]];
        St& x = st[k];
        gb_transcript_new(&x.t, "sumcheck");
        tr_append_ext2(&x.t, "", E2{canon(seed[0]), canon(seed[1])});
        tr_append_u64(&x.t, "", in.index);
        for (int w = 0; w < 4 * x.d; w++) tr_append_u64(&x.t, "", in.h_proof[w]);
        tr_append_u64(&x.t, "num_var", (u64)x.n);
        tr_append_u64(&x.t, "num_poly", (u64)x.d);
    });
    std::vector<int> active;
    for (int k = 0; k < maxn && !rc; k++) {
        // the instances still in the protocol, grouped by degree
        active.clear();
        for (int dd = 1; dd <= LSC_MAX_D; dd++)
            for (int w = 0; w < nw; w++)
                if (st[w].d == dd && st[w].n > k) active.push_back(w);
        const int mode = k == 0 ? 0 : k == 1 ? 1 : 2;
        u64 pblock = 0;
        for (size_t a = 0; a < active.size(); a++) {
            St& x = st[active[a]];
            ScSeg& g = h_segs[a];
            g.in = x.cur;
            g.in_stride = x.cur_stride;
            g.out = k == 0 ? nullptr : x.buf[x.pp];
            g.out_stride = x.N >> 1;
            g.r0 = x.r.c0;
            g.r1 = x.r.c1;
            g.items = x.N >> (k + 1);
            g.pblock0 = pblock;
            g.rec = (u64)active[a];
            g.d = (u64)x.d;
            pblock += lsc_blocks(g.items);
        }
        // block0 is relative to the launch of the segment's degree
        for (size_t a = 0; a < active.size();) {
            size_t b = a;
            u64 nb = 0;
            while (b < active.size() && st[active[b]].d == st[active[a]].d) {
                h_segs[b].block0 = nb;
                nb += lsc_blocks(h_segs[b].items);
                b++;
            }
            a = b;
        }
        e = cudaMemcpyAsync(d_segs, h_segs, active.size() * sizeof(ScSeg), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return fail("lockstep sumcheck segments", e);
        for (size_t a = 0; a < active.size();) {
            size_t b = a;
            u64 nb = 0;
            while (b < active.size() && st[active[b]].d == st[active[a]].d) nb += lsc_blocks(h_segs[b++].items);
            lsc_launch_d(st[active[a]].d, mode, (unsigned)nb, d_segs + a, (int)(b - a), partials, s);
            rc = check_launch("ls_sc_round_kernel");
            if (rc) break;
            a = b;
        }
        if (rc) break;
        ls_sc_reduce_kernel<<<(unsigned)((active.size() * 32 + 255) / 256), 256, 0, s>>>(d_segs, (int)active.size(),
                                                                                        partials, d_recs);
        rc = check_launch("ls_sc_reduce_kernel");
        if (rc) break;
        // every instance's first message label does not depend on the message: absorb it while the
        // round runs on the device (the absorb sequence is unchanged)
        ls_parallel(active.size(), [&](size_t a) { tr_label(&st[active[a]].t, "round_message"); });
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return fail("lockstep sumcheck round", e);
        ls_parallel(active.size(), [&](size_t a) {
            const int w = active[a];
            St& x = st[w];
            const gb_instance& in = insts[wave[w]];
            const int words = 2 * (x.d + 1);
            const u64* m = h_recs + (size_t)w * LSC_W;
            u64* msgs = in.h_proof + (size_t)x.d * 4 + (size_t)k * words;
            for (int c = 0; c < words; c++) msgs[c] = m[c];
            tr_absorb(&x.t, m[0]);
            tr_absorb(&x.t, m[1]);
            for (int c = 1; c <= x.d; c++) tr_append_ext2(&x.t, "round_message", E2{m[2 * c], m[2 * c + 1]});
            x.r = tr_challenge_ext2(&x.t, "challenge");
            u64* chal = in.h_proof + (size_t)x.d * 4 + (size_t)x.n * words;
            chal[2 * k] = x.r.c0;
            chal[2 * k + 1] = x.r.c1;
            if (k >= 1) {
                x.cur = x.buf[x.pp];
                x.cur_stride = x.N >> 1;
                x.pp ^= 1;
            }
        });
    }
    if (!rc) {
        // the final values: every instance's last level folded with its last challenge
        for (int w = 0; w < nw; w++) {
            St& x = st[w];
            ScSeg& g = h_segs[w];
            g = ScSeg{};
            g.in = x.cur;
            g.in_stride = x.cur_stride;
            g.r0 = x.r.c0;
            g.r1 = x.r.c1;
            g.rec = (u64)w;
            g.d = (u64)x.d;
        }
        e = cudaMemcpyAsync(d_segs, h_segs, (size_t)nw * sizeof(ScSeg), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return fail("lockstep sumcheck finals", e);
        ls_sc_final_kernel<<<(unsigned)nw, 32, 0, s>>>(d_segs, nw, d_fins);
        rc = check_launch("ls_sc_final_kernel");
        if (!rc) {
            e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return fail("lockstep sumcheck finals", e);
            for (int w = 0; w < nw; w++) {
                St& x = st[w];
                const gb_instance& in = insts[wave[w]];
                const int words = 2 * (x.d + 1);
                u64* finals = in.h_proof + (size_t)x.d * 4 + (size_t)x.n * words + (size_t)x.n * 2;
                E2 fe{1, 0};
                for (int i = 0; i < x.d; i++) {
                    finals[2 * i] = h_fins[(size_t)w * LSC_FIN + 2 * i];
                    finals[2 * i + 1] = h_fins[(size_t)w * LSC_FIN + 2 * i + 1];
                    fe = e2mul(fe, E2{finals[2 * i], finals[2 * i + 1]});
                }
                finals[2 * x.d] = fe.c0;
                finals[2 * x.d + 1] = fe.c1;
            }
        }
    }
    cleanup();
    return rc;
}

// ---------------------------------------------------------------------------
// driver: waves of instances; commits + sumchecks on worker threads, openings in lockstep
// ---------------------------------------------------------------------------
// words of an instance proof before its openings (batch.cu's layout)
static size_t inst_proof_words_before_opens(int n, int d) {
    return (size_t)d * 4 + (size_t)n * (d + 1) * 2 + (size_t)n * 2 + (size_t)d * 2 + 2;
}

static size_t ls_inst_bytes(const gb_instance& in) {
    size_t N = (size_t)1 << in.num_vars;
    // uploaded inputs, commitment workspace, the sumcheck's levels and the opening workspace,
    // per polynomial
    return (size_t)in.degree * (N * (8 + 16) + (ls_commit_words(in.num_vars) + ls_poly_words(in.num_vars, 1)) * 8) +
           ((size_t)1 << 20);
}

// wall time of the last lockstep batch on this thread: commits + sumchecks, openings
static thread_local double t_ls_ms[3] = {0, 0, 0};  // commit + sumcheck, open, of which sumcheck

// parts[0] on the calling thread and its stream; parts[k] (k >= 1) on helper thread k with a stream
// of its own that starts after the work already queued on the caller's stream.  Synchronising;
// returns the first failing part's code (in part order) with its message.
static int ls_on_streams(const std::vector<std::function<int()>>& parts) {
    if (parts.empty()) return GB_OK;
    if (parts.size() == 1) return parts[0]();
    cudaStream_t s = stream();
    int dev = 0;
    cudaEvent_t ready = nullptr;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ready, s);
    if (e != cudaSuccess) {
        if (ready) cudaEventDestroy(ready);
        set_error("lockstep helper streams", e);
        return GB_ECUDA;
    }
    const size_t n = parts.size();
    std::vector<int> rcs(n, GB_OK);
    std::vector<std::string> errs(n);
    std::vector<std::thread> helpers;
    for (size_t k = 1; k < n; k++)
        helpers.emplace_back([&, k] {
            cudaStream_t st = nullptr;
            cudaError_t he = cudaSetDevice(dev);
            if (he == cudaSuccess) he = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
            if (he == cudaSuccess) he = cudaStreamWaitEvent(st, ready, 0);
            if (he != cudaSuccess) {
                // the part still runs (on this thread's default stream), so that what it signals to
                // the other parts happens; the failure is reported
                if (st) cudaStreamDestroy(st);
                st = nullptr;
                parts[k]();
                rcs[k] = GB_ECUDA;
                errs[k] = std::string("lockstep helper stream: ") + cudaGetErrorString(he);
            } else {
                gb_set_stream(st);
                rcs[k] = parts[k]();
                if (rcs[k]) errs[k] = gb_last_error();
                cudaStreamSynchronize(st);
                gb_set_stream(nullptr);
            }
            if (st) cudaStreamDestroy(st);
        });
    rcs[0] = parts[0]();
    if (rcs[0]) errs[0] = gb_last_error();
    for (auto& t : helpers) t.join();
    cudaEventDestroy(ready);
    for (size_t k = 0; k < n; k++)
        if (rcs[k]) {
            set_error_msg(errs[k]);
            return rcs[k];
        }
    return GB_OK;
}

// Schedule of the calling thread's lockstep batches (gb_set_lockstep_schedule): the wave's
// instances in this many staggered groups, each group's openings in this many parts.
static thread_local int t_ls_groups = 2, t_ls_open_parts = 2;

// One group of a wave, on the calling thread's stream: inputs on the device, the commits of every
// polynomial in lockstep (roots into the proofs), then `committed()` (called exactly once, also
// on failure), the product sumchecks in lockstep and the openings in lockstep, in `open_parts`
// parts on as many streams.  Synchronising.
static int ls_prove_group(const BfTable* tab, const u64 seed[2], int q, const gb_instance* insts,
                          const std::vector<int>& wave, size_t coop, int open_parts,
                          const std::function<void()>& committed) {
    using namespace host;
    bool signalled = false;
    auto signal = [&] {
        if (!signalled) committed();
        signalled = true;
    };
    auto t0 = std::chrono::steady_clock::now();
    cudaStream_t s = stream();
    // inputs on the device
    std::vector<const u64*> polys(wave.size());
    std::vector<u64*> owned(wave.size(), nullptr);
    int rc = GB_OK;
    for (size_t k = 0; k < wave.size() && !rc; k++) {
        const gb_instance& in = insts[wave[k]];
        if (in.h_polys) {
            size_t bytes = ((size_t)in.degree << in.num_vars) * 8;
            cudaError_t e = cudaMallocAsync(&owned[k], bytes, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(owned[k], in.h_polys, bytes, cudaMemcpyHostToDevice, s);
            if (e != cudaSuccess) {
                set_error("input upload", e);
                rc = GB_ECUDA;
            }
            polys[k] = owned[k];
        } else {
            polys[k] = in.d_polys;
        }
    }
    // commits of every polynomial of the group, in lockstep
    std::vector<LsCommitJob> jobs;
    std::vector<size_t> first_job(wave.size());
    size_t cwords = 0;
    for (size_t k = 0; k < wave.size(); k++) {
        const gb_instance& in = insts[wave[k]];
        first_job[k] = jobs.size();
        for (int j = 0; j < in.degree; j++) {
            LsCommitJob cj;
            cj.n = in.num_vars;
            cj.evals = polys[k] + ((size_t)j << in.num_vars);
            jobs.push_back(cj);
            cwords += ls_commit_words(in.num_vars);
        }
    }
    u64* cws = nullptr;
    if (!rc) {
        cudaError_t e = cudaMallocAsync(&cws, std::max<size_t>(cwords, 2) * 8, s);
        if (e != cudaSuccess) {
            set_error("commit workspace", e);
            rc = GB_ECUDA;
        }
    }
    if (!rc) {
        LsCommitter committer(coop);
        rc = committer.commit(jobs, cws);
    }
    signal();
    if (!rc)
        for (size_t k = 0; k < wave.size(); k++) {
            const gb_instance& in = insts[wave[k]];
            for (int j = 0; j < in.degree; j++)
                for (int w = 0; w < 4; w++) in.h_proof[4 * j + w] = jobs[first_job[k] + j].com.root[w];
        }
    // product sumchecks of the group, all rounds in lockstep
    const auto ts = std::chrono::steady_clock::now();
    if (!rc) {
        // on a stream of the highest priority: the sumchecks are a chain of small launches and
        // host round trips, which another group's commit or open launches would otherwise delay
        int lo = 0, hi = 0;
        cudaStream_t hs = nullptr;
        cudaEvent_t inputs = nullptr;
        cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&hs, cudaStreamNonBlocking, hi);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&inputs, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(inputs, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(hs, inputs, 0);
        if (e != cudaSuccess) {
            set_error("lockstep sumcheck stream", e);
            rc = GB_ECUDA;
        } else {
            gb_set_stream(hs);
            rc = ls_sumchecks(seed, insts, wave, polys);  // synchronises hs before it returns
            gb_set_stream(s);
        }
        if (inputs) cudaEventDestroy(inputs);
        if (hs) cudaStreamDestroy(hs);
    }
    t_ls_ms[2] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - ts).count();
    auto t1 = std::chrono::steady_clock::now();
    t_ls_ms[0] += std::chrono::duration<double, std::milli>(t1 - t0).count();
    if (!rc) {
        // openings of every polynomial of the group, in lockstep
        std::vector<LsPoly> P;
        for (size_t k = 0; k < wave.size(); k++) {
            const gb_instance& in = insts[wave[k]];
            const int n = in.num_vars, d = in.degree;
            const size_t plen = gb_basefold_proof_len(n, 1, q);
            const u64* chal = in.h_proof + (size_t)d * 4 + (size_t)n * (d + 1) * 2;
            u64* opens = in.h_proof + inst_proof_words_before_opens(n, d);
            for (int j = 0; j < d; j++) {
                LsPoly p;
                p.n = n;
                p.N = (size_t)1 << n;
                p.L = p.N << 1;
                p.com = &jobs[first_job[k] + j].com;
                p.point = chal;
                gb_transcript_new(&p.t, "bf-open");
                tr_append_ext2(&p.t, "", E2{canon(seed[0]), canon(seed[1])});
                tr_append_u64(&p.t, "", 8 * in.index + (u64)j);
                p.proof = opens + (size_t)j * plen;
                P.push_back(std::move(p));
            }
        }
        // open_parts parts of the polynomials (dealt out in size order, so that each carries about
        // the same work), each opened by its own runner: part 0 on this thread, the others on
        // helper threads with streams of their own, so that one part's host round trip between
        // rounds overlaps the others' device work
        std::vector<size_t> idx(P.size());
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) { return P[a].N > P[b].N; });
        const size_t np = std::max<size_t>(1, std::min<size_t>((size_t)open_parts, P.size()));
        std::vector<std::vector<LsPoly>> part(np);
        for (size_t k = 0; k < idx.size(); k++) part[k % np].push_back(std::move(P[idx[k]]));
        std::vector<std::function<int()>> runs;
        for (size_t k = 0; k < np; k++)
            runs.push_back([&, k] {
                LsRunner runner(tab, q, coop);
                return runner.open(part[k]);
            });
        rc = ls_on_streams(runs);
        t_ls_ms[1] += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
    }
    if (cws) cudaFreeAsync(cws, s);
    for (size_t k = 0; k < wave.size(); k++)
        if (owned[k]) cudaFreeAsync(owned[k], s);
    if (rc) {
        cudaStreamSynchronize(s);
        return rc;
    }
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    return GB_OK;
}

static int lockstep_prove(void* table, const u64 seed[2], int q, const gb_instance* insts, int count, int workers,
                          size_t budget) {
    using namespace host;
    const BfTable* tab = (const BfTable*)table;
    if (!tab || !seed || count < 0 || (count && !insts) || workers < 1 || q < 0 || tab->log_rate != 1) {
        set_error_msg("gb_batch_prove_lockstep: invalid argument (the table must have log_rate 1)");
        return GB_EINVAL;
    }
    for (int i = 0; i < count; i++) {
        const gb_instance& in = insts[i];
        if (in.num_vars < 2 || in.num_vars > 30 || in.degree < 1 || in.degree > 8 || (!in.h_polys == !in.d_polys) ||
            !in.h_proof || tab->num_vars < in.num_vars || tab->num_rounds < in.num_vars) {
            set_error_msg("gb_batch_prove_lockstep: invalid instance " + std::to_string(i));
            return GB_EINVAL;
        }
    }
    std::vector<int> order(count);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return ls_inst_bytes(insts[a]) > ls_inst_bytes(insts[b]); });
    const size_t coop = gb_get_coop_threshold();  // the 8-lane form below this many parents a layer
    const int groups = t_ls_groups, open_parts = t_ls_open_parts;
    t_ls_ms[0] = t_ls_ms[1] = t_ls_ms[2] = 0;
    size_t next = 0;
    while (next < order.size()) {
        // the wave: largest remaining first, as many as fit the budget (at least one)
        std::vector<int> wave;
        size_t used = 0;
        while (next < order.size() && (wave.empty() || used + ls_inst_bytes(insts[order[next]]) <= budget)) {
            used += ls_inst_bytes(insts[order[next]]);
            wave.push_back(order[next++]);
        }
        // `groups` groups (dealt out in size order), staggered: group k + 1's commits start once
        // group k's are done, so they run beside group k's sumchecks (a chain of host round trips
        // with little device work), and group k's openings beside group k + 1's sumchecks.  Each
        // group's proofs are those it gives alone.
        const int G = std::max(1, std::min(groups, (int)wave.size()));
        std::vector<std::vector<int>> grp(G);
        for (size_t k = 0; k < wave.size(); k++) grp[k % G].push_back(wave[k]);
        std::mutex mu;
        std::condition_variable cv;
        int committed = 0;  // groups whose commits are done
        std::vector<std::function<int()>> parts;
        for (int k = 0; k < G; k++)
            parts.push_back([&, k] {
                if (k > 0) {
                    std::unique_lock<std::mutex> l(mu);
                    cv.wait(l, [&] { return committed >= k; });
                }
                return ls_prove_group(tab, seed, q, insts, grp[k], coop, open_parts, [&, k] {
                    {
                        std::lock_guard<std::mutex> l(mu);
                        committed = std::max(committed, k + 1);
                    }
                    cv.notify_all();
                });
            });
        const int rc = ls_on_streams(parts);
        if (rc) return rc;
    }
    return GB_OK;
}

// ---------------------------------------------------------------------------
// Continuous open engine (open_engine.cuh): the rounds of LsRunner::open, with every polynomial
// at its own round.  Step = one round for all polynomials in flight: the eq/bh fold + oracle
// partials and the codeword fold + leaf hash go out as one launch per input kind (round 0 reads
// base-field inputs, later rounds Ext2), the Merkle layers as one launch per layer over every
// tree, then roots and final folds; one host round trip advances each transcript.  Joining
// polynomials get their eq tables and round-0 oracles at the step boundary; finished ones their
// queries, in one gather launch.
// ---------------------------------------------------------------------------
struct EngPoly : LsPoly {
    int rd = 0;
    u64* ws = nullptr;
    OpenTask task;
};

class OpenEngine {
  public:
    OpenEngine(const BfTable* tab, int q, int device)
        : tab_(tab), q_(q), device_(device), coop_(gb_get_coop_threshold()) {
        th_ = std::thread([this] { run(); });
        std::unique_lock<std::mutex> l(mu_);
        cv_.wait(l, [this] { return started_; });
    }
    ~OpenEngine() {
        {
            std::lock_guard<std::mutex> l(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
    }
    int start_rc() const { return start_rc_; }
    void submit(OpenTask&& t) {
        {
            std::lock_guard<std::mutex> l(mu_);
            intake_.push_back(std::move(t));
            waiting_++;
        }
        cv_.notify_all();
    }
    size_t in_flight() {
        std::lock_guard<std::mutex> l(mu_);
        return waiting_;
    }

  private:
    using PolyList = std::vector<EngPoly*>;

    void run() {
        cudaStream_t st = nullptr;
        cudaError_t e = cudaSetDevice(device_);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        {
            std::lock_guard<std::mutex> l(mu_);
            start_rc_ = e == cudaSuccess ? GB_OK : GB_ECUDA;
            started_ = true;
        }
        cv_.notify_all();
        if (e != cudaSuccess) return;
        gb_set_stream(st);
        for (;;) {
            std::vector<OpenTask> in;
            {
                std::unique_lock<std::mutex> l(mu_);
                cv_.wait(l, [&] { return stop_ || !intake_.empty() || !active_.empty(); });
                if (intake_.empty() && active_.empty()) break;  // stop, with nothing left
                in.swap(intake_);
            }
            int rc = GB_OK;
            if (!in.empty()) rc = join(in);
            if (!rc && !active_.empty()) rc = step();
            if (!rc) rc = finish();
            if (rc) fail_all(rc, gb_last_error());
        }
        cudaStreamSynchronize(st);
        release_buffers();
        gb_set_stream(nullptr);
        cudaStreamDestroy(st);
    }

    // carve one polynomial's workspace (the layout of LsRunner::open)
    static void carve(EngPoly& p) {
        u64* cur = p.ws;
        p.d_point = cur;
        cur += align2(2 * (size_t)p.n);
        p.eq = cur;
        cur += 2 * p.N;
        p.bufs_eq[0] = cur;
        cur += p.N;
        p.bufs_eq[1] = cur;
        cur += p.N;
        p.bufs_bh[0] = cur;
        cur += p.N;
        p.bufs_bh[1] = cur;
        cur += p.N;
        p.fcw.assign(p.n, nullptr);
        p.ftree.assign(p.n - 1, nullptr);
        for (int r = 0; r < p.n; r++) {
            p.fcw[r] = cur;
            cur += align2(2 * (p.L >> (r + 1)));
        }
        for (int r = 0; r + 1 < p.n; r++) {
            p.ftree[r] = cur;
            cur += 4 * (2 * ((p.L >> (r + 1)) / 2) - 1) + 2;
        }
    }

    // Per-step buffers sized for the polynomials in flight (called with the stream idle).
    int reserve(size_t polys, int maxn, size_t partial_blocks) {
        cudaStream_t s = stream();
        const size_t segs = polys * (size_t)(maxn + 8);
        if (segs > seg_cap_) {
            if (d_segs_) cudaFreeAsync(d_segs_, s);
            if (h_segs_) cudaFreeHost(h_segs_);
            d_segs_ = nullptr;
            h_segs_ = nullptr;
            seg_cap_ = std::max(segs, 2 * seg_cap_);
            GB_CUDA_TRY(cudaMallocAsync(&d_segs_, seg_cap_ * sizeof(LsSeg), s));
            GB_CUDA_TRY(cudaMallocHost(&h_segs_, seg_cap_ * sizeof(LsSeg)));
        }
        if (polys > rec_cap_) {
            if (h_recs_) cudaFreeHost(h_recs_);
            h_recs_ = nullptr;
            rec_cap_ = std::max(polys, 2 * rec_cap_);
            GB_CUDA_TRY(cudaMallocHost(&h_recs_, rec_cap_ * LS_REC * 8));
            void* d = nullptr;
            GB_CUDA_TRY(cudaHostGetDevicePointer(&d, h_recs_, 0));
            d_recs_ = (u64*)d;
        }
        if (partial_blocks > part_cap_) {
            if (d_partials_) cudaFreeAsync(d_partials_, s);
            d_partials_ = nullptr;
            part_cap_ = std::max(partial_blocks, 2 * part_cap_);
            GB_CUDA_TRY(cudaMallocAsync(&d_partials_, part_cap_ * 6 * 8, s));
        }
        seg_used_ = 0;
        return GB_OK;
    }
    void release_buffers() {
        cudaStream_t s = stream();
        if (d_segs_) cudaFreeAsync(d_segs_, s);
        if (d_partials_) cudaFreeAsync(d_partials_, s);
        cudaStreamSynchronize(s);
        if (h_segs_) cudaFreeHost(h_segs_);
        if (h_recs_) cudaFreeHost(h_recs_);
        d_segs_ = nullptr;
        h_segs_ = nullptr;
        h_recs_ = nullptr;
        d_partials_ = nullptr;
        seg_cap_ = rec_cap_ = part_cap_ = 0;
    }
    // descriptor entries for one launch (valid until the next synchronisation)
    LsSeg* segs(size_t count) {
        if (seg_used_ + count > seg_cap_) return nullptr;
        LsSeg* p = h_segs_ + seg_used_;
        seg_used_ += count;
        return p;
    }
    const LsSeg* upload(const LsSeg* hs, size_t count) {
        if (!hs) return nullptr;
        const size_t off = (size_t)(hs - h_segs_);
        if (cudaMemcpyAsync(d_segs_ + off, hs, count * sizeof(LsSeg), cudaMemcpyHostToDevice, stream()) != cudaSuccess)
            return nullptr;
        return d_segs_ + off;
    }
    static u64 blocks_red(u64 items) {
        const u64 per = (u64)LS_RED_THREADS * LS_ITEMS;
        return items ? (items + per - 1) / per : 1;
    }
    static host::E2 put_oracle(LsPoly& p, int r, const u64* rec) {
        using namespace host;
        E2 c0{rec[0], rec[1]}, s1{rec[2], rec[3]}, c2{rec[4], rec[5]};
        E2 c1 = e2sub(e2sub(s1, c0), c2);
        u64* o = p.proof + 2 + (size_t)r * 6;
        o[0] = c0.c0;
        o[1] = c0.c1;
        o[2] = c1.c0;
        o[3] = c1.c1;
        o[4] = c2.c0;
        o[5] = c2.c1;
        tr_append_ext2(&p.t, "", c0);
        tr_append_ext2(&p.t, "", c1);
        tr_append_ext2(&p.t, "", c2);
        return s1;
    }
    int sync() {
        GB_CUDA_TRY(cudaStreamSynchronize(stream()));
        seg_used_ = 0;
        return GB_OK;
    }
    size_t partial_need() const {
        size_t b = 0;
        for (auto& p : active_) b += blocks_red(p->N / 2) + 1;
        return b;
    }
    int max_vars() const {
        int m = 1;
        for (auto& p : active_) m = std::max(m, p->n);
        return m;
    }

    // new openings: workspaces, transcript preambles, eq tables and round-0 oracles
    int join(std::vector<OpenTask>& in) {
        using namespace host;
        cudaStream_t s = stream();
        PolyList P;
        // ownership moves to active_ first, so that a failure below reaches every callback
        for (auto& t : in) {
            auto p = std::make_unique<EngPoly>();
            p->task = std::move(t);
            p->n = p->task.com->num_vars;
            p->N = (size_t)1 << p->n;
            p->L = p->N << 1;
            p->com = p->task.com;
            p->point = p->task.point.data();
            p->t = p->task.t;
            p->proof = p->task.proof;
            P.push_back(p.get());
            active_.push_back(std::move(p));
        }
        for (auto* p : P) {
            if (p->n < 2 || p->task.com->log_rate != 1 || p->task.point.size() != 2 * (size_t)p->n ||
                tab_->num_rounds < p->n || tab_->num_vars < p->n) {
                set_error_msg("open engine: invalid opening (n >= 2, log_rate 1, 2n point words, table covering n)");
                return GB_EINVAL;
            }
            GB_CUDA_TRY(cudaMallocAsync(&p->ws, ls_poly_words(p->n, 1) * 8, s));
            carve(*p);
        }
        LS_RC(reserve(active_.size(), max_vars(), partial_need()));
        const int np = (int)P.size();
        ls_parallel(P.size(), [&](size_t k) {
            EngPoly& p = *P[k];
            for (int w = 0; w < 4; w++) tr_append_u64(&p.t, "", p.com->root[w]);
            for (int i = 0; i < p.n; i++) tr_append_ext2(&p.t, "", E2{canon(p.point[2 * i]), canon(p.point[2 * i + 1])});
        });
        // every joining point in one copy, then every eq table in two launches
        std::vector<EqSeg> eqsegs(np);
        size_t scratch = 0;
        for (auto* p : P) scratch += 2 * (((size_t)1 << (p->n / 2)) + ((size_t)1 << (p->n - p->n / 2)));
        std::vector<u64> pts;
        for (auto* p : P)
            for (int i = 0; i < 2 * p->n; i++) pts.push_back(canon(p->point[i]));
        u64 *eqs = nullptr, *d_pts = nullptr;
        EqSeg* d_eqsegs = nullptr;
        GB_CUDA_TRY(cudaMallocAsync(&d_pts, pts.size() * 8, s));
        GB_CUDA_TRY(cudaMemcpyAsync(d_pts, pts.data(), pts.size() * 8, cudaMemcpyHostToDevice, s));
        GB_CUDA_TRY(cudaMallocAsync(&eqs, scratch * 8, s));
        GB_CUDA_TRY(cudaMallocAsync(&d_eqsegs, (size_t)np * sizeof(EqSeg), s));
        {
            u64 nb = 0;
            u64* cur = eqs;
            size_t po = 0;
            for (int k = 0; k < np; k++) {
                EngPoly& p = *P[k];
                EqSeg& g = eqsegs[k];
                g.r = d_pts + po;
                po += 2 * (size_t)p.n;
                g.n = (u64)p.n;
                g.k = (u64)(p.n / 2);
                g.lo = cur;
                cur += 2 * ((size_t)1 << g.k);
                g.hi = cur;
                cur += 2 * ((size_t)1 << (g.n - g.k));
                g.out = p.eq;
                g.block0 = nb;
                nb += ((u64)1 << p.n) / 256 + 1;
            }
            GB_CUDA_TRY(cudaMemcpyAsync(d_eqsegs, eqsegs.data(), (size_t)np * sizeof(EqSeg), cudaMemcpyHostToDevice, s));
            ls_eq_halves_kernel<<<(unsigned)(2 * np), 256, 0, s>>>(d_eqsegs, np);
            GB_LAUNCH_CHECK("ls_eq_halves_kernel");
            ls_eq_expand_kernel<<<(unsigned)nb, 256, 0, s>>>(d_eqsegs, np);
            GB_LAUNCH_CHECK("ls_eq_expand_kernel");
        }
        // round-0 oracles
        {
            LsSeg* hs = segs(np);
            if (!hs) return GB_EINVAL;
            u64 nb = 0;
            for (int k = 0; k < np; k++) {
                EngPoly& p = *P[k];
                hs[k] = LsSeg{p.com->d_evals, p.eq, nullptr, nullptr, 0, 0, p.N / 2, nb};
                nb += blocks_red(p.N / 2);
            }
            const LsSeg* ds = upload(hs, np);
            if (!ds) return GB_ECUDA;
            ls_round0_kernel<<<(unsigned)nb, LS_RED_THREADS, 0, s>>>(ds, np, d_partials_);
            GB_LAUNCH_CHECK("ls_round0_kernel");
            ls_reduce_kernel<<<(unsigned)((np * 32 + 255) / 256), 256, 0, s>>>(ds, np, d_partials_, d_recs_);
            GB_LAUNCH_CHECK("ls_reduce_kernel");
        }
        cudaFreeAsync(eqs, s);
        cudaFreeAsync(d_eqsegs, s);
        cudaFreeAsync(d_pts, s);
        LS_RC(sync());
        ls_parallel(P.size(), [&](size_t k) {
            EngPoly& p = *P[k];
            const u64* rec = h_recs_ + k * LS_REC;
            E2 ev = e2add(E2{rec[0], rec[1]}, put_oracle(p, 0, rec));
            p.proof[0] = ev.c0;
            p.proof[1] = ev.c1;
            p.eq_cur = p.eq;
            p.bh_cur = p.com->d_evals;
            p.pp = 0;
            p.sc = p.N;
            p.rd = 0;
        });
        return GB_OK;
    }

    // one round of every opening in flight
    int step() {
        using namespace host;
        cudaStream_t s = stream();
        LS_RC(reserve(active_.size(), max_vars(), partial_need()));
        const size_t na = active_.size();
        std::vector<E2> ch(na);
        ls_parallel(na, [&](size_t k) { ch[k] = tr_challenge_ext2(&active_[k]->t, ""); });
        // `mid`: openings with a tree this round, round-0 ones first (they read base-field
        // inputs); `last`: the final fold.  Every opening has n >= 2.
        std::vector<size_t> mid, last;
        for (size_t k = 0; k < na; k++)
            if (active_[k]->rd == 0) mid.push_back(k);
        const size_t mid0 = mid.size();
        for (size_t k = 0; k < na; k++) {
            const EngPoly& p = *active_[k];
            if (p.rd >= 1 && p.rd < p.n - 1) mid.push_back(k);
            else if (p.rd >= 1 && p.rd == p.n - 1) last.push_back(k);
        }
        if (!mid.empty()) {
            // eq/bh folds + next oracles: record m of `mid` in mid order
            u64 part_off = 0;
            for (int g = 0; g < 2; g++) {
                const size_t b = g ? mid0 : 0, e = g ? mid.size() : mid0;
                if (b == e) continue;
                LsSeg* hs = segs(e - b);
                if (!hs) return GB_EINVAL;
                u64 nb = 0;
                for (size_t m = b; m < e; m++) {
                    EngPoly& p = *active_[mid[m]];
                    const size_t quarter = p.sc / 4;
                    hs[m - b] = LsSeg{p.eq_cur, p.bh_cur, p.bufs_eq[p.pp], p.bufs_bh[p.pp], ch[mid[m]].c0,
                                      ch[mid[m]].c1, quarter, nb};
                    nb += blocks_red(quarter);
                }
                const LsSeg* ds = upload(hs, e - b);
                if (!ds) return GB_ECUDA;
                u64* part = d_partials_ + part_off * 6;
                if (g == 0) ls_open_round_kernel<true><<<(unsigned)nb, LS_RED_THREADS, 0, s>>>(ds, (int)(e - b), part);
                else ls_open_round_kernel<false><<<(unsigned)nb, LS_RED_THREADS, 0, s>>>(ds, (int)(e - b), part);
                GB_LAUNCH_CHECK("ls_open_round_kernel");
                ls_reduce_kernel<<<(unsigned)(((e - b) * 32 + 255) / 256), 256, 0, s>>>(ds, (int)(e - b), part,
                                                                                        d_recs_ + b * LS_REC);
                GB_LAUNCH_CHECK("ls_reduce_kernel");
                part_off += nb;
            }
            for (size_t k : mid) {
                EngPoly& p = *active_[k];
                p.eq_cur = p.bufs_eq[p.pp];
                p.bh_cur = p.bufs_bh[p.pp];
                p.pp ^= 1;
                p.sc /= 2;
            }
            // codeword folds + leaf hashes
            for (int g = 0; g < 2; g++) {
                const size_t b = g ? mid0 : 0, e = g ? mid.size() : mid0;
                if (b == e) continue;
                LsSeg* hs = segs(e - b);
                if (!hs) return GB_EINVAL;
                for (size_t m = b; m < e; m++) {
                    EngPoly& p = *active_[mid[m]];
                    const int rd = p.rd;
                    const size_t leaves = (p.L >> (rd + 1)) / 2;
                    const u64* cw_in = rd == 0 ? p.com->d_codeword : p.fcw[rd - 1];
                    hs[m - b] = LsSeg{cw_in, tab_->d_entries + 2 * tab_->level_offsets[rd], p.fcw[rd], p.ftree[rd],
                                      ch[mid[m]].c0, ch[mid[m]].c1, leaves, 0};
                }
                u64 nb = 0;
                const int cnt = (int)(e - b);
                const int th = ls_p2_assign(hs, cnt, nb);
                const LsSeg* ds = upload(hs, e - b);
                if (!ds) return GB_ECUDA;
                if (th == P2_WIDE) {
                    if (g == 0) ls_fold_hash_kernel<true, P2_WIDE><<<(unsigned)nb, th, 0, s>>>(ds, cnt);
                    else ls_fold_hash_kernel<false, P2_WIDE><<<(unsigned)nb, th, 0, s>>>(ds, cnt);
                } else {
                    if (g == 0) ls_fold_hash_kernel<true, P2_NARROW><<<(unsigned)nb, th, 0, s>>>(ds, cnt);
                    else ls_fold_hash_kernel<false, P2_NARROW><<<(unsigned)nb, th, 0, s>>>(ds, cnt);
                }
                GB_LAUNCH_CHECK("ls_fold_hash_kernel");
            }
            // Merkle layers of every tree, one launch per layer
            for (int lvl = 0;; lvl++) {
                LsSeg* hs = segs(mid.size());
                if (!hs) return GB_EINVAL;
                int cnt = 0;
                for (size_t k : mid) {
                    EngPoly& p = *active_[k];
                    const size_t leaves = (p.L >> (p.rd + 1)) / 2;
                    const size_t nodes = leaves >> lvl;
                    if (nodes < 2) continue;
                    size_t off = 0;
                    for (int l = 0; l < lvl; l++) off += leaves >> l;
                    u64* layer = p.ftree[p.rd] + 4 * off;
                    hs[cnt++] = LsSeg{layer, nullptr, layer + 4 * nodes, nullptr, 0, 0, nodes / 2, 0};
                }
                if (!cnt) {
                    seg_used_ -= mid.size();
                    break;
                }
                u64 nb = 0;
                const LsLayerForm form = ls_layer_assign(hs, cnt, coop_, nb);
                const LsSeg* ds = upload(hs, cnt);
                if (!ds) return GB_ECUDA;
                LS_RC(ls_layer_launch(form, nb, ds, cnt, s));
            }
            // roots into records m of `mid`
            LsSeg* hs = segs(mid.size());
            if (!hs) return GB_EINVAL;
            for (size_t m = 0; m < mid.size(); m++) {
                EngPoly& p = *active_[mid[m]];
                const size_t leaves = (p.L >> (p.rd + 1)) / 2;
                hs[m] = LsSeg{p.ftree[p.rd] + 4 * (2 * leaves - 2), nullptr, nullptr, nullptr, 0, 0, 0, 0};
            }
            const LsSeg* ds = upload(hs, mid.size());
            if (!ds) return GB_ECUDA;
            ls_root_kernel<<<(unsigned)((mid.size() + 127) / 128), 128, 0, s>>>(ds, (int)mid.size(), d_recs_);
            GB_LAUNCH_CHECK("ls_root_kernel");
        }
        if (!last.empty()) {
            // final folds into records |mid| + m
            LsSeg* hs = segs(last.size());
            if (!hs) return GB_EINVAL;
            for (size_t m = 0; m < last.size(); m++) {
                EngPoly& p = *active_[last[m]];
                const int rd = p.rd;
                hs[m] = LsSeg{p.fcw[rd - 1], tab_->d_entries + 2 * tab_->level_offsets[rd], p.fcw[rd], nullptr,
                              ch[last[m]].c0, ch[last[m]].c1, p.L >> (rd + 1), 0};
            }
            const LsSeg* ds = upload(hs, last.size());
            if (!ds) return GB_ECUDA;
            ls_fold_final_kernel<<<(unsigned)last.size(), 32, 0, s>>>(ds, (int)last.size(), d_recs_ + mid.size() * LS_REC);
            GB_LAUNCH_CHECK("ls_fold_final_kernel");
        }
        LS_RC(sync());
        ls_parallel(mid.size(), [&](size_t m) {
            EngPoly& p = *active_[mid[m]];
            const u64* rec = h_recs_ + m * LS_REC;
            put_oracle(p, p.rd + 1, rec);
            u64* root = p.proof + 2 + (size_t)p.n * 6 + (size_t)p.rd * 4;
            for (int k = 0; k < 4; k++) {
                root[k] = rec[8 + k];
                tr_append_u64(&p.t, "", root[k]);
            }
        });
        for (size_t m = 0; m < last.size(); m++) {
            EngPoly& p = *active_[last[m]];
            u64* fin = p.proof + 2 + (size_t)p.n * 6 + (size_t)(p.n - 1) * 4;
            for (int k = 0; k < 4; k++) fin[k] = h_recs_[(mid.size() + m) * LS_REC + 12 + k];
        }
        for (auto& p : active_) p->rd++;
        return GB_OK;
    }

    // queries of the openings that finished their rounds, then their callbacks
    int finish() {
        using namespace host;
        cudaStream_t s = stream();
        PolyList D;
        for (auto& p : active_)
            if (p->rd >= p->n) D.push_back(p.get());
        if (D.empty()) return GB_OK;
        const int np = (int)D.size(), lr = 1;
        if (q_ > 0) {
            std::vector<QueryJob> jobs(np);
            std::vector<u64> idx((size_t)np * q_), per_q(np);
            std::vector<const u64*> ptrs;
            std::vector<size_t> out_off(np), ptr_off(np);
            size_t out_words = 0;
            ls_parallel(D.size(), [&](size_t k) {
                EngPoly& p = *D[k];
                for (int j = 0; j < q_; j++) idx[k * q_ + j] = tr_challenge(&p.t, "") % (u64)(p.L / 2);
            });
            for (int k = 0; k < np; k++) {
                EngPoly& p = *D[k];
                size_t pw = 0;
                for (int r = 0; r < p.n; r++) pw += (size_t)(p.n + lr - 1 - r);
                per_q[k] = 1 + (size_t)p.n * 4 + pw * 4;
                out_off[k] = out_words;
                out_words += per_q[k] * q_;
                ptr_off[k] = ptrs.size();
                for (int r = 0; r + 1 < p.n; r++) ptrs.push_back(p.fcw[r]);
                for (int r = 0; r + 1 < p.n; r++) ptrs.push_back(p.ftree[r]);
            }
            u64 *d_idx = nullptr, *d_perq = nullptr, *d_out = nullptr;
            const u64** d_ptrs = nullptr;
            QueryJob* d_jobs = nullptr;
            u64** d_outs = nullptr;
            GB_CUDA_TRY(cudaMallocAsync(&d_idx, idx.size() * 8, s));
            GB_CUDA_TRY(cudaMallocAsync(&d_perq, per_q.size() * 8, s));
            GB_CUDA_TRY(cudaMallocAsync(&d_out, std::max<size_t>(out_words, 1) * 8, s));
            GB_CUDA_TRY(cudaMallocAsync(&d_ptrs, std::max<size_t>(ptrs.size(), 1) * sizeof(u64*), s));
            GB_CUDA_TRY(cudaMallocAsync(&d_jobs, (size_t)np * sizeof(QueryJob), s));
            GB_CUDA_TRY(cudaMallocAsync(&d_outs, (size_t)np * sizeof(u64*), s));
            std::vector<u64*> outs(np);
            for (int k = 0; k < np; k++) {
                EngPoly& p = *D[k];
                const u64* const* base = d_ptrs + ptr_off[k];
                jobs[k] = QueryJob{p.com->d_codeword, p.com->d_tree, base, base + (p.n - 1), p.n, lr, false};
                outs[k] = d_out + out_off[k];
            }
            GB_CUDA_TRY(cudaMemcpyAsync(d_idx, idx.data(), idx.size() * 8, cudaMemcpyHostToDevice, s));
            GB_CUDA_TRY(cudaMemcpyAsync(d_perq, per_q.data(), per_q.size() * 8, cudaMemcpyHostToDevice, s));
            if (!ptrs.empty())
                GB_CUDA_TRY(cudaMemcpyAsync(d_ptrs, ptrs.data(), ptrs.size() * sizeof(u64*), cudaMemcpyHostToDevice, s));
            GB_CUDA_TRY(cudaMemcpyAsync(d_jobs, jobs.data(), jobs.size() * sizeof(QueryJob), cudaMemcpyHostToDevice, s));
            GB_CUDA_TRY(cudaMemcpyAsync(d_outs, outs.data(), outs.size() * sizeof(u64*), cudaMemcpyHostToDevice, s));
            ls_query_kernel<<<dim3((unsigned)q_, (unsigned)np), 128, 0, s>>>(d_jobs, d_idx, q_, d_outs, d_perq);
            GB_LAUNCH_CHECK("ls_query_kernel");
            std::vector<u64> host_out(out_words);
            GB_CUDA_TRY(cudaMemcpyAsync(host_out.data(), d_out, out_words * 8, cudaMemcpyDeviceToHost, s));
            for (void* x : {(void*)d_idx, (void*)d_perq, (void*)d_out, (void*)d_ptrs, (void*)d_jobs, (void*)d_outs})
                cudaFreeAsync(x, s);
            LS_RC(sync());
            for (int k = 0; k < np; k++) {
                EngPoly& p = *D[k];
                u64* dst = p.proof + 2 + (size_t)p.n * 6 + (size_t)(p.n - 1) * 4 + ((size_t)2 << lr);
                std::memcpy(dst, host_out.data() + out_off[k], per_q[k] * q_ * 8);
            }
        }
        for (auto* p : D) {
            cudaFreeAsync(p->ws, s);
            p->ws = nullptr;
        }
        LS_RC(sync());
        // the finished polynomials leave the set, then their callbacks run (a callback may
        // complete the job, and whoever waits on it may count the openings in flight at once)
        std::vector<std::unique_ptr<EngPoly>> keep, gone;
        for (auto& p : active_) (p->rd >= p->n ? gone : keep).push_back(std::move(p));
        active_.swap(keep);
        for (auto& p : gone) {
            {
                std::lock_guard<std::mutex> l(mu_);
                waiting_--;
            }
            if (p->task.done) p->task.done(GB_OK, std::string());
        }
        return GB_OK;
    }

    // a failed step: every opening in flight ends with the error
    void fail_all(int rc, const std::string& err) {
        cudaStream_t s = stream();
        cudaStreamSynchronize(s);
        std::vector<std::unique_ptr<EngPoly>> gone;
        gone.swap(active_);
        for (auto& p : gone) {
            if (p->ws) cudaFreeAsync(p->ws, s);
            {
                std::lock_guard<std::mutex> l(mu_);
                waiting_--;
            }
            if (p->task.done) p->task.done(rc, err);
        }
        cudaStreamSynchronize(s);
        seg_used_ = 0;
    }

    const BfTable* tab_;
    int q_, device_;
    size_t coop_;  // the creating thread's cooperative threshold, for the Merkle layers
    std::thread th_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::vector<OpenTask> intake_;
    std::vector<std::unique_ptr<EngPoly>> active_;  // engine thread only
    size_t waiting_ = 0;
    bool stop_ = false, started_ = false;
    int start_rc_ = GB_OK;
    LsSeg* d_segs_ = nullptr;
    LsSeg* h_segs_ = nullptr;
    u64* d_recs_ = nullptr;
    u64* h_recs_ = nullptr;
    u64* d_partials_ = nullptr;
    size_t seg_cap_ = 0, rec_cap_ = 0, part_cap_ = 0, seg_used_ = 0;
};

OpenEngine* open_engine_create(const BfTable* tab, int q, int device, int* rc) {
    if (!tab || q < 0 || tab->log_rate != 1) {
        set_error_msg("open engine: invalid table (log_rate must be 1) or query count");
        if (rc) *rc = GB_EINVAL;
        return nullptr;
    }
    auto* e = new OpenEngine(tab, q, device);
    if (e->start_rc()) {
        if (rc) *rc = e->start_rc();
        set_error_msg("open engine: could not set the device or create its stream");
        delete e;
        return nullptr;
    }
    if (rc) *rc = GB_OK;
    return e;
}
void open_engine_submit(OpenEngine* e, OpenTask&& task) { e->submit(std::move(task)); }
size_t open_engine_in_flight(OpenEngine* e) { return e->in_flight(); }
void open_engine_destroy(OpenEngine* e) { delete e; }

}  // namespace gb

using namespace gb;

extern "C" {

int gb_batch_prove_lockstep(void* table, const uint64_t master_seed[2], int num_queries, const gb_instance* insts,
                            int count, int workers, size_t hbm_budget) {
    return lockstep_prove(table, master_seed, num_queries, insts, count, workers, hbm_budget);
}

int gb_set_lockstep_schedule(int groups, int open_parts) {
    if (groups < 1 || groups > 8 || open_parts < 1 || open_parts > 8) {
        set_error_msg("gb_set_lockstep_schedule: groups and open_parts must lie in [1, 8]");
        return GB_EINVAL;
    }
    t_ls_groups = groups;
    t_ls_open_parts = open_parts;
    return GB_OK;
}

void gb_get_lockstep_schedule(int* groups, int* open_parts) {
    if (groups) *groups = t_ls_groups;
    if (open_parts) *open_parts = t_ls_open_parts;
}

void gb_lockstep_last_timing(double* commit_sumcheck_ms, double* open_ms, double* sumcheck_ms) {
    if (commit_sumcheck_ms) *commit_sumcheck_ms = t_ls_ms[0];
    if (open_ms) *open_ms = t_ls_ms[1];
    if (sumcheck_ms) *sumcheck_ms = t_ls_ms[2];
}

}  // extern "C"
