// Per-item device math of the Basefold open, shared by the per-call kernels (basefold.cu)
// and the round-synchronous batch engine (lockstep.cu).
#pragma once
#include "gl.cuh"

namespace gb {

// ===========================================================================
// 2x2 per-variable transforms applied to K consecutive bits [b, b+K) in registers
// MAT 0: T = (e1, 2 e0 - e1)   1: Moebius (e0, e1 - e0)   2: WHT (e0 + e1, e0 - e1)
// ===========================================================================
template <int MAT>
__device__ __forceinline__ void bf_butterfly(u64& x0, u64& x1) {
    if (MAT == 0) {
        u64 t = gl_sub(gl_double(x0), x1);
        x0 = x1;
        x1 = t;
    } else if (MAT == 1) {
        x1 = gl_sub(x1, x0);
    } else {
        u64 a = gl_add(x0, x1), b = gl_sub(x0, x1);
        x0 = a;
        x1 = b;
    }
}

// group g of a radix-2^K pass over bits [b, b+K): the 2^K elements base + (j << b); in may equal out
template <int MAT, int K>
__device__ __forceinline__ void bf_transform_group(const u64* __restrict__ in, u64* __restrict__ out, int b, size_t g) {
    size_t low = g & (((size_t)1 << b) - 1), high = g >> b;
    size_t base = (high << (b + K)) | low;
    u64 v[1 << K];
#pragma unroll
    for (int j = 0; j < (1 << K); j++) v[j] = in[base + ((size_t)j << b)];
#pragma unroll
    for (int l = 0; l < K; l++) {
#pragma unroll
        for (int j = 0; j < (1 << K); j++) {
            if (!(j & (1 << l))) bf_butterfly<MAT>(v[j], v[j | (1 << l)]);
        }
    }
#pragma unroll
    for (int j = 0; j < (1 << K); j++) out[base + ((size_t)j << b)] = v[j];
}

__device__ __forceinline__ size_t bitrev_dev(size_t x, int bits) { return bits ? (__brevll(x) >> (64 - bits)) : 0; }

// val0 + (ch - x0) (val1 - val0) w     (basefold.cuh:397-419, :522-548, :739-761)
// MODE 0: base cw + base ch; 1: base cw + Ext2 ch (mixed); 2: Ext2 cw + Ext2 ch
template <int MODE>
__device__ __forceinline__ void fold_pair(const u64* cw, size_t i, u64 x0, u64 w, u64 c0, u64 c1, u64* o) {
    if (MODE == 0) {
        u64 v0 = cw[2 * i], v1 = cw[2 * i + 1];
        o[0] = gl_add(v0, gl_mul(gl_mul(gl_sub(c0, x0), gl_sub(v1, v0)), w));
    } else if (MODE == 1) {
        u64 v0 = cw[2 * i], v1 = cw[2 * i + 1];
        u64 dw = gl_mul(gl_sub(v1, v0), w);
        o[0] = gl_add(v0, gl_mul(gl_sub(c0, x0), dw));
        o[1] = gl_mul(c1, dw);
    } else {
        e2 v0 = e2_make(cw[4 * i], cw[4 * i + 1]), v1 = e2_make(cw[4 * i + 2], cw[4 * i + 3]);
        e2 dw = e2_mul_base(e2_sub(v1, v0), w);
        e2 r = e2_add(v0, e2_mul(e2_make(gl_sub(c0, x0), c1), dw));
        o[0] = r.c0;
        o[1] = r.c1;
    }
}

// Round 0 oracle terms of pair i over (bh base, eq Ext2): (eq_e bh_e, eq_o bh_o, (eq_o - eq_e)(bh_o - bh_e))
__device__ __forceinline__ void open_round0_item(const u64* __restrict__ bh, const u64* __restrict__ eq, size_t i,
                                                 u64 (&acc)[6]) {
    ulonglong2 b2 = __ldg(reinterpret_cast<const ulonglong2*>(bh) + i);
    e2 ee = e2_ld(eq + 4 * i), eo = e2_ld(eq + 4 * i + 2);
    u64 bd = gl_sub(b2.y, b2.x);
    e2 ed = e2_sub(eo, ee);
    e2 t0 = e2_mul_base(ee, b2.x), t1 = e2_mul_base(eo, b2.y), t2 = e2_mul_base(ed, bd);
    acc[0] = gl_add(acc[0], t0.c0);
    acc[1] = gl_add(acc[1], t0.c1);
    acc[2] = gl_add(acc[2], t1.c0);
    acc[3] = gl_add(acc[3], t1.c1);
    acc[4] = gl_add(acc[4], t2.c0);
    acc[5] = gl_add(acc[5], t2.c1);
}

// Same over Ext2 evaluations (the combined evaluations of a batch opening)
__device__ __forceinline__ void open_round0_e2_item(const u64* __restrict__ bh, const u64* __restrict__ eq, size_t i,
                                                    u64 (&acc)[6]) {
    e2 be = e2_ld(bh + 4 * i), bo = e2_ld(bh + 4 * i + 2);
    e2 ee = e2_ld(eq + 4 * i), eo = e2_ld(eq + 4 * i + 2);
    e2 t0 = e2_mul(ee, be), t1 = e2_mul(eo, bo), t2 = e2_mul(e2_sub(eo, ee), e2_sub(bo, be));
    acc[0] = gl_add(acc[0], t0.c0);
    acc[1] = gl_add(acc[1], t0.c1);
    acc[2] = gl_add(acc[2], t1.c0);
    acc[3] = gl_add(acc[3], t1.c1);
    acc[4] = gl_add(acc[4], t2.c0);
    acc[5] = gl_add(acc[5], t2.c1);
}

// Open round r >= 1, output pair y: fold eq (Ext2) and bh (base when BH_BASE) with ch, store
// the folded pair of each, add the new pair's oracle terms.
template <bool BH_BASE>
__device__ __forceinline__ void open_round_item(const u64* __restrict__ eq_in, const u64* __restrict__ bh_in,
                                                u64* __restrict__ eq_out, u64* __restrict__ bh_out, size_t y, e2 ch,
                                                u64 (&acc)[6]) {
    const u64* q = eq_in + 8 * y;
    e2 x0 = e2_ld(q), x1 = e2_ld(q + 2), x2 = e2_ld(q + 4), x3 = e2_ld(q + 6);
    e2 ea = e2_add(x0, e2_mul(ch, e2_sub(x1, x0)));
    e2 eb = e2_add(x2, e2_mul(ch, e2_sub(x3, x2)));
    e2 ba, bb;
    if (BH_BASE) {
        ulonglong2 p = __ldg(reinterpret_cast<const ulonglong2*>(bh_in + 4 * y));
        ulonglong2 r = __ldg(reinterpret_cast<const ulonglong2*>(bh_in + 4 * y + 2));
        u64 d0 = gl_sub(p.y, p.x), d1 = gl_sub(r.y, r.x);
        ba = e2_make(gl_add(p.x, gl_mul(ch.c0, d0)), gl_mul(ch.c1, d0));
        bb = e2_make(gl_add(r.x, gl_mul(ch.c0, d1)), gl_mul(ch.c1, d1));
    } else {
        const u64* h = bh_in + 8 * y;
        e2 h0 = e2_ld(h), h1 = e2_ld(h + 2), h2 = e2_ld(h + 4), h3 = e2_ld(h + 6);
        ba = e2_add(h0, e2_mul(ch, e2_sub(h1, h0)));
        bb = e2_add(h2, e2_mul(ch, e2_sub(h3, h2)));
    }
    e2_st(eq_out + 4 * y, ea);
    e2_st(eq_out + 4 * y + 2, eb);
    e2_st(bh_out + 4 * y, ba);
    e2_st(bh_out + 4 * y + 2, bb);
    e2 t0 = e2_mul(ea, ba), t1 = e2_mul(eb, bb), t2 = e2_mul(e2_sub(eb, ea), e2_sub(bb, ba));
    acc[0] = gl_add(acc[0], t0.c0);
    acc[1] = gl_add(acc[1], t0.c1);
    acc[2] = gl_add(acc[2], t1.c0);
    acc[3] = gl_add(acc[3], t1.c1);
    acc[4] = gl_add(acc[4], t2.c0);
    acc[5] = gl_add(acc[5], t2.c1);
}

// The two folded values f0, f1 that make up leaf i of a round's folded codeword:
// f[k] = fold(cw[2k], cw[2k+1], table[k]), k = 2i, 2i + 1.  BASE_IN: the committed base codeword.
template <bool BASE_IN>
__device__ __forceinline__ void fold_leaf_item(const u64* __restrict__ cw, const u64* __restrict__ tab, size_t i, u64 c0,
                                               u64 c1, e2& f0, e2& f1) {
    ulonglong2 t0 = __ldg(reinterpret_cast<const ulonglong2*>(tab) + 2 * i);
    ulonglong2 t1 = __ldg(reinterpret_cast<const ulonglong2*>(tab) + 2 * i + 1);
    if (BASE_IN) {
        ulonglong2 v = __ldg(reinterpret_cast<const ulonglong2*>(cw) + 2 * i);
        ulonglong2 u = __ldg(reinterpret_cast<const ulonglong2*>(cw) + 2 * i + 1);
        u64 dw0 = gl_mul(gl_sub(v.y, v.x), t0.y), dw1 = gl_mul(gl_sub(u.y, u.x), t1.y);
        f0 = e2_make(gl_add(v.x, gl_mul(gl_sub(c0, t0.x), dw0)), gl_mul(c1, dw0));
        f1 = e2_make(gl_add(u.x, gl_mul(gl_sub(c0, t1.x), dw1)), gl_mul(c1, dw1));
    } else {
        const u64* p = cw + 8 * i;
        e2 a0 = e2_ld(p), a1 = e2_ld(p + 2), b0 = e2_ld(p + 4), b1 = e2_ld(p + 6);
        e2 dw0 = e2_mul_base(e2_sub(a1, a0), t0.y), dw1 = e2_mul_base(e2_sub(b1, b0), t1.y);
        f0 = e2_add(a0, e2_mul(e2_make(gl_sub(c0, t0.x), c1), dw0));
        f1 = e2_add(b0, e2_mul(e2_make(gl_sub(c0, t1.x), c1), dw1));
    }
}

// Query gather.  For query q with leaf index L (computed on the host from the transcript):
// index, values of every round (initial pair lifted to Ext2, then the folded pairs) and all
// authentication paths, written canonical into the flat proof layout.
struct QueryJob {
    const u64* cw0;           // round-0 codeword: base, or Ext2 when cw0_ext2
    const u64* tree0;         // its tree
    const u64* const* fcw;    // folded codewords r = 0..n-2 (device array of pointers)
    const u64* const* ftree;  // their trees
    int n, lr;
    bool cw0_ext2;
};

// One query, gathered by the calling block into o (per_query words).
__device__ __forceinline__ void query_gather_block(const QueryJob& job, size_t leaf, u64* __restrict__ o) {
    const int n = job.n, lr = job.lr;
    u64* vals = o + 1;
    u64* paths = vals + (size_t)n * 4;
    if (threadIdx.x == 0) {
        o[0] = leaf;
        if (job.cw0_ext2) {
            for (int k = 0; k < 4; k++) vals[k] = gl_canon(job.cw0[4 * leaf + k]);
        } else {
            vals[0] = gl_canon(job.cw0[2 * leaf]);
            vals[1] = 0;
            vals[2] = gl_canon(job.cw0[2 * leaf + 1]);
            vals[3] = 0;
        }
    }
    for (int r = threadIdx.x; r + 1 < n; r += blockDim.x) {
        size_t pi = leaf >> (r + 1);
        const u64* f = job.fcw[r] + 4 * pi;
        u64* v = vals + 4 * (r + 1);
        for (int k = 0; k < 4; k++) v[k] = gl_canon(f[k]);
    }
    // path words: tree 0 has depth n+lr-1, tree r+1 (folded r) depth n+lr-2-r
    size_t total_depth = 0;
    for (int r = 0; r < n; r++) total_depth += (size_t)(n + lr - 1 - r);
    for (size_t node = threadIdx.x; node < total_depth; node += blockDim.x) {
        // locate (tree t, level l) of this path node
        size_t rem = node;
        int t = 0;
        size_t depth = (size_t)(n + lr - 1);
        while (rem >= depth) {
            rem -= depth;
            t++;
            depth--;
        }
        int level = (int)rem;
        size_t leaves = (size_t)1 << (n + lr - 1 - t);
        const u64* tree = t == 0 ? job.tree0 : job.ftree[t - 1];
        size_t li = (t == 0 ? leaf : (leaf >> t)) >> level;
        size_t off = 0, sz = leaves;
        for (int l = 0; l < level; l++) {
            off += sz;
            sz >>= 1;
        }
        const u64* dg = tree + 4 * (off + (li ^ 1));
        u64* dst = paths + 4 * node;
        for (int k = 0; k < 4; k++) dst[k] = gl_canon(dg[k]);
    }
}

}  // namespace gb
