// Poseidon2 over Goldilocks, width 8, S-box x^7, 4 external + 22 internal +
// 4 external rounds: one register-resident permutation per thread.
//
// Structure and constants follow the reference's three copies of this
// permutation (cuda/poseidon2.cuh:322-362, goldilocks-cuda-rs/src/cpu_poseidon2.rs:117-140,
// zk-torch-3/src/transcript.rs:60-172): no initial linear layer, the external
// layer is the circulant [2 3 1 1] per half plus the column sums of both halves,
// the internal layer is diag(v) + 1.  The constants live in function-local
// constexpr tables so that every fully unrolled use becomes an immediate.
#pragma once
#include "gl.cuh"

namespace gb {

// The tables are written once, as macros, and expanded into a host table (P2Const)
// and into device function-local tables that fold to immediates when unrolled.
#define GB_P2_RC_EXT \
    { \
    {0xdd5743e7f2a5a5d9ull, 0xcb3a864e58ada44bull, 0xd5a3726889dedc0dull, 0x79365a7f967583c1ull, \
    0xb7820c177b0a3c30ull, 0x68a60479943b7240ull, 0x0a22eeab67b97c41ull, 0xbee9d90e037fa7d4ull}, \
    {0xf1dda5b9259dfcb4ull, 0x27515210be112d59ull, 0x654a4db8f15f6c3aull, 0x5a9bfff8c29db0c4ull, \
    0xb72f2628c95a885bull, 0xffcb54fc166beaddull, 0xe32f91d59c463772ull, 0x9e0ff2a9bbea79dbull}, \
    {0xce57d6245ddca6b2ull, 0xb1fc8d402bba1eb1ull, 0x64df974fb666d528ull, 0x59e4e5b237e52e78ull, \
    0x5e255e2742caa8fcull, 0xc4a17304e330ef9aull, 0x60e3a513cdd9f0b1ull, 0xbf29a6a5a0c9c8baull}, \
    {0xcea721cce82fb11bull, 0xe5b55eb8098ece81ull, 0x4ec66bfb89f7c380ull, 0xc33be12b6ef7e4faull, \
    0xa41b5f5b84c57d7dull, 0xb526206b2138a936ull, 0x9f7a5ac62f16eb4eull, 0x7de77f405f683aa5ull}, \
    {0x014ef1197d341346ull, 0x9725e20825d07394ull, 0xc8ff2a22516f3604ull, 0xde1b51f7cf493493ull, \
    0xa7e3af1a53eadb78ull, 0x9b7b7ee0ddf9f229ull, 0xf0a460f2dc649e7dull, 0xdc4448d02c2cb823ull}, \
    {0xaa62c88e0b294011ull, 0x058eb9d810ce9f74ull, 0x4e3d7a5403566d24ull, 0xe8ae66da2f8b7a63ull, \
    0x3fdad3b08dae2e0bull, 0xec81e61303dd409bull, 0x3cbaa1cd35d31fc4ull, 0x847f7806eec88ffaull}, \
    {0x98ae09a325893803ull, 0xf8a6475077968838ull, 0xdf55b7419443de5bull, 0xdbe15699e696ca70ull, \
    0x8e54a27d8db00424ull, 0x7679a45cd9d1e12aull, 0x2844f52be73e0e2full, 0xd41f8eb31ada34f8ull}, \
    {0xe9dd318bae1f3961ull, 0xf7462137299efe1aull, 0x6dbbe06779e1d573ull, 0xfe35b05cbe707632ull, \
    0x5d8896b12654fd8cull, 0x6f96ef47c32d4ae2ull, 0xb0caa221dbbfc0daull, 0x0bc2a5bf1f238d3full}, \
    }
#define GB_P2_RC_INT \
    { \
    0x488897d85ff51f56ull, 0x1140737ccb162218ull, 0xa7eeb9215866ed35ull, 0x9bd2976fee49fcc9ull, \
    0xc0c8f0de580a3fccull, 0x4fb2dae6ee8fc793ull, 0x343a89f35f37395bull, 0x223b525a77ca72c8ull, \
    0x56ccb62574aaa918ull, 0xc4d507d8027af9edull, 0xa080673cf0b7e95cull, 0xf0184884eb70dcf8ull, \
    0x044f10b0cb3d5c69ull, 0xe9e3f7993938f186ull, 0x1b761c80e772f459ull, 0x606cec607a1b5facull, \
    0x14a0c2e1d45f03cdull, 0x4eace8855398574full, 0xf905ca7103eff3e6ull, 0xf8c8f8d20862c059ull, \
    0xb524fe8bdd678e5aull, 0xfbb7865901a1ec41ull, \
    }
#define GB_P2_DIAG \
    { \
    0xa98811a1fed4e3a5ull, 0x1cc48b54f377e2a0ull, 0xe40cd4f6c5609a26ull, 0x11de79ebca97a4a3ull, \
    0x9177c73d8b7e929cull, 0x2a6fe8085797e791ull, 0x3de6e93329f8d5adull, 0x3f7af9125da962feull, \
    }

// sbox(rc_ext[0][i]) = rc_ext[0][i]^7 mod p: the first round of a lane whose input is zero (leaf
// hashes pad the state with zeros), precomputed
#define GB_P2_SBOX_RC0 \
    { \
    0x387c7997ddb86b2dull, 0xeaef0e16d57a01b1ull, 0x56194e5f22b13d3full, 0xf1c2b617a3fb0d63ull, \
    0x2cf5b8a51a6f0ae2ull, 0xcfa4b3786daf48b0ull, 0x1c4c56702fac6714ull, 0xcd56a4eb1f507954ull, \
    }

struct P2Const {
    static constexpr u64 ext[8][8] = GB_P2_RC_EXT;
    static constexpr u64 inner[22] = GB_P2_RC_INT;
    static constexpr u64 diag[8] = GB_P2_DIAG;
};
// p2_permute's multiply-add needs every diagonal entry below p
static_assert(P2Const::diag[0] < GL_P && P2Const::diag[1] < GL_P && P2Const::diag[2] < GL_P &&
                  P2Const::diag[3] < GL_P && P2Const::diag[4] < GL_P && P2Const::diag[5] < GL_P &&
                  P2Const::diag[6] < GL_P && P2Const::diag[7] < GL_P,
              "internal diagonal must be canonical");

__device__ __forceinline__ u64 p2_rc_ext(int r, int i) {
    constexpr u64 t[8][8] = GB_P2_RC_EXT;
    return t[r][i];
}
__device__ __forceinline__ u64 p2_rc_int(int r) {
    constexpr u64 t[22] = GB_P2_RC_INT;
    return t[r];
}
__device__ __forceinline__ u64 p2_diag(int i) {
    constexpr u64 t[8] = GB_P2_DIAG;
    return t[i];
}
__device__ __forceinline__ u64 p2_sbox_rc0(int i) {
    constexpr u64 t[8] = GB_P2_SBOX_RC0;
    return t[i];
}

__device__ __forceinline__ u64 p2_sbox(u64 x) {
    u64 x2 = gl_sqr(x);
    u64 x4 = gl_sqr(x2);
    u64 x3 = gl_mul(x2, x);
    return gl_mul(x4, x3);
}

// External linear layer on the S-box outputs x, with lazy sums: per half the circulant
// [2 3 1 1] (each output a sum of the half's inputs with coefficients 1..3), then each
// output plus the column sum of both halves; add[i] (the next round's constant) is folded
// into the same sum, and each output is reduced once (its high part is at most 21 + 1).
__device__ __forceinline__ void p2_external_linear_add(u64* x, const u64* add, bool has_add) {
    glw o[8];
#pragma unroll
    for (int h = 0; h < 8; h += 4) {
        glw a = glw_of(x[h]), b = glw_of(x[h + 1]), c = glw_of(x[h + 2]), d = glw_of(x[h + 3]);
        glw t01 = glw_add(a, b), t23 = glw_add(c, d);
        glw t0123 = glw_add(t01, t23);
        glw t01123 = glw_add(t0123, b), t01233 = glw_add(t0123, d);
        o[h] = glw_add(t01123, t01);                 // 2a + 3b + c + d
        o[h + 1] = glw_add(t01123, glw_add(c, c));   // a + 2b + 3c + d
        o[h + 2] = glw_add(t01233, t23);             // a + b + 2c + 3d
        o[h + 3] = glw_add(t01233, glw_add(a, a));   // 3a + b + c + 2d
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        glw col = glw_add(o[i], o[i + 4]);
        glw u = glw_add(o[i], col), v = glw_add(o[i + 4], col);
        if (has_add) {
            u = glw_add(u, add[i]);
            v = glw_add(v, add[i + 4]);
        }
        x[i] = glw_reduce(u);
        x[i + 4] = glw_reduce(v);
    }
}

// The permutation with every round constant folded into the preceding linear layer:
//   external round r: s <- E(sbox(s + rc_ext[r]));  internal round r: s0 <- sbox(s0 + rc_int[r]),
//   s_i <- diag_i s_i + sum(s) -- computed as one multiply-add per lane with the sum (and the
//   next round's constant) unreduced.
// LIVE < 8: lanes LIVE..7 of the input are zero (a leaf hash), so their first S-box is a constant
// and s[LIVE..7] are not read.
template <int LIVE = 8>
__device__ __forceinline__ void p2_permute(u64* s) {
    u64 rc[8];
#pragma unroll
    for (int i = 0; i < 8; i++)
        s[i] = i < LIVE ? p2_sbox(glw_reduce(glw_add(glw_of(s[i]), p2_rc_ext(0, i)))) : p2_sbox_rc0(i);
#pragma unroll
    for (int r = 0; r < 4; r++) {
        if (r < 3) {
#pragma unroll
            for (int i = 0; i < 8; i++) rc[i] = p2_rc_ext(r + 1, i);
            p2_external_linear_add(s, rc, true);
#pragma unroll
            for (int i = 0; i < 8; i++) s[i] = p2_sbox(s[i]);
        } else {
#pragma unroll
            for (int i = 0; i < 8; i++) rc[i] = i == 0 ? p2_rc_int(0) : 0;
            p2_external_linear_add(s, rc, true);
        }
    }
    // internal rounds; s[0] already holds s0 + rc_int[r]
#pragma unroll
    for (int r = 0; r < 22; r++) {
        s[0] = p2_sbox(s[0]);
        glw sum = glw_add(glw_add(glw_add(glw_of(s[0]), glw_of(s[1])), glw_add(glw_of(s[2]), glw_of(s[3]))),
                          glw_add(glw_add(glw_of(s[4]), glw_of(s[5])), glw_add(glw_of(s[6]), glw_of(s[7]))));
        if (r < 21) {
            s[0] = gl_mul_add(s[0], p2_diag(0), glw_add(sum, p2_rc_int(r + 1)));
#pragma unroll
            for (int i = 1; i < 8; i++) s[i] = gl_mul_add(s[i], p2_diag(i), sum);
        } else {
#pragma unroll
            for (int i = 0; i < 8; i++) s[i] = gl_mul_add(s[i], p2_diag(i), glw_add(sum, p2_rc_ext(4, i)));
        }
    }
#pragma unroll
    for (int i = 0; i < 8; i++) s[i] = p2_sbox(s[i]);
#pragma unroll
    for (int r = 4; r < 8; r++) {
        if (r < 7) {
#pragma unroll
            for (int i = 0; i < 8; i++) rc[i] = p2_rc_ext(r + 1, i);
            p2_external_linear_add(s, rc, true);
#pragma unroll
            for (int i = 0; i < 8; i++) s[i] = p2_sbox(s[i]);
        } else {
            p2_external_linear_add(s, rc, false);
        }
    }
}

// ---------------------------------------------------------------------------
// Cooperative form: 8 lanes of a warp hold one state, lane l holding s[l].
// One thread's permutation is a serial chain of ~112 dependent multiplications;
// spreading the lanes over 8 threads leaves only the S-box chain and the linear
// layers' shuffles on the critical path, which is what latency-bound work (the
// small top layers of a Merkle tree) needs.  All 32 lanes of a warp must call it.
// ---------------------------------------------------------------------------
static __constant__ u64 c_p2_ext[8][8] = GB_P2_RC_EXT;
static __constant__ u64 c_p2_int[22] = GB_P2_RC_INT;
static __constant__ u64 c_p2_diag[8] = GB_P2_DIAG;

__device__ __forceinline__ u64 shfl_xor64(u64 v, int m) {
    u32 lo = __shfl_xor_sync(0xffffffffu, (u32)v, m), hi = __shfl_xor_sync(0xffffffffu, (u32)(v >> 32), m);
    return ((u64)hi << 32) | lo;
}
__device__ __forceinline__ u64 shfl_idx64(u64 v, int src) {
    u32 lo = __shfl_sync(0xffffffffu, (u32)v, src), hi = __shfl_sync(0xffffffffu, (u32)(v >> 32), src);
    return ((u64)hi << 32) | lo;
}

// per-lane round constants of lane l (8 external-round constants and the diagonal entry)
struct P2Lane {
    u64 ext[8];
    u64 diag;
};
__device__ __forceinline__ P2Lane p2_lane_consts(int l) {
    P2Lane c;
#pragma unroll
    for (int r = 0; r < 8; r++) c.ext[r] = c_p2_ext[r][l];
    c.diag = c_p2_diag[l];
    return c;
}

// external layer on 8 lanes: within a half, out_j = (x0+x1+x2+x3) + x_j + 2 x_{j+1};
// then every lane adds the column sum of both halves
__device__ __forceinline__ u64 p2_coop_external_linear(u64 x) {
    int lane = threadIdx.x & 31;
    u64 t = gl_add(x, shfl_xor64(x, 1));
    u64 all = gl_add(t, shfl_xor64(t, 2));
    u64 nxt = shfl_idx64(x, (lane & ~3) | ((lane + 1) & 3));
    u64 out = gl_add(gl_add(all, x), gl_double(nxt));
    return gl_add(out, gl_add(out, shfl_xor64(out, 4)));
}

// Latency-oriented multiply for the cooperative form, whose cost is the S-box chain's latency,
// not its instruction count: two independent 64-bit products and the compare-based reduction
// (fewer dependent steps than the carry-chain product that the throughput kernels use).
__device__ __forceinline__ u64 gl_mul_lat(u64 a, u64 b) {
    u64 lo = a * b, hi = __umul64hi(a, b);
    u64 h1 = hi >> 32, h0 = hi & GL_EPS;
    u64 t0 = lo - h1;
    if (lo < h1) t0 -= GL_EPS;
    u64 t1 = (h0 << 32) - h0;
    u64 r = t0 + t1;
    if (r < t1) r += GL_EPS;
    return r;
}
__device__ __forceinline__ u64 p2_sbox_lat(u64 x) {
    u64 x2 = gl_mul_lat(x, x);
    u64 x3 = gl_mul_lat(x2, x), x4 = gl_mul_lat(x2, x2);
    return gl_mul_lat(x4, x3);
}
__device__ __forceinline__ glw shfl_xor_glw(glw v, int m) {
    glw r;
    r.lo = shfl_xor64(v.lo, m);
    r.hi = __shfl_xor_sync(0xffffffffu, v.hi, m);
    return r;
}

// Internal rounds: the sum of lanes 1..7 is all-reduced while lane 0 computes its S-box (lane 0
// adds 0), then lane 0's S-box output is broadcast and added, so the shuffles leave the S-box
// chain.  The sum stays lazy (64 bits + carries) and enters the lane's multiply-add unreduced;
// lane 0 also folds in the next round's constant.
__device__ __forceinline__ u64 p2_permute_coop(u64 x, int l, const P2Lane& c) {
    const int lane0 = (threadIdx.x & 31) & ~7;
#pragma unroll
    for (int r = 0; r < 4; r++) x = p2_coop_external_linear(p2_sbox_lat(gl_add(x, c.ext[r])));
    if (l == 0) x = gl_add(x, c_p2_int[0]);
#pragma unroll
    for (int r = 0; r < 22; r++) {
        glw t = glw_of(l == 0 ? 0ull : x);
        t = glw_add(t, shfl_xor_glw(t, 1));
        t = glw_add(t, shfl_xor_glw(t, 2));
        t = glw_add(t, shfl_xor_glw(t, 4));
        const u64 y = p2_sbox_lat(x);
        if (l == 0) x = y;
        t = glw_add(t, shfl_idx64(y, lane0));
        if (l == 0 && r < 21) t = glw_add(t, c_p2_int[r + 1]);
        x = gl_mul_add(x, c.diag, t);
    }
#pragma unroll
    for (int r = 4; r < 8; r++) x = p2_coop_external_linear(p2_sbox_lat(gl_add(x, c.ext[r])));
    return x;
}

// ---------------------------------------------------------------------------
// Pair form: 2 adjacent lanes hold one state, lane h (h = lane & 1) holding s[4h .. 4h+3].
// The external circulant stays within a lane; the column sums and the internal rounds'
// sum take one exchange with the partner.  It issues about as many instructions per
// permutation as the one-thread form, in warp streams half as long, which suits layers too
// small to fill the GPU with one-thread permutations.  All 32 lanes of a warp must call it.
// ---------------------------------------------------------------------------
__device__ __forceinline__ u64 p2_sel(int h, u64 lo, u64 hi) { return h ? hi : lo; }

// this lane's half of the external layer, plus add[] (the next round's constants) when has_add
__device__ __forceinline__ void p2_pair_external(u64* x, const u64* add, bool has_add) {
    glw a = glw_of(x[0]), b = glw_of(x[1]), c = glw_of(x[2]), d = glw_of(x[3]);
    glw t01 = glw_add(a, b), t23 = glw_add(c, d);
    glw t0123 = glw_add(t01, t23);
    glw t01123 = glw_add(t0123, b), t01233 = glw_add(t0123, d);
    u64 o[4] = {glw_reduce(glw_add(t01123, t01)), glw_reduce(glw_add(t01123, glw_add(c, c))),
                glw_reduce(glw_add(t01233, t23)), glw_reduce(glw_add(t01233, glw_add(a, a)))};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        glw v = glw_add(glw_add(glw_of(o[i]), o[i]), shfl_xor64(o[i], 1));  // 2 o_i + partner's o_i
        if (has_add) v = glw_add(v, add[i]);
        x[i] = glw_reduce(v);
    }
}

__device__ __forceinline__ void p2_permute_pair(u64* s, int h) {
    u64 rc[4];
#pragma unroll
    for (int i = 0; i < 4; i++) s[i] = p2_sbox(glw_reduce(glw_add(glw_of(s[i]), p2_sel(h, p2_rc_ext(0, i), p2_rc_ext(0, 4 + i)))));
#pragma unroll
    for (int r = 0; r < 4; r++) {
        if (r < 3) {
#pragma unroll
            for (int i = 0; i < 4; i++) rc[i] = p2_sel(h, p2_rc_ext(r + 1, i), p2_rc_ext(r + 1, 4 + i));
            p2_pair_external(s, rc, true);
#pragma unroll
            for (int i = 0; i < 4; i++) s[i] = p2_sbox(s[i]);
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++) rc[i] = (i == 0 && h == 0) ? p2_rc_int(0) : 0;
            p2_pair_external(s, rc, true);
        }
    }
    u64 dg[4];
#pragma unroll
    for (int i = 0; i < 4; i++) dg[i] = p2_sel(h, p2_diag(i), p2_diag(4 + i));
    // internal rounds: lane 0 of the pair holds s0 (already plus rc_int[r]); both lanes run the
    // S-box on their s[0], lane 1 keeps its own value
#pragma unroll
    for (int r = 0; r < 22; r++) {
        const u64 y = p2_sbox(s[0]);
        if (h == 0) s[0] = y;
        glw loc = glw_add(glw_add(glw_of(s[0]), glw_of(s[1])), glw_add(glw_of(s[2]), glw_of(s[3])));
        glw sum = glw_add(loc, shfl_xor_glw(loc, 1));
        if (r < 21) {
            s[0] = gl_mul_add(s[0], dg[0], h == 0 ? glw_add(sum, p2_rc_int(r + 1)) : sum);
#pragma unroll
            for (int i = 1; i < 4; i++) s[i] = gl_mul_add(s[i], dg[i], sum);
        } else {
#pragma unroll
            for (int i = 0; i < 4; i++)
                s[i] = gl_mul_add(s[i], dg[i], glw_add(sum, p2_sel(h, p2_rc_ext(4, i), p2_rc_ext(4, 4 + i))));
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++) s[i] = p2_sbox(s[i]);
#pragma unroll
    for (int r = 4; r < 8; r++) {
        if (r < 7) {
#pragma unroll
            for (int i = 0; i < 4; i++) rc[i] = p2_sel(h, p2_rc_ext(r + 1, i), p2_rc_ext(r + 1, 4 + i));
            p2_pair_external(s, rc, true);
#pragma unroll
            for (int i = 0; i < 4; i++) s[i] = p2_sbox(s[i]);
        } else {
            p2_pair_external(s, rc, false);
        }
    }
}

// 2-to-1 compression P2(l || r)[0..4]
__device__ __forceinline__ void p2_compress(const u64* l, const u64* r, u64* out) {
    u64 s[8] = {l[0], l[1], l[2], l[3], r[0], r[1], r[2], r[3]};
    p2_permute(s);
    out[0] = s[0];
    out[1] = s[1];
    out[2] = s[2];
    out[3] = s[3];
}

}  // namespace gb
