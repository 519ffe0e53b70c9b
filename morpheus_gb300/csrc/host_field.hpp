// Host-side Goldilocks arithmetic, Poseidon2 and the Fiat-Shamir transcript
// used by the C++ proof drivers.  Canonical values throughout.
//
// The transcript is the zk-torch-3 overwrite-mode duplex sponge (width 8,
// rate 4; zk-torch-3/src/transcript.rs:174-330): absorbed values overwrite the
// rate, squeezes pop the rate in reverse order, labels are a length prefix plus
// one element per byte (empty labels absorb nothing).  gb_transcript carries
// exactly the Rust Transcript's fields so a caller can hand its state across the
// C ABI and take it back.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../../include/goldilocks_cuda_wrapper.h"
#include "poseidon2.cuh"

namespace gb {
namespace host {

typedef unsigned __int128 u128;

inline u64 canon(u64 a) { return a >= GL_P ? a - GL_P : a; }
inline u64 add(u64 a, u64 b) {
    a = canon(a);
    b = canon(b);
    u64 s = a + b;
    if (s < a || s >= GL_P) s -= GL_P;
    return s;
}
inline u64 sub(u64 a, u64 b) {
    a = canon(a);
    b = canon(b);
    return a >= b ? a - b : a + (GL_P - b);
}
inline u64 neg(u64 a) {
    a = canon(a);
    return a ? GL_P - a : 0;
}
inline u64 reduce(u128 x) {
    u64 lo = (u64)x, hi = (u64)(x >> 64);
    u64 h1 = hi >> 32, h0 = hi & GL_EPS;
    u64 t0 = lo - h1;
    if (lo < h1) t0 -= GL_EPS;
    u64 t1 = (h0 << 32) - h0;
    u64 r = t0 + t1;
    if (r < t1) r += GL_EPS;
    return canon(r);
}
inline u64 mul(u64 a, u64 b) { return reduce((u128)a * b); }
inline u64 pow(u64 a, u64 e) {
    u64 r = 1;
    while (e) {
        if (e & 1) r = mul(r, a);
        a = mul(a, a);
        e >>= 1;
    }
    return r;
}
inline u64 inv(u64 a) { return canon(a) ? pow(a, GL_P - 2) : 0; }

struct E2 {
    u64 c0, c1;
};
inline E2 e2(u64 a, u64 b) { return E2{canon(a), canon(b)}; }
inline E2 e2add(E2 a, E2 b) { return E2{add(a.c0, b.c0), add(a.c1, b.c1)}; }
inline E2 e2sub(E2 a, E2 b) { return E2{sub(a.c0, b.c0), sub(a.c1, b.c1)}; }
inline E2 e2mul(E2 a, E2 b) {
    u64 m0 = mul(a.c0, b.c0), m1 = mul(a.c1, b.c1);
    return E2{add(m0, mul(7, m1)), add(mul(a.c0, b.c1), mul(a.c1, b.c0))};
}

// Poseidon2 (width 8) on the host, branch-free: values stay any u64 congruent mod p inside the
// permutation, sums are lazy 128-bit, and every reduction selects its corrections arithmetically
// (data-dependent branches on random field elements mispredict about half the time).  The
// output is canonical, equal to the canonical-throughout form of the same rounds.
inline u64 red128(u128 x) {  // any 128-bit value -> a u64 congruent to it
    const u64 lo = (u64)x, hi = (u64)(x >> 64);
    const u64 h1 = hi >> 32, h0 = hi & GL_EPS;
    u64 t0 = lo - h1;
    t0 -= ((u64)0 - (u64)(lo < h1)) & GL_EPS;  // a borrow is worth 2^64 == EPS: take it back
    const u64 t1 = (h0 << 32) - h0;
    u64 r = t0 + t1;
    r += ((u64)0 - (u64)(r < t1)) & GL_EPS;  // a carry is worth EPS (no second carry is possible)
    return r;
}
inline u64 mulr(u64 a, u64 b) { return red128((u128)a * b); }

// x + c for any u64 x and c < p: on a carry the wrapped sum is below c, and 2^64 == EPS (mod p)
inline u64 add_rc(u64 x, u64 c) {
    const u64 s = x + c;
    return s + (((u64)0 - (u64)(s < c)) & GL_EPS);
}

inline void p2_permute(u64 s[8]) {
    auto sbox = [](u64 x) {
        const u64 x2 = mulr(x, x), x4 = mulr(x2, x2), x3 = mulr(x2, x);
        return mulr(x4, x3);
    };
    // external layer: per half the circulant [2 3 1 1], then each output plus its column sum
    auto ext = [](u64* v) {
        u128 o[8];
        for (int h = 0; h < 8; h += 4) {
            const u128 a = v[h], b = v[h + 1], c = v[h + 2], d = v[h + 3];
            const u128 ab = a + b, cd = c + d, all = ab + cd;
            o[h] = all + b + ab;
            o[h + 1] = all + b + c + c;
            o[h + 2] = all + d + cd;
            o[h + 3] = all + d + a + a;
        }
        for (int i = 0; i < 4; i++) {
            const u128 col = o[i] + o[i + 4];
            v[i] = red128(o[i] + col);
            v[i + 4] = red128(o[i + 4] + col);
        }
    };
    for (int r = 0; r < 4; r++) {
        for (int i = 0; i < 8; i++) s[i] = sbox(add_rc(s[i], P2Const::ext[r][i]));
        ext(s);
    }
    // Internal round: x = s0 + rc, tot = x^7 + s1 + .. + s7, s_i' = s_i d_i + tot.  Lane 0 is the
    // round's dependency chain, so s0' = x^7 (d0 + 1) + (s1 + .. + s7) is formed as
    // x4 * (x2 * (x (d0 + 1))): three dependent multiplications from x instead of four.  The host
    // transcript's permutations run back to back between rounds, so this chain is their latency.
    static_assert(P2Const::diag[0] + 1 < GL_P, "d0 + 1 is a canonical constant");
    const u64 d0p1 = P2Const::diag[0] + 1;
    for (int r = 0; r < 22; r++) {
        const u128 rest = (u128)s[1] + s[2] + s[3] + s[4] + s[5] + s[6] + s[7];
        const u64 x = add_rc(s[0], P2Const::inner[r]);
        const u64 x2 = mulr(x, x), xc = mulr(x, d0p1);
        const u64 x4 = mulr(x2, x2), x3 = mulr(x2, x), x3c = mulr(x2, xc);
        const u128 tot = rest + mulr(x4, x3);
        s[0] = red128((u128)x4 * x3c + rest);
        for (int i = 1; i < 8; i++) s[i] = red128((u128)s[i] * P2Const::diag[i] + tot);
    }
    for (int r = 4; r < 8; r++) {
        for (int i = 0; i < 8; i++) s[i] = sbox(add_rc(s[i], P2Const::ext[r][i]));
        ext(s);
    }
    for (int i = 0; i < 8; i++) s[i] = canon(s[i]);
}

// ---- transcript ----
inline void tr_duplex(gb_transcript* t) {
    for (uint32_t i = 0; i < t->nin; i++) t->st[i] = t->inb[i];
    for (uint32_t i = t->nin; i < 4; i++) t->st[i] = 0;
    t->nin = 0;
    p2_permute(t->st);
    for (int i = 0; i < 4; i++) t->outb[3 - i] = t->st[i];
    t->nout = 4;
}
inline void tr_absorb(gb_transcript* t, u64 v) {
    t->nout = 0;
    t->inb[t->nin++] = v;
    if (t->nin == 4) tr_duplex(t);
}
inline u64 tr_squeeze(gb_transcript* t) {
    if (t->nout == 0) tr_duplex(t);
    return t->outb[--t->nout];
}
inline void tr_label(gb_transcript* t, const char* label) {
    size_t len = std::strlen(label);
    if (len == 0) return;
    tr_absorb(t, (u64)len);
    for (size_t i = 0; i < len; i++) tr_absorb(t, (u64)(unsigned char)label[i]);
}
inline void tr_append_u64(gb_transcript* t, const char* label, u64 v) {
    tr_label(t, label);
    tr_absorb(t, v);
}
inline void tr_append_ext2(gb_transcript* t, const char* label, E2 v) {
    tr_label(t, label);
    tr_absorb(t, v.c0);
    tr_absorb(t, v.c1);
}
inline u64 tr_challenge(gb_transcript* t, const char* label) {
    tr_label(t, label);
    return tr_squeeze(t);
}
inline E2 tr_challenge_ext2(gb_transcript* t, const char* label) {
    tr_label(t, label);
    u64 a = tr_squeeze(t);
    u64 b = tr_squeeze(t);
    return E2{a, b};
}

}  // namespace host
}  // namespace gb
