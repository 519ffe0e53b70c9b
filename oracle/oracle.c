/*
 * oracle.c -- CPU restatement of the zk-torch prover field hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product).  Each function
 * names the reference file:line whose behaviour it restates.  Arithmetic is
 * canonical mod p throughout; parity with the CUDA path is equality after
 * reduction mod p, the criterion the reference's own tests use.
 */
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef uint64_t u64;
typedef unsigned __int128 u128;

/* ----------------------------------------------------------------------
 * Host threads for the CPU baseline.  The reference's CPU prover runs one
 * opening per thread under rayon (zk-torch-3/src/dag/mod.rs:1120-1140); here
 * the large element-wise loops of one proof (Merkle layers, transform layers,
 * folds, sums) can instead be split over or_set_threads() threads.  Every split
 * loop writes disjoint outputs or reduces exactly mod p, so results do not
 * depend on the thread count.  Default: 1 thread.
 * ---------------------------------------------------------------------- */
#define OR_MAX_THREADS 256
static int g_threads = 1;
void or_set_threads(int k) { g_threads = k < 1 ? 1 : (k > OR_MAX_THREADS ? OR_MAX_THREADS : k); }
int or_get_threads(void) { return g_threads; }

typedef void (*or_range_fn)(void *ctx, size_t lo, size_t hi, int part);
typedef struct { or_range_fn fn; void *ctx; size_t lo, hi; int part; } or_job;
static void *or_job_run(void *a) {
    or_job *j = (or_job *)a;
    j->fn(j->ctx, j->lo, j->hi, j->part);
    return NULL;
}
/* Runs fn over [0, n) in at most or_parts(n, min_chunk) contiguous parts (part = 0, 1, ...). */
static int or_parts(size_t n, size_t min_chunk) {
    size_t k = (size_t)g_threads;
    if (min_chunk < 1) min_chunk = 1;
    if (k > n / min_chunk) k = n / min_chunk;
    return k < 1 ? 1 : (int)k;
}
static void par_for(size_t n, size_t min_chunk, or_range_fn fn, void *ctx) {
    int k = or_parts(n, min_chunk);
    if (k == 1) {
        fn(ctx, 0, n, 0);
        return;
    }
    pthread_t th[OR_MAX_THREADS];
    or_job jobs[OR_MAX_THREADS] = {{0}};
    int started[OR_MAX_THREADS];
    for (int t = 0; t < k; t++) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].lo = n * (size_t)t / (size_t)k;
        jobs[t].hi = n * (size_t)(t + 1) / (size_t)k;
        jobs[t].part = t;
        started[t] = t > 0 && pthread_create(&th[t], NULL, or_job_run, &jobs[t]) == 0;
    }
    or_job_run(&jobs[0]);
    for (int t = 1; t < k; t++) {
        if (started[t]) pthread_join(th[t], NULL);
        else or_job_run(&jobs[t]); /* no thread available: run it here */
    }
}
#define PAR_MIN 4096 /* elements per part below which a loop stays on one thread */

/* ======================================================================
 * Goldilocks p = 2^64 - 2^32 + 1   (goldilocks-cuda-rs/src/field.rs:9-100,
 * zk-torch-3/src/util/arith.rs:94-135)
 * ====================================================================== */
#define GL_P 0xFFFFFFFF00000001ULL
#define GL_EPS 0xFFFFFFFFULL /* 2^64 mod p */

static inline u64 gl_canon(u64 a) { return a >= GL_P ? a - GL_P : a; }

static inline u64 gl_add(u64 a, u64 b) {
    a = gl_canon(a);
    b = gl_canon(b);
    u64 s = a + b;
    if (s < a || s >= GL_P) s -= GL_P;
    return s;
}

static inline u64 gl_sub(u64 a, u64 b) {
    a = gl_canon(a);
    b = gl_canon(b);
    return a >= b ? a - b : a + (GL_P - b);
}

static inline u64 gl_neg(u64 a) {
    a = gl_canon(a);
    return a == 0 ? 0 : GL_P - a;
}

/* x = lo + 2^64 (hh 2^32 + hl) == lo - hh + hl (2^32 - 1)  (2^96 == -1). */
static inline u64 gl_reduce128(u128 x) {
    u64 lo = (u64)x, hi = (u64)(x >> 64);
    u64 hh = hi >> 32, hl = hi & GL_EPS;
    u64 t0 = lo - hh;
    if (lo < hh) t0 -= GL_EPS;
    u64 t1 = hl * GL_EPS;
    u64 r = t0 + t1;
    if (r < t0) r += GL_EPS;
    return gl_canon(r);
}

static inline u64 gl_mul(u64 a, u64 b) { return gl_reduce128((u128)a * b); }

static u64 gl_pow(u64 a, u64 e) {
    u64 r = 1;
    while (e) {
        if (e & 1) r = gl_mul(r, a);
        a = gl_mul(a, a);
        e >>= 1;
    }
    return r;
}

/* Fermat inverse, 0 -> 0 (arith.rs gl_inv). */
static inline u64 gl_inv(u64 a) {
    a = gl_canon(a);
    return a == 0 ? 0 : gl_pow(a, GL_P - 2);
}

u64 or_gl_add(u64 a, u64 b) { return gl_add(a, b); }
u64 or_gl_sub(u64 a, u64 b) { return gl_sub(a, b); }
u64 or_gl_mul(u64 a, u64 b) { return gl_mul(a, b); }
u64 or_gl_inv(u64 a) { return gl_inv(a); }

/* ---- Ext2 = F_p[X]/(X^2 - 7)  (goldilocks-cuda-rs/src/extension.rs:89-130) ---- */
typedef struct { u64 c0, c1; } e2;

static inline e2 e2_mk(u64 c0, u64 c1) { e2 r = {gl_canon(c0), gl_canon(c1)}; return r; }
static inline e2 e2_base(u64 a) { return e2_mk(a, 0); }
static inline e2 e2_add(e2 a, e2 b) { return e2_mk(gl_add(a.c0, b.c0), gl_add(a.c1, b.c1)); }
static inline e2 e2_sub(e2 a, e2 b) { return e2_mk(gl_sub(a.c0, b.c0), gl_sub(a.c1, b.c1)); }
static inline e2 e2_mul(e2 a, e2 b) {
    u64 m0 = gl_mul(a.c0, b.c0);
    u64 m1 = gl_mul(a.c1, b.c1);
    u64 c1 = gl_add(gl_mul(a.c0, b.c1), gl_mul(a.c1, b.c0));
    return e2_mk(gl_add(m0, gl_mul(7, m1)), c1);
}
static inline e2 e2_scale(e2 a, u64 s) { return e2_mk(gl_mul(a.c0, s), gl_mul(a.c1, s)); }
static inline int e2_eq(e2 a, e2 b) { return gl_canon(a.c0) == gl_canon(b.c0) && gl_canon(a.c1) == gl_canon(b.c1); }

/* norm-based inverse (zk-torch-3/src/util/arith.rs ext2_inv). */
static e2 e2_inv(e2 a) {
    u64 norm = gl_sub(gl_mul(a.c0, a.c0), gl_mul(7, gl_mul(a.c1, a.c1)));
    u64 ni = gl_inv(norm);
    return e2_mk(gl_mul(a.c0, ni), gl_neg(gl_mul(a.c1, ni)));
}

void or_ext2_mul(const u64 a[2], const u64 b[2], u64 out[2]) {
    e2 r = e2_mul(e2_mk(a[0], a[1]), e2_mk(b[0], b[1]));
    out[0] = r.c0;
    out[1] = r.c1;
}
void or_ext2_inv(const u64 a[2], u64 out[2]) {
    e2 r = e2_inv(e2_mk(a[0], a[1]));
    out[0] = r.c0;
    out[1] = r.c1;
}

/* ======================================================================
 * Poseidon2, width 8, x^7, 4 + 22 + 4 rounds.  Plonky3 Goldilocks
 * constants as carried by goldilocks-cuda-rs/src/cpu_poseidon2.rs:16-50 and
 * zk-torch-3/src/transcript.rs:6-58; permutation per cpu_poseidon2.rs:117-140.
 * ====================================================================== */
static const u64 P2_RC_EXT[8][8] = {
    {0xdd5743e7f2a5a5d9ULL, 0xcb3a864e58ada44bULL, 0xd5a3726889dedc0dULL, 0x79365a7f967583c1ULL,
     0xb7820c177b0a3c30ULL, 0x68a60479943b7240ULL, 0x0a22eeab67b97c41ULL, 0xbee9d90e037fa7d4ULL},
    {0xf1dda5b9259dfcb4ULL, 0x27515210be112d59ULL, 0x654a4db8f15f6c3aULL, 0x5a9bfff8c29db0c4ULL,
     0xb72f2628c95a885bULL, 0xffcb54fc166beaddULL, 0xe32f91d59c463772ULL, 0x9e0ff2a9bbea79dbULL},
    {0xce57d6245ddca6b2ULL, 0xb1fc8d402bba1eb1ULL, 0x64df974fb666d528ULL, 0x59e4e5b237e52e78ULL,
     0x5e255e2742caa8fcULL, 0xc4a17304e330ef9aULL, 0x60e3a513cdd9f0b1ULL, 0xbf29a6a5a0c9c8baULL},
    {0xcea721cce82fb11bULL, 0xe5b55eb8098ece81ULL, 0x4ec66bfb89f7c380ULL, 0xc33be12b6ef7e4faULL,
     0xa41b5f5b84c57d7dULL, 0xb526206b2138a936ULL, 0x9f7a5ac62f16eb4eULL, 0x7de77f405f683aa5ULL},
    {0x014ef1197d341346ULL, 0x9725e20825d07394ULL, 0xc8ff2a22516f3604ULL, 0xde1b51f7cf493493ULL,
     0xa7e3af1a53eadb78ULL, 0x9b7b7ee0ddf9f229ULL, 0xf0a460f2dc649e7dULL, 0xdc4448d02c2cb823ULL},
    {0xaa62c88e0b294011ULL, 0x058eb9d810ce9f74ULL, 0x4e3d7a5403566d24ULL, 0xe8ae66da2f8b7a63ULL,
     0x3fdad3b08dae2e0bULL, 0xec81e61303dd409bULL, 0x3cbaa1cd35d31fc4ULL, 0x847f7806eec88ffaULL},
    {0x98ae09a325893803ULL, 0xf8a6475077968838ULL, 0xdf55b7419443de5bULL, 0xdbe15699e696ca70ULL,
     0x8e54a27d8db00424ULL, 0x7679a45cd9d1e12aULL, 0x2844f52be73e0e2fULL, 0xd41f8eb31ada34f8ULL},
    {0xe9dd318bae1f3961ULL, 0xf7462137299efe1aULL, 0x6dbbe06779e1d573ULL, 0xfe35b05cbe707632ULL,
     0x5d8896b12654fd8cULL, 0x6f96ef47c32d4ae2ULL, 0xb0caa221dbbfc0daULL, 0x0bc2a5bf1f238d3fULL},
};
static const u64 P2_RC_INT[22] = {
    0x488897d85ff51f56ULL, 0x1140737ccb162218ULL, 0xa7eeb9215866ed35ULL, 0x9bd2976fee49fcc9ULL,
    0xc0c8f0de580a3fccULL, 0x4fb2dae6ee8fc793ULL, 0x343a89f35f37395bULL, 0x223b525a77ca72c8ULL,
    0x56ccb62574aaa918ULL, 0xc4d507d8027af9edULL, 0xa080673cf0b7e95cULL, 0xf0184884eb70dcf8ULL,
    0x044f10b0cb3d5c69ULL, 0xe9e3f7993938f186ULL, 0x1b761c80e772f459ULL, 0x606cec607a1b5facULL,
    0x14a0c2e1d45f03cdULL, 0x4eace8855398574fULL, 0xf905ca7103eff3e6ULL, 0xf8c8f8d20862c059ULL,
    0xb524fe8bdd678e5aULL, 0xfbb7865901a1ec41ULL,
};
static const u64 P2_DIAG[8] = {
    0xa98811a1fed4e3a5ULL, 0x1cc48b54f377e2a0ULL, 0xe40cd4f6c5609a26ULL, 0x11de79ebca97a4a3ULL,
    0x9177c73d8b7e929cULL, 0x2a6fe8085797e791ULL, 0x3de6e93329f8d5adULL, 0x3f7af9125da962feULL,
};

static inline u64 p2_sbox(u64 x) {
    u64 x2 = gl_mul(x, x), x4 = gl_mul(x2, x2), x3 = gl_mul(x2, x);
    return gl_mul(x4, x3);
}

/* circulant [2 3 1 1] on each half, then add the column sums of both halves. */
static void p2_external_linear(u64 s[8]) {
    for (int h = 0; h < 8; h += 4) {
        u64 a = s[h], b = s[h + 1], c = s[h + 2], d = s[h + 3];
        u64 ab = gl_add(a, b), cd = gl_add(c, d), all = gl_add(ab, cd);
        u64 all_b = gl_add(all, b), all_d = gl_add(all, d);
        s[h] = gl_add(all_b, ab);
        s[h + 1] = gl_add(all_b, gl_add(c, c));
        s[h + 2] = gl_add(all_d, cd);
        s[h + 3] = gl_add(all_d, gl_add(a, a));
    }
    for (int i = 0; i < 4; i++) {
        u64 col = gl_add(s[i], s[i + 4]);
        s[i] = gl_add(s[i], col);
        s[i + 4] = gl_add(s[i + 4], col);
    }
}

void or_poseidon2_permute(u64 s[8]) {
    for (int i = 0; i < 8; i++) s[i] = gl_canon(s[i]);
    for (int r = 0; r < 4; r++) {
        for (int i = 0; i < 8; i++) s[i] = p2_sbox(gl_add(s[i], P2_RC_EXT[r][i]));
        p2_external_linear(s);
    }
    for (int r = 0; r < 22; r++) {
        s[0] = p2_sbox(gl_add(s[0], P2_RC_INT[r]));
        u64 sum = 0;
        for (int i = 0; i < 8; i++) sum = gl_add(sum, s[i]);
        for (int i = 0; i < 8; i++) s[i] = gl_add(gl_mul(s[i], P2_DIAG[i]), sum);
    }
    for (int r = 4; r < 8; r++) {
        for (int i = 0; i < 8; i++) s[i] = p2_sbox(gl_add(s[i], P2_RC_EXT[r][i]));
        p2_external_linear(s);
    }
}

/* leaf = P2(a, b, 0^6)[0..4]  (cpu_poseidon2.rs:170-181; wrapper.cu hash_gl_leaves_kernel) */
void or_poseidon2_hash_gl_leaf(u64 a, u64 b, u64 out[4]) {
    u64 s[8] = {a, b, 0, 0, 0, 0, 0, 0};
    or_poseidon2_permute(s);
    memcpy(out, s, 32);
}
/* leaf = P2(a.c0, a.c1, b.c0, b.c1, 0^4)[0..4]  (cpu_poseidon2.rs:183-196) */
void or_poseidon2_hash_ext2_leaf(const u64 a[2], const u64 b[2], u64 out[4]) {
    u64 s[8] = {a[0], a[1], b[0], b[1], 0, 0, 0, 0};
    or_poseidon2_permute(s);
    memcpy(out, s, 32);
}
/* compress = P2(l || r)[0..4]  (cpu_poseidon2.rs:152-167) */
void or_poseidon2_compress(const u64 l[4], const u64 r[4], u64 out[4]) {
    u64 s[8];
    memcpy(s, l, 32);
    memcpy(s + 4, r, 32);
    or_poseidon2_permute(s);
    memcpy(out, s, 32);
}

/* ======================================================================
 * Transcript: overwrite-mode duplex sponge, width 8 / rate 4
 * (zk-torch-3/src/transcript.rs:174-330)
 * ====================================================================== */
size_t or_transcript_size(void) { return sizeof(or_transcript); }

static void tr_duplex(or_transcript *t) {
    for (int i = 0; i < t->nin; i++) t->st[i] = t->inb[i];
    for (int i = t->nin; i < 4; i++) t->st[i] = 0;
    t->nin = 0;
    or_poseidon2_permute(t->st);
    for (int i = 0; i < 4; i++) t->outb[3 - i] = t->st[i];
    t->nout = 4;
}
static void tr_absorb(or_transcript *t, u64 v) {
    t->nout = 0;
    t->inb[t->nin++] = v;
    if (t->nin == 4) tr_duplex(t);
}
static u64 tr_squeeze(or_transcript *t) {
    if (t->nout == 0) tr_duplex(t);
    return t->outb[--t->nout];
}
/* length prefix + bytes; empty labels absorb nothing (transcript.rs:199-208) */
static void tr_label(or_transcript *t, const uint8_t *label, size_t len) {
    if (len == 0) return;
    tr_absorb(t, (u64)len);
    for (size_t i = 0; i < len; i++) tr_absorb(t, label[i]);
}

void or_tr_new(or_transcript *t, const uint8_t *label, size_t len) {
    memset(t, 0, sizeof(*t));
    for (size_t i = 0; i < len; i++) tr_absorb(t, label[i]);
}
void or_tr_append_u64(or_transcript *t, const uint8_t *label, size_t len, u64 v) {
    tr_label(t, label, len);
    tr_absorb(t, v);
}
void or_tr_append_scalar(or_transcript *t, const uint8_t *label, size_t len, u64 v) {
    tr_label(t, label, len);
    tr_absorb(t, v);
}
void or_tr_append_ext2(or_transcript *t, const uint8_t *label, size_t len, const u64 v[2]) {
    tr_label(t, label, len);
    tr_absorb(t, v[0]);
    tr_absorb(t, v[1]);
}
u64 or_tr_challenge_scalar(or_transcript *t, const uint8_t *label, size_t len) {
    tr_label(t, label, len);
    return tr_squeeze(t);
}
void or_tr_challenge_ext2(or_transcript *t, const uint8_t *label, size_t len, u64 out[2]) {
    tr_label(t, label, len);
    out[0] = tr_squeeze(t);
    out[1] = tr_squeeze(t);
}

#define LBL(s) (const uint8_t *)(s), (sizeof(s) - 1)

/* BasefoldTranscript impl for Transcript (transcript.rs:331-350): empty labels. */
static void bt_observe_ext2(or_transcript *t, e2 v) {
    u64 a[2] = {v.c0, v.c1};
    or_tr_append_ext2(t, (const uint8_t *)"", 0, a);
}
static void bt_observe_hash(or_transcript *t, const u64 h[4]) {
    for (int i = 0; i < 4; i++) or_tr_append_scalar(t, (const uint8_t *)"", 0, h[i]);
}
static u64 bt_sample(or_transcript *t) { return or_tr_challenge_scalar(t, (const uint8_t *)"", 0); }
static e2 bt_sample_ext2(or_transcript *t) {
    u64 c[2];
    or_tr_challenge_ext2(t, (const uint8_t *)"", 0, c);
    return e2_mk(c[0], c[1]);
}

/* ======================================================================
 * Product sumcheck
 * ====================================================================== */

/* CpuLinearSumcheckProverExt2::{new,prove} on base inputs lifted to Ext2
 * (zk-torch-3/src/sumcheck/cpu_ext2_prover.rs:23-110; identical transcript calls
 * to GpuLinearSumcheckProver::prove, gpu_prover.rs:21-89). */
static int sumcheck_ext2_rounds(or_transcript *t, int n, int d, e2 *w, u64 *msgs, u64 *challenges, u64 *finals,
                                u64 *final_eval);

int or_sumcheck_prove_ext2(or_transcript *t, int n, int d, const u64 *polys, u64 *msgs,
                           u64 *challenges, u64 *finals, u64 *final_eval) {
    if (n < 0 || d < 1) return -1;
    size_t N = (size_t)1 << n;
    e2 *w = (e2 *)malloc(sizeof(e2) * N * d);
    if (!w) return -2;
    for (int i = 0; i < d; i++)
        for (size_t k = 0; k < N; k++) w[i * N + k] = e2_base(polys[i * N + k]);
    return sumcheck_ext2_rounds(t, n, d, w, msgs, challenges, finals, final_eval);
}

/* The same prover on Ext2 polynomials, polys[d][2^n][2] (CpuLinearSumcheckProverExt2::prove takes
 * Ext2 vectors, cpu_ext2_prover.rs:35-110). */
int or_sumcheck_prove_ext2_polys(or_transcript *t, int n, int d, const u64 *polys, u64 *msgs,
                                 u64 *challenges, u64 *finals, u64 *final_eval) {
    if (n < 0 || d < 1) return -1;
    size_t N = (size_t)1 << n;
    e2 *w = (e2 *)malloc(sizeof(e2) * N * d);
    if (!w) return -2;
    for (size_t k = 0; k < N * d; k++) w[k] = e2_mk(polys[2 * k], polys[2 * k + 1]);
    return sumcheck_ext2_rounds(t, n, d, w, msgs, challenges, finals, final_eval);
}

/* rounds of the Ext2 prover over w (freed here) */
static int sumcheck_ext2_rounds(or_transcript *t, int n, int d, e2 *w, u64 *msgs, u64 *challenges, u64 *finals,
                                u64 *final_eval) {
    size_t N = (size_t)1 << n;
    or_tr_append_u64(t, LBL("num_var"), (u64)n);
    or_tr_append_u64(t, LBL("num_poly"), (u64)d);
    size_t cur = N;
    for (int rd = 0; rd < n; rd++) {
        size_t half = cur / 2;
        for (int c = 0; c <= d; c++) {
            e2 cc = e2_base((u64)c), sum = e2_base(0);
            for (size_t j = 0; j < half; j++) {
                e2 prod = e2_base(1);
                for (int i = 0; i < d; i++) {
                    e2 a = w[i * N + 2 * j], b = w[i * N + 2 * j + 1];
                    prod = e2_mul(prod, e2_add(a, e2_mul(cc, e2_sub(b, a))));
                }
                sum = e2_add(sum, prod);
            }
            u64 *m = msgs + ((size_t)rd * (d + 1) + c) * 2;
            m[0] = sum.c0;
            m[1] = sum.c1;
        }
        for (int c = 0; c <= d; c++)
            or_tr_append_ext2(t, LBL("round_message"), msgs + ((size_t)rd * (d + 1) + c) * 2);
        u64 ch[2];
        or_tr_challenge_ext2(t, LBL("challenge"), ch);
        challenges[2 * rd] = ch[0];
        challenges[2 * rd + 1] = ch[1];
        e2 r = e2_mk(ch[0], ch[1]);
        for (int i = 0; i < d; i++)
            for (size_t j = 0; j < half; j++) {
                e2 a = w[i * N + 2 * j], b = w[i * N + 2 * j + 1];
                w[i * N + j] = e2_add(a, e2_mul(r, e2_sub(b, a)));
            }
        cur = half;
    }
    e2 fe = e2_base(1);
    for (int i = 0; i < d; i++) {
        finals[2 * i] = w[i * N].c0;
        finals[2 * i + 1] = w[i * N].c1;
        fe = e2_mul(fe, w[i * N]);
    }
    final_eval[0] = fe.c0;
    final_eval[1] = fe.c1;
    free(w);
    return 0;
}

/* LinearSumcheckProver::{new,prove} (zk-torch-3/src/sumcheck/linear_prover.rs:23-131). */
int or_sumcheck_prove_base(or_transcript *t, int n, int d, const u64 *polys, u64 *msgs,
                           u64 *challenges, u64 *finals, u64 *final_eval) {
    if (n < 0 || d < 1) return -1;
    size_t N = (size_t)1 << n;
    or_tr_append_u64(t, LBL("num_var"), (u64)n);
    or_tr_append_u64(t, LBL("num_poly"), (u64)d);
    u64 *w = (u64 *)malloc(sizeof(u64) * N * d);
    if (!w) return -2;
    for (size_t k = 0; k < N * d; k++) w[k] = gl_canon(polys[k]);
    size_t cur = N;
    for (int rd = 0; rd < n; rd++) {
        size_t half = cur / 2;
        for (int c = 0; c <= d; c++) {
            u64 sum = 0;
            for (size_t j = 0; j < half; j++) {
                u64 prod = 1;
                for (int i = 0; i < d; i++) {
                    u64 a = w[i * N + 2 * j], b = w[i * N + 2 * j + 1];
                    prod = gl_mul(prod, gl_add(a, gl_mul((u64)c, gl_sub(b, a))));
                }
                sum = gl_add(sum, prod);
            }
            msgs[(size_t)rd * (d + 1) + c] = sum;
        }
        for (int c = 0; c <= d; c++)
            or_tr_append_scalar(t, LBL("round_message"), msgs[(size_t)rd * (d + 1) + c]);
        u64 r = or_tr_challenge_scalar(t, LBL("challenge"));
        challenges[rd] = r;
        for (int i = 0; i < d; i++)
            for (size_t j = 0; j < half; j++) {
                u64 a = w[i * N + 2 * j], b = w[i * N + 2 * j + 1];
                w[i * N + j] = gl_add(a, gl_mul(r, gl_sub(b, a)));
            }
        cur = half;
    }
    u64 fe = 1;
    for (int i = 0; i < d; i++) {
        finals[i] = w[i * N];
        fe = gl_mul(fe, w[i * N]);
    }
    final_eval[0] = fe;
    free(w);
    return 0;
}

/* Lagrange interpolation through (0..d-1, evals) evaluated at x (verifier.rs:112-133). */
static e2 interp_eval_ext2(const e2 *ev, int cnt, e2 x) {
    e2 res = e2_base(0);
    for (int i = 0; i < cnt; i++) {
        e2 basis = e2_base(1), xi = e2_base((u64)i);
        for (int j = 0; j < cnt; j++) {
            if (j == i) continue;
            e2 xj = e2_base((u64)j);
            basis = e2_mul(basis, e2_mul(e2_sub(x, xj), e2_inv(e2_sub(xi, xj))));
        }
        res = e2_add(res, e2_mul(basis, ev[i]));
    }
    return res;
}

int or_sumcheck_verify_ext2(or_transcript *t, int n, int d, const u64 claimed[2], const u64 *msgs,
                            const u64 final_eval[2]) {
    or_tr_append_u64(t, LBL("num_var"), (u64)n);
    or_tr_append_u64(t, LBL("num_poly"), (u64)d);
    e2 cur = e2_mk(claimed[0], claimed[1]);
    e2 *ev = (e2 *)malloc(sizeof(e2) * (d + 1));
    for (int rd = 0; rd < n; rd++) {
        const u64 *m = msgs + (size_t)rd * (d + 1) * 2;
        for (int c = 0; c <= d; c++) ev[c] = e2_mk(m[2 * c], m[2 * c + 1]);
        if (!e2_eq(e2_add(ev[0], ev[1]), cur)) {
            free(ev);
            return 0;
        }
        for (int c = 0; c <= d; c++) or_tr_append_ext2(t, LBL("round_message"), m + 2 * c);
        u64 ch[2];
        or_tr_challenge_ext2(t, LBL("challenge"), ch);
        cur = interp_eval_ext2(ev, d + 1, e2_mk(ch[0], ch[1]));
    }
    free(ev);
    return e2_eq(cur, e2_mk(final_eval[0], final_eval[1]));
}

/* ======================================================================
 * eq(r, x), variable i <-> bit i of x  (zk-torch-3/src/poly/mod.rs:106-161)
 * ====================================================================== */
void or_eq_table_base(const u64 *r, int n, u64 *out) {
    size_t N = (size_t)1 << n;
    memset(out, 0, N * 8);
    out[0] = 1;
    for (int i = 0; i < n; i++) {
        size_t half = (size_t)1 << i;
        u64 ri = gl_canon(r[i]), omr = gl_sub(1, ri);
        for (size_t j = half; j-- > 0;) {
            out[j | half] = gl_mul(out[j], ri);
            out[j] = gl_mul(out[j], omr);
        }
    }
}

typedef struct { e2 *out; size_t half; e2 r, omr; } eq_layer_ctx;
static void eq_layer_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    eq_layer_ctx *c = (eq_layer_ctx *)ctx;
    for (size_t j = lo; j < hi; j++) {
        c->out[j | c->half] = e2_mul(c->out[j], c->r);
        c->out[j] = e2_mul(c->out[j], c->omr);
    }
}
static void eq_table_ext2(const e2 *r, int n, e2 *out) {
    size_t N = (size_t)1 << n;
    for (size_t k = 0; k < N; k++) out[k] = e2_base(0);
    out[0] = e2_base(1);
    for (int i = 0; i < n; i++) {
        eq_layer_ctx c = {out, (size_t)1 << i, r[i], e2_sub(e2_base(1), r[i])};
        par_for(c.half, PAR_MIN, eq_layer_range, &c);
    }
}

void or_eq_table_ext2(const u64 *r, int n, u64 *out) {
    e2 *rr = (e2 *)malloc(sizeof(e2) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++) rr[i] = e2_mk(r[2 * i], r[2 * i + 1]);
    eq_table_ext2(rr, n, (e2 *)out);
    free(rr);
}

/* multilinear extension of base-field evals at an Ext2 point: sum_x evals[x] eq(r, x) */
void or_ml_eval_ext2(const u64 *evals, int n, const u64 *point, u64 out[2]) {
    size_t N = (size_t)1 << n;
    e2 *eq = (e2 *)malloc(sizeof(e2) * N);
    e2 *rr = (e2 *)calloc(n > 0 ? n : 1, sizeof(e2));
    for (int i = 0; i < n; i++) rr[i] = e2_mk(point[2 * i], point[2 * i + 1]);
    eq_table_ext2(rr, n, eq);
    e2 acc = e2_base(0);
    for (size_t k = 0; k < N; k++) acc = e2_add(acc, e2_scale(eq[k], evals[k]));
    out[0] = acc.c0;
    out[1] = acc.c1;
    free(eq);
    free(rr);
}

/* ======================================================================
 * Basefold
 * ====================================================================== */

size_t or_basefold_table_entries(int num_vars, int log_rate, int num_rounds) {
    size_t tot = 0;
    for (int i = 0; i < num_rounds; i++) tot += (size_t)1 << (num_vars + log_rate - i - 1);
    return tot;
}

static void table_invert_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    u64 *e = (u64 *)ctx;
    for (size_t k = lo; k < hi; k++) e[2 * k + 1] = gl_inv(e[2 * k + 1]);
}

/* BasefoldTable::generate: xorshift64 (13, 7, 17), each draw reduced % p; x1 redrawn
 * while equal to x0; weight = 1 / (x1 - x0)  (goldilocks-cuda-rs/src/basefold.rs:281-321). */
void or_basefold_table_generate(int num_vars, int log_rate, int num_rounds, u64 seed, u64 *entries,
                                u64 *level_offsets) {
    u64 st = seed;
#define XS_NEXT() (st ^= st << 13, st ^= st >> 7, st ^= st << 17, st % GL_P)
    size_t pos = 0;
    for (int i = 0; i < num_rounds; i++) {
        size_t sz = (size_t)1 << (num_vars + log_rate - i - 1);
        level_offsets[i] = pos;
        for (size_t k = 0; k < sz; k++) {
            u64 x0 = XS_NEXT();
            u64 x1 = XS_NEXT();
            while (x1 == x0) x1 = XS_NEXT();
            entries[2 * pos] = x0;
            entries[2 * pos + 1] = gl_sub(x1, x0);
            pos++;
        }
    }
#undef XS_NEXT
    par_for(pos, PAR_MIN, table_invert_range, entries);
}

static inline size_t bitrev(size_t x, int bits) {
    size_t r = 0;
    for (int i = 0; i < bits; i++) {
        r = (r << 1) | (x & 1);
        x >>= 1;
    }
    return r;
}

/* in-place bit-reversal of 2^log_n items of stride_words u64 (basefold.cuh:57-90) */
typedef struct { u64 *data; int log_n, stride; } bitrev_ctx;
/* each swap (i, j), i < j, is made by the part that owns i */
static void bitrev_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    bitrev_ctx *c = (bitrev_ctx *)ctx;
    u64 tmp[8];
    size_t w = (size_t)c->stride;
    for (size_t i = lo; i < hi; i++) {
        size_t j = bitrev(i, c->log_n);
        if (i < j) {
            memcpy(tmp, c->data + i * w, 8 * w);
            memcpy(c->data + i * w, c->data + j * w, 8 * w);
            memcpy(c->data + j * w, tmp, 8 * w);
        }
    }
}
void or_bit_reverse_u64(u64 *data, int log_n, int stride_words) {
    bitrev_ctx c = {data, log_n, stride_words};
    par_for((size_t)1 << log_n, PAR_MIN, bitrev_range, &c);
}

/* basefold_bhc_interpolate_ffi (goldilocks-cuda-rs/cuda/wrapper.cu:1242-1274 with
 * cuda/basefold.cuh:103-147): Moebius transform evals -> coeffs; bh_evals is the
 * bit-reversed copy of evals. */
/* one butterfly layer over pairs p = (base, j): base = (p / h) 2h, lo = base + j, hi = lo + h */
typedef struct { u64 *v; size_t h; int kind; } layer_ctx;
static void layer_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    layer_ctx *c = (layer_ctx *)ctx;
    size_t h = c->h;
    for (size_t p = lo; p < hi; p++) {
        size_t a = (p / h) * 2 * h + (p % h), b = a + h;
        if (c->kind == 0) { /* Moebius: hi -= lo */
            c->v[b] = gl_sub(c->v[b], c->v[a]);
        } else { /* +-1 butterfly */
            u64 x = c->v[a], y = c->v[b];
            c->v[a] = gl_add(x, y);
            c->v[b] = gl_sub(x, y);
        }
    }
}
typedef struct { u64 *dst; const u64 *src; int shift; } copy_ctx;
static void canon_copy_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    copy_ctx *c = (copy_ctx *)ctx;
    for (size_t k = lo; k < hi; k++) c->dst[k] = gl_canon(c->src[k >> c->shift]);
}

void or_bhc_interpolate(const u64 *evals, int n, u64 *coeffs, u64 *bh_evals) {
    size_t N = (size_t)1 << n;
    copy_ctx cc = {coeffs, evals, 0};
    par_for(N, PAR_MIN, canon_copy_range, &cc);
    for (int lvl = 0; lvl < n; lvl++) {
        layer_ctx lc = {coeffs, (size_t)1 << lvl, 0};
        par_for(N / 2, PAR_MIN, layer_range, &lc);
    }
    copy_ctx cb = {bh_evals, evals, 0};
    par_for(N, PAR_MIN, canon_copy_range, &cb);
    or_bit_reverse_u64(bh_evals, n, 1);
}

/* basefold_encode_ffi (wrapper.cu:1277-1313, basefold.cuh:157-205): repetition code
 * x 2^lr, n layers of (lo + hi, lo - hi) at half-chunk 2^(i+lr), then bit reversal. */
void or_basefold_encode(const u64 *coeffs, int n, int log_rate, u64 *cw) {
    size_t L = (size_t)1 << (n + log_rate);
    copy_ctx cc = {cw, coeffs, log_rate};
    par_for(L, PAR_MIN, canon_copy_range, &cc);
    for (int i = 0; i < n; i++) {
        layer_ctx lc = {cw, (size_t)1 << (i + log_rate), 1};
        par_for(L / 2, PAR_MIN, layer_range, &lc);
    }
    or_bit_reverse_u64(cw, n + log_rate, 1);
}

typedef struct { const u64 *in; u64 *out; } hash_ctx;
static void compress_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    hash_ctx *c = (hash_ctx *)ctx;
    for (size_t i = lo; i < hi; i++) or_poseidon2_compress(c->in + 8 * i, c->in + 8 * i + 4, c->out + 4 * i);
}
static void gl_leaf_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    hash_ctx *c = (hash_ctx *)ctx;
    for (size_t i = lo; i < hi; i++) or_poseidon2_hash_gl_leaf(c->in[2 * i], c->in[2 * i + 1], c->out + 4 * i);
}
static void ext2_leaf_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    hash_ctx *c = (hash_ctx *)ctx;
    for (size_t i = lo; i < hi; i++) or_poseidon2_hash_ext2_leaf(c->in + 4 * i, c->in + 4 * i + 2, c->out + 4 * i);
}
#define PAR_MIN_HASH 256 /* permutations per part */

static void merkle_layers(u64 *tree, size_t num_leaves) {
    size_t off = 0, sz = num_leaves;
    while (sz > 1) {
        hash_ctx c = {tree + off * 4, tree + (off + sz) * 4};
        par_for(sz / 2, PAR_MIN_HASH, compress_range, &c);
        off += sz;
        sz /= 2;
    }
}

/* DeviceMerkleTree::build_from_gl_codeword (merkle.rs:34-60; cpu_basefold.rs:22-78) */
void or_merkle_tree_gl(const u64 *cw, size_t num_leaves, u64 *tree) {
    hash_ctx c = {cw, tree};
    par_for(num_leaves, PAR_MIN_HASH, gl_leaf_range, &c);
    merkle_layers(tree, num_leaves);
}
void or_merkle_tree_ext2(const u64 *cw, size_t num_leaves, u64 *tree) {
    hash_ctx c = {cw, tree};
    par_for(num_leaves, PAR_MIN_HASH, ext2_leaf_range, &c);
    merkle_layers(tree, num_leaves);
}

static size_t tree_root_off(size_t num_leaves) { return (2 * num_leaves - 2) * 4; }

static void tree_path(const u64 *tree, size_t num_leaves, size_t leaf, u64 *out) {
    size_t off = 0, sz = num_leaves, idx = leaf, k = 0;
    while (sz > 1) {
        memcpy(out + 4 * k, tree + (off + (idx ^ 1)) * 4, 32);
        k++;
        off += sz;
        sz /= 2;
        idx >>= 1;
    }
}

void or_basefold_commit(const u64 *evals, int n, int log_rate, u64 *cw, u64 *bh_evals, u64 *tree,
                        u64 root[4]) {
    size_t N = (size_t)1 << n;
    u64 *coeffs = (u64 *)malloc(N * 8);
    or_bhc_interpolate(evals, n, coeffs, bh_evals);
    or_basefold_encode(coeffs, n, log_rate, cw);
    free(coeffs);
    size_t leaves = ((size_t)1 << (n + log_rate)) / 2;
    or_merkle_tree_gl(cw, leaves, tree);
    memcpy(root, tree + tree_root_off(leaves), 32);
}

static size_t path_words_total(int n, int lr) {
    size_t s = 0;
    for (int r = 0; r < n; r++) s += (size_t)(n + lr - 1 - r);
    return s * 4;
}

size_t or_basefold_proof_len(int n, int lr, int q) {
    size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    return 2 + (size_t)n * 6 + (size_t)(n - 1) * 4 + ((size_t)2 << lr) + (size_t)q * per_q;
}

/* P(0), P(1), P(2) partial sums of pairs [lo, hi), written to part's slot */
typedef struct { const e2 *bh, *eq; e2 (*acc)[3]; } pairs_ctx;
static void pairs_range(void *ctx, size_t lo, size_t hi, int part) {
    pairs_ctx *c = (pairs_ctx *)ctx;
    const e2 *eq = c->eq, *bh = c->bh;
    e2 two = e2_base(2);
    e2 p0 = e2_base(0), p1 = e2_base(0), p2 = e2_base(0);
    for (size_t j = lo; j < hi; j++) {
        p0 = e2_add(p0, e2_mul(eq[2 * j], bh[2 * j]));
        p1 = e2_add(p1, e2_mul(eq[2 * j + 1], bh[2 * j + 1]));
        e2 ei = e2_sub(e2_mul(two, eq[2 * j + 1]), eq[2 * j]);
        e2 bi = e2_sub(e2_mul(two, bh[2 * j + 1]), bh[2 * j]);
        p2 = e2_add(p2, e2_mul(ei, bi));
    }
    c->acc[part][0] = p0;
    c->acc[part][1] = p1;
    c->acc[part][2] = p2;
}

/* sumcheck oracle in coefficient form from P(0), P(1), P(2) (cpu_basefold.rs:157-221) */
static void oracle_from_pairs(const e2 *bh, const e2 *eq, size_t size, e2 out[3]) {
    e2 two = e2_base(2), inv2 = e2_base(9223372034707292161ULL);
    e2 acc[OR_MAX_THREADS][3];
    pairs_ctx pc = {bh, eq, acc};
    int parts = or_parts(size / 2, PAR_MIN);
    par_for(size / 2, PAR_MIN, pairs_range, &pc);
    e2 p0 = e2_base(0), p1 = e2_base(0), p2 = e2_base(0);
    for (int k = 0; k < parts; k++) {
        p0 = e2_add(p0, acc[k][0]);
        p1 = e2_add(p1, acc[k][1]);
        p2 = e2_add(p2, acc[k][2]);
    }
    e2 c2 = e2_mul(e2_add(e2_sub(p0, e2_mul(two, p1)), p2), inv2);
    out[0] = p0;
    out[2] = c2;
    out[1] = e2_sub(e2_sub(p1, p0), c2);
}

/* val0 + (ch - x0) * (val1 - val0) * w  (cpu_basefold.rs:87-129) */
static inline e2 fold_one(e2 v0, e2 v1, u64 x0, u64 w, e2 ch) {
    e2 diff_w = e2_scale(e2_sub(v1, v0), w);
    return e2_add(v0, e2_mul(e2_sub(ch, e2_base(x0)), diff_w));
}

static void put_e2(u64 *p, e2 v) {
    p[0] = v.c0;
    p[1] = v.c1;
}

/* open-phase loops split over host threads */
typedef struct { e2 *bh; const u64 *bh_evals; int n; } bh_init_ctx;
static void bh_init_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    bh_init_ctx *c = (bh_init_ctx *)ctx;
    for (size_t k = lo; k < hi; k++) c->bh[k] = e2_base(c->bh_evals[bitrev(k, c->n)]);
}
typedef struct { const e2 *a, *b; e2 *acc; } dot_ctx;
static void dot_range(void *ctx, size_t lo, size_t hi, int part) {
    dot_ctx *c = (dot_ctx *)ctx;
    e2 s = e2_base(0);
    for (size_t k = lo; k < hi; k++) s = e2_add(s, e2_mul(c->a[k], c->b[k]));
    c->acc[part] = s;
}
static e2 dot_ext2(const e2 *a, const e2 *b, size_t n) {
    e2 acc[OR_MAX_THREADS];
    dot_ctx c = {a, b, acc};
    int parts = or_parts(n, PAR_MIN);
    par_for(n, PAR_MIN, dot_range, &c);
    e2 s = e2_base(0);
    for (int k = 0; k < parts; k++) s = e2_add(s, acc[k]);
    return s;
}
/* eq and bh halves: dst[j] = src[2j] + ch (src[2j+1] - src[2j]), out of place */
typedef struct { const e2 *eq, *bh; e2 *eq_out, *bh_out; e2 ch; } half_fold_ctx;
static void half_fold_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    half_fold_ctx *c = (half_fold_ctx *)ctx;
    for (size_t j = lo; j < hi; j++) {
        e2 l = c->eq[2 * j], h = c->eq[2 * j + 1];
        c->eq_out[j] = e2_add(l, e2_mul(c->ch, e2_sub(h, l)));
        l = c->bh[2 * j];
        h = c->bh[2 * j + 1];
        c->bh_out[j] = e2_add(l, e2_mul(c->ch, e2_sub(h, l)));
    }
}
/* codeword fold: out[i] = fold(v[2i], v[2i+1]) with level table entry i */
typedef struct { const u64 *base_cw; const e2 *prev; const u64 *lv; e2 *out; e2 ch; } cw_fold_ctx;
static void cw_fold_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    cw_fold_ctx *c = (cw_fold_ctx *)ctx;
    for (size_t i = lo; i < hi; i++) {
        e2 v0, v1;
        if (c->base_cw) {
            v0 = e2_base(c->base_cw[2 * i]);
            v1 = e2_base(c->base_cw[2 * i + 1]);
        } else {
            v0 = c->prev[2 * i];
            v1 = c->prev[2 * i + 1];
        }
        c->out[i] = fold_one(v0, v1, c->lv[2 * i], c->lv[2 * i + 1], c->ch);
    }
}

int or_basefold_open_ext2(const u64 *cw0, const u64 *bh_evals, const u64 *tree0, const u64 root[4], int n,
                          int lr, const u64 *point, const u64 *tab, const u64 *lvl_off, or_transcript *t,
                          int num_queries, u64 *proof) {
    if (n < 2) return -1;
    size_t N = (size_t)1 << n;
    size_t L = (size_t)1 << (n + lr);
    u64 *pp = proof;

    bt_observe_hash(t, root);
    e2 *pt = (e2 *)malloc(sizeof(e2) * n);
    for (int i = 0; i < n; i++) {
        pt[i] = e2_mk(point[2 * i], point[2 * i + 1]);
        bt_observe_ext2(t, pt[i]);
    }
    e2 *eq = (e2 *)malloc(sizeof(e2) * N);
    eq_table_ext2(pt, n, eq);
    e2 *bh = (e2 *)malloc(sizeof(e2) * N);
    bh_init_ctx bc = {bh, bh_evals, n};
    par_for(N, PAR_MIN, bh_init_range, &bc);
    e2 *eq_b = (e2 *)malloc(sizeof(e2) * (N / 2));
    e2 *bh_b = (e2 *)malloc(sizeof(e2) * (N / 2));

    e2 eval = dot_ext2(bh, eq, N);
    put_e2(pp, eval);
    pp += 2;

    u64 *oracles = pp;
    pp += (size_t)n * 6;
    u64 *roots = pp;
    pp += (size_t)(n - 1) * 4;
    u64 *final_cw = pp;
    pp += (size_t)2 << lr;
    u64 *queries = pp;

    e2 o[3];
    oracle_from_pairs(bh, eq, N, o);
    for (int c = 0; c < 3; c++) {
        put_e2(oracles + 2 * c, o[c]);
        bt_observe_ext2(t, o[c]);
    }

    /* folded codewords kept for the query phase: fcw[r] has L >> (r+1) Ext2 elements */
    e2 **fcw = (e2 **)calloc(n, sizeof(e2 *));
    u64 **ftree = (u64 **)calloc(n, sizeof(u64 *));
    size_t sc = N;
    for (int rd = 0; rd < n; rd++) {
        e2 ch = bt_sample_ext2(t);
        if (rd < n - 1) {
            size_t half = sc / 2;
            half_fold_ctx hc = {eq, bh, eq_b, bh_b, ch};
            par_for(half, PAR_MIN, half_fold_range, &hc);
            e2 *t0 = eq, *t1 = bh;
            eq = eq_b;
            bh = bh_b;
            eq_b = t0;
            bh_b = t1;
            sc = half;
            oracle_from_pairs(bh, eq, sc, o);
            for (int c = 0; c < 3; c++) {
                put_e2(oracles + (size_t)(rd + 1) * 6 + 2 * c, o[c]);
                bt_observe_ext2(t, o[c]);
            }
        }
        /* fold codeword of L >> rd elements into L >> (rd+1) */
        size_t pairs = L >> (rd + 1);
        const u64 *lv = tab + 2 * lvl_off[rd];
        e2 *out = (e2 *)malloc(sizeof(e2) * pairs);
        cw_fold_ctx fc = {rd == 0 ? cw0 : NULL, rd == 0 ? NULL : fcw[rd - 1], lv, out, ch};
        par_for(pairs, PAR_MIN, cw_fold_range, &fc);
        fcw[rd] = out;
        if (rd < n - 1) {
            size_t leaves = pairs / 2;
            ftree[rd] = (u64 *)malloc((2 * leaves - 1) * 32);
            or_merkle_tree_ext2((const u64 *)out, leaves, ftree[rd]);
            memcpy(roots + 4 * rd, ftree[rd] + tree_root_off(leaves), 32);
            bt_observe_hash(t, roots + 4 * rd);
        }
    }
    for (size_t i = 0; i < ((size_t)1 << lr); i++) put_e2(final_cw + 2 * i, fcw[n - 1][i]);

    /* query phase (basefold.rs:2310-2406 / cpu_basefold.rs:371-411) */
    size_t leaves0 = L / 2;
    for (int q = 0; q < num_queries; q++) {
        u64 raw = bt_sample(t);
        size_t leaf = (size_t)(raw % (u64)leaves0);
        *queries++ = leaf;
        u64 *vals = queries;
        queries += (size_t)n * 4;
        put_e2(vals, e2_base(cw0[2 * leaf]));
        put_e2(vals + 2, e2_base(cw0[2 * leaf + 1]));
        size_t idx = leaf / 2;
        for (int r = 0; r + 1 < n; r++) {
            put_e2(vals + 4 * (r + 1), fcw[r][2 * idx]);
            put_e2(vals + 4 * (r + 1) + 2, fcw[r][2 * idx + 1]);
            idx /= 2;
        }
        tree_path(tree0, leaves0, leaf, queries);
        queries += (size_t)(n + lr - 1) * 4;
        idx = leaf / 2;
        for (int r = 0; r + 1 < n; r++) {
            size_t leaves = (L >> (r + 1)) / 2;
            tree_path(ftree[r], leaves, idx, queries);
            queries += (size_t)(n + lr - 2 - r) * 4;
            idx /= 2;
        }
    }
    for (int r = 0; r < n; r++) {
        free(fcw[r]);
        free(ftree[r]);
    }
    free(fcw);
    free(ftree);
    free(pt);
    free(eq);
    free(bh);
    free(eq_b);
    free(bh_b);
    return 0;
}

static int verify_path(const u64 leaf_hash[4], const u64 *path, int depth, size_t idx, const u64 root[4]) {
    u64 cur[4];
    memcpy(cur, leaf_hash, 32);
    for (int k = 0; k < depth; k++) {
        if (idx & 1)
            or_poseidon2_compress(path + 4 * k, cur, cur);
        else
            or_poseidon2_compress(cur, path + 4 * k, cur);
        idx >>= 1;
    }
    for (int i = 0; i < 4; i++)
        if (gl_canon(cur[i]) != gl_canon(root[i])) return 0;
    return 1;
}

int or_basefold_verify_ext2(const u64 root[4], int n, int lr, const u64 *point, const u64 *proof,
                            int num_queries, const u64 *tab, const u64 *lvl_off, or_transcript *t) {
    if (n < 2) return 0;
    const u64 *pp = proof;
    e2 eval = e2_mk(pp[0], pp[1]);
    pp += 2;
    const u64 *oracles = pp;
    pp += (size_t)n * 6;
    const u64 *roots = pp;
    pp += (size_t)(n - 1) * 4;
    const u64 *final_cw = pp;
    pp += (size_t)2 << lr;
    const u64 *queries = pp;

    bt_observe_hash(t, root);
    for (int i = 0; i < n; i++) bt_observe_ext2(t, e2_mk(point[2 * i], point[2 * i + 1]));
#define OR(r, c) e2_mk(oracles[(size_t)(r) * 6 + 2 * (c)], oracles[(size_t)(r) * 6 + 2 * (c) + 1])
    e2 s = e2_add(OR(0, 0), e2_add(OR(0, 0), e2_add(OR(0, 1), OR(0, 2))));
    if (!e2_eq(s, eval)) return 0;
    for (int c = 0; c < 3; c++) bt_observe_ext2(t, OR(0, c));
    e2 *ch = (e2 *)malloc(sizeof(e2) * n);
    for (int rd = 0; rd + 1 < n; rd++) {
        ch[rd] = bt_sample_ext2(t);
        e2 v = e2_add(OR(rd, 0), e2_add(e2_mul(OR(rd, 1), ch[rd]), e2_mul(OR(rd, 2), e2_mul(ch[rd], ch[rd]))));
        e2 nx = e2_add(OR(rd + 1, 0), e2_add(OR(rd + 1, 0), e2_add(OR(rd + 1, 1), OR(rd + 1, 2))));
        if (!e2_eq(v, nx)) {
            free(ch);
            return 0;
        }
        for (int c = 0; c < 3; c++) bt_observe_ext2(t, OR(rd + 1, c));
        bt_observe_hash(t, roots + 4 * rd);
    }
#undef OR
    ch[n - 1] = bt_sample_ext2(t);
    size_t L = (size_t)1 << (n + lr);
    int ok = 1;
    for (int q = 0; q < num_queries && ok; q++) {
        (void)bt_sample(t);
        size_t index = (size_t)*queries++;
        const u64 *vals = queries;
        queries += (size_t)n * 4;
        const u64 *paths = queries;
        queries += path_words_total(n, lr);
        if (index >= L / 2) {
            ok = 0;
            break;
        }
        u64 lh[4];
        or_poseidon2_hash_gl_leaf(vals[0], vals[2], lh);
        if (!verify_path(lh, paths, n + lr - 1, index, root)) {
            ok = 0;
            break;
        }
        const u64 *pth = paths + (size_t)(n + lr - 1) * 4;
        size_t fidx = index;
        for (int r = 0; r < n; r++) {
            e2 v0 = e2_mk(vals[4 * r], vals[4 * r + 1]), v1 = e2_mk(vals[4 * r + 2], vals[4 * r + 3]);
            const u64 *ent = tab + 2 * (lvl_off[r] + fidx);
            e2 f = e2_add(v0, e2_mul(e2_mul(e2_sub(ch[r], e2_base(ent[0])), e2_sub(v1, v0)), e2_base(ent[1])));
            if (r < n - 1) {
                const u64 *nv = vals + 4 * (r + 1);
                e2 exp = (fidx & 1) ? e2_mk(nv[2], nv[3]) : e2_mk(nv[0], nv[1]);
                if (!e2_eq(f, exp)) {
                    ok = 0;
                    break;
                }
                u64 nh[4];
                or_poseidon2_hash_ext2_leaf(nv, nv + 2, nh);
                int depth = n + lr - 2 - r;
                if (!verify_path(nh, pth, depth, fidx / 2, roots + 4 * r)) {
                    ok = 0;
                    break;
                }
                pth += (size_t)depth * 4;
            } else {
                size_t fi = fidx / 2;
                const u64 *e = final_cw + (fi * 2 + (fidx & 1)) * 2;
                if (!e2_eq(f, e2_mk(e[0], e[1]))) {
                    ok = 0;
                    break;
                }
            }
            fidx /= 2;
        }
    }
    free(ch);
    return ok;
}

/* ======================================================================
 * Batch opening of several committed polynomials at Ext2 points
 * (batch_open_ext2, goldilocks-cuda-rs/src/basefold.rs:1202-1532; verifier
 * batch_verify_ext2, :1931-2220).  Flat proof layout:
 *   outer oracles n x (c0, c1, c2) Ext2 | combined root 4 | inner eval 2 |
 *   inner oracles n x 6 | folded roots (n-1) x 4 | final codeword 2^lr Ext2 |
 *   q combined queries (the open_ext2 query layout, Ext2 values in round 0) |
 *   q x E individual queries: (v0, v1) base + path of depth n+lr-1.
 * ====================================================================== */

size_t or_basefold_batch_proof_len(int n, int lr, int q, int num_evals) {
    size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    size_t indiv = 2 + (size_t)(n + lr - 1) * 4;
    return (size_t)n * 6 + 4 + 2 + (size_t)n * 6 + (size_t)(n - 1) * 4 + ((size_t)2 << lr) + (size_t)q * per_q +
           (size_t)q * num_evals * indiv;
}

/* batching weights: eq(t, .) with t_0 on the most significant index bit (basefold.rs:3008-3026);
 * ell = 1 for a single evaluation, else log2 of the next power of two */
static int batch_ell(int num_evals) {
    int ell = 0;
    while (((size_t)1 << ell) < (size_t)num_evals) ell++;
    return num_evals <= 1 ? 1 : ell;
}
static void batch_weights(or_transcript *t, int num_evals, u64 *w) {
    int ell = batch_ell(num_evals);
    size_t sz = (size_t)1 << ell;
    u64 *res = (u64 *)calloc(sz, 8);
    res[0] = 1;
    for (int i = 0; i < ell; i++) {
        u64 ti = bt_sample(t);
        u64 omt = gl_sub(1, ti);
        size_t half = (size_t)1 << i;
        for (size_t j = half; j-- > 0;) {
            u64 v = res[j];
            res[2 * j] = gl_mul(v, omt);
            res[2 * j + 1] = gl_mul(v, ti);
        }
    }
    for (int i = 0; i < num_evals; i++) w[i] = res[i];
    free(res);
}

/* eq(r, pt) = prod_i (r_i pt_i + (1 - r_i)(1 - pt_i))  (basefold.rs:3218-3230) */
static e2 eq_eval_ext2(const e2 *r, const u64 *pt, int n) {
    e2 one = e2_base(1), acc = one;
    for (int i = 0; i < n; i++) {
        e2 p = e2_mk(pt[2 * i], pt[2 * i + 1]);
        e2 term = e2_add(e2_mul(r[i], p), e2_mul(e2_sub(one, r[i]), e2_sub(one, p)));
        acc = e2_mul(acc, term);
    }
    return acc;
}

static void put_oracle(u64 *dst, const e2 o[3], or_transcript *t) {
    for (int c = 0; c < 3; c++) {
        put_e2(dst + 2 * c, o[c]);
        bt_observe_ext2(t, o[c]);
    }
}

int or_basefold_batch_open_ext2(const u64 *const *codewords, const u64 *const *bh_evals, const u64 *const *trees,
                                const u64 *roots, int num_comms, int n, int lr, const u64 *points, int num_points,
                                const int *ev_poly, const int *ev_point, const u64 *ev_vals, int num_evals,
                                const u64 *tab, const u64 *lvl_off, or_transcript *t, int num_queries, u64 *proof) {
    if (n < 2 || num_comms < 1 || num_points < 1 || num_evals < 1) return -1;
    for (int i = 0; i < num_evals; i++)
        if (ev_poly[i] < 0 || ev_poly[i] >= num_comms || ev_point[i] < 0 || ev_point[i] >= num_points) return -1;
    const size_t N = (size_t)1 << n, L = (size_t)1 << (n + lr);
    u64 *outer = proof;
    u64 *croot = outer + (size_t)n * 6;
    u64 *ieval = croot + 4;
    u64 *inner = ieval + 2;
    u64 *froots = inner + (size_t)n * 6;
    u64 *final_cw = froots + (size_t)(n - 1) * 4;
    u64 *cq = final_cw + ((size_t)2 << lr);
    const size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    u64 *iq = cq + (size_t)num_queries * per_q;

    /* 1. transcript: every root, every point, every claimed value */
    for (int c = 0; c < num_comms; c++) bt_observe_hash(t, roots + 4 * c);
    for (int p = 0; p < num_points; p++)
        for (int i = 0; i < n; i++) bt_observe_ext2(t, e2_mk(points[((size_t)p * n + i) * 2], points[((size_t)p * n + i) * 2 + 1]));
    for (int i = 0; i < num_evals; i++) bt_observe_ext2(t, e2_mk(ev_vals[2 * i], ev_vals[2 * i + 1]));
    /* 2. weights */
    u64 *w = (u64 *)malloc(8 * (size_t)num_evals);
    batch_weights(t, num_evals, w);
    /* 3. g_p = sum over the point's evaluations of w_i * evals (natural order = bit-reversed bh_evals) */
    e2 *g = (e2 *)malloc(sizeof(e2) * N * num_points);
    e2 *eq = (e2 *)malloc(sizeof(e2) * N * num_points);
    for (size_t k = 0; k < N * num_points; k++) g[k] = e2_base(0);
    for (int i = 0; i < num_evals; i++) {
        e2 *gp = g + N * ev_point[i];
        const u64 *bh = bh_evals[ev_poly[i]];
        for (size_t k = 0; k < N; k++) gp[k] = e2_add(gp[k], e2_base(gl_mul(w[i], bh[bitrev(k, n)])));
    }
    /* 4. eq tables of the points */
    e2 *pt = (e2 *)malloc(sizeof(e2) * n);
    for (int p = 0; p < num_points; p++) {
        for (int i = 0; i < n; i++) pt[i] = e2_mk(points[((size_t)p * n + i) * 2], points[((size_t)p * n + i) * 2 + 1]);
        eq_table_ext2(pt, n, eq + N * p);
    }
    /* 5-7. outer sumcheck over sum_p eq_p g_p: n oracles, n challenges */
    e2 *r = (e2 *)malloc(sizeof(e2) * n);
    size_t sz = N;
    for (int rd = 0; rd < n; rd++) {
        if (rd > 0) {
            e2 ch = r[rd - 1];
            size_t half = sz / 2;
            for (int p = 0; p < num_points; p++) {
                e2 *gp = g + N * p, *ep = eq + N * p;
                for (size_t j = 0; j < half; j++) {
                    gp[j] = e2_add(gp[2 * j], e2_mul(ch, e2_sub(gp[2 * j + 1], gp[2 * j])));
                    ep[j] = e2_add(ep[2 * j], e2_mul(ch, e2_sub(ep[2 * j + 1], ep[2 * j])));
                }
            }
            sz = half;
        }
        e2 tot[3] = {e2_base(0), e2_base(0), e2_base(0)};
        for (int p = 0; p < num_points; p++) {
            e2 o[3];
            oracle_from_pairs(g + N * p, eq + N * p, sz, o);
            for (int c = 0; c < 3; c++) tot[c] = e2_add(tot[c], o[c]);
        }
        put_oracle(outer + (size_t)rd * 6, tot, t);
        r[rd] = bt_sample_ext2(t);
    }
    /* 8. combined codeword and evaluations with scalar_i = eq(r, point_i) w_i */
    e2 *eqr = (e2 *)malloc(sizeof(e2) * num_points);
    for (int p = 0; p < num_points; p++) eqr[p] = eq_eval_ext2(r, points + (size_t)p * n * 2, n);
    e2 *sc = (e2 *)malloc(sizeof(e2) * num_evals);
    for (int i = 0; i < num_evals; i++) sc[i] = e2_mul(eqr[ev_point[i]], e2_base(w[i]));
    e2 *ccw = (e2 *)malloc(sizeof(e2) * L);
    e2 *cbh = (e2 *)malloc(sizeof(e2) * N);
    for (size_t k = 0; k < L; k++) ccw[k] = e2_base(0);
    for (size_t k = 0; k < N; k++) cbh[k] = e2_base(0);
    for (int i = 0; i < num_evals; i++) {
        const u64 *cw = codewords[ev_poly[i]], *bh = bh_evals[ev_poly[i]];
        for (size_t k = 0; k < L; k++) ccw[k] = e2_add(ccw[k], e2_scale(sc[i], cw[k]));
        for (size_t k = 0; k < N; k++) cbh[k] = e2_add(cbh[k], e2_scale(sc[i], bh[bitrev(k, n)]));
    }
    /* 9. combined tree */
    size_t leaves0 = L / 2;
    u64 *ctree = (u64 *)malloc((2 * leaves0 - 1) * 32);
    or_merkle_tree_ext2((const u64 *)ccw, leaves0, ctree);
    memcpy(croot, ctree + tree_root_off(leaves0), 32);
    bt_observe_hash(t, croot);
    /* 10. inner phase: open_ext2's rounds on the Ext2 codeword and evaluations at r */
    e2 *ieq = (e2 *)malloc(sizeof(e2) * N);
    eq_table_ext2(r, n, ieq);
    e2 o[3];
    oracle_from_pairs(cbh, ieq, N, o);
    e2 iev = e2_add(o[0], e2_add(o[0], e2_add(o[1], o[2])));
    put_e2(ieval, iev);
    put_oracle(inner, o, t);
    e2 **fcw = (e2 **)calloc(n, sizeof(e2 *));
    u64 **ftree = (u64 **)calloc(n, sizeof(u64 *));
    sz = N;
    for (int rd = 0; rd < n; rd++) {
        e2 ch = bt_sample_ext2(t);
        if (rd < n - 1) {
            size_t half = sz / 2;
            for (size_t j = 0; j < half; j++) {
                ieq[j] = e2_add(ieq[2 * j], e2_mul(ch, e2_sub(ieq[2 * j + 1], ieq[2 * j])));
                cbh[j] = e2_add(cbh[2 * j], e2_mul(ch, e2_sub(cbh[2 * j + 1], cbh[2 * j])));
            }
            sz = half;
            oracle_from_pairs(cbh, ieq, sz, o);
            put_oracle(inner + (size_t)(rd + 1) * 6, o, t);
        }
        size_t pairs = L >> (rd + 1);
        const u64 *lv = tab + 2 * lvl_off[rd];
        const e2 *in = rd == 0 ? ccw : fcw[rd - 1];
        e2 *out = (e2 *)malloc(sizeof(e2) * pairs);
        for (size_t i = 0; i < pairs; i++) out[i] = fold_one(in[2 * i], in[2 * i + 1], lv[2 * i], lv[2 * i + 1], ch);
        fcw[rd] = out;
        if (rd < n - 1) {
            size_t lv_leaves = pairs / 2;
            ftree[rd] = (u64 *)malloc((2 * lv_leaves - 1) * 32);
            or_merkle_tree_ext2((const u64 *)out, lv_leaves, ftree[rd]);
            memcpy(froots + 4 * rd, ftree[rd] + tree_root_off(lv_leaves), 32);
            bt_observe_hash(t, froots + 4 * rd);
        }
    }
    for (size_t i = 0; i < ((size_t)1 << lr); i++) put_e2(final_cw + 2 * i, fcw[n - 1][i]);
    /* 11. queries: combined (Ext2) then individual (base) */
    size_t *leaf_of = (size_t *)malloc(sizeof(size_t) * (num_queries > 0 ? num_queries : 1));
    for (int q = 0; q < num_queries; q++) {
        size_t leaf = (size_t)(bt_sample(t) % (u64)leaves0);
        leaf_of[q] = leaf;
        u64 *qq = cq + (size_t)q * per_q;
        qq[0] = leaf;
        u64 *vals = qq + 1;
        put_e2(vals, ccw[2 * leaf]);
        put_e2(vals + 2, ccw[2 * leaf + 1]);
        size_t idx = leaf / 2;
        for (int rr = 0; rr + 1 < n; rr++) {
            put_e2(vals + 4 * (rr + 1), fcw[rr][2 * idx]);
            put_e2(vals + 4 * (rr + 1) + 2, fcw[rr][2 * idx + 1]);
            idx /= 2;
        }
        u64 *paths = vals + (size_t)n * 4;
        tree_path(ctree, leaves0, leaf, paths);
        paths += (size_t)(n + lr - 1) * 4;
        idx = leaf / 2;
        for (int rr = 0; rr + 1 < n; rr++) {
            tree_path(ftree[rr], (L >> (rr + 1)) / 2, idx, paths);
            paths += (size_t)(n + lr - 2 - rr) * 4;
            idx /= 2;
        }
    }
    const size_t indiv = 2 + (size_t)(n + lr - 1) * 4;
    for (int q = 0; q < num_queries; q++) {
        for (int i = 0; i < num_evals; i++) {
            u64 *d = iq + ((size_t)q * num_evals + i) * indiv;
            const u64 *cw = codewords[ev_poly[i]];
            d[0] = gl_canon(cw[2 * leaf_of[q]]);
            d[1] = gl_canon(cw[2 * leaf_of[q] + 1]);
            tree_path(trees[ev_poly[i]], leaves0, leaf_of[q], d + 2);
        }
    }
    for (int rd = 0; rd < n; rd++) {
        free(fcw[rd]);
        free(ftree[rd]);
    }
    free(fcw);
    free(ftree);
    free(leaf_of);
    free(ieq);
    free(ctree);
    free(ccw);
    free(cbh);
    free(sc);
    free(eqr);
    free(r);
    free(pt);
    free(eq);
    free(g);
    free(w);
    return 0;
}

static e2 oracle_at(const u64 *o, e2 x) {
    e2 c0 = e2_mk(o[0], o[1]), c1 = e2_mk(o[2], o[3]), c2 = e2_mk(o[4], o[5]);
    return e2_add(c0, e2_add(e2_mul(c1, x), e2_mul(c2, e2_mul(x, x))));
}
static e2 oracle_sum(const u64 *o) {
    e2 c0 = e2_mk(o[0], o[1]), c1 = e2_mk(o[2], o[3]), c2 = e2_mk(o[4], o[5]);
    return e2_add(c0, e2_add(c0, e2_add(c1, c2)));
}
static void observe_oracle(or_transcript *t, const u64 *o) {
    for (int c = 0; c < 3; c++) bt_observe_ext2(t, e2_mk(o[2 * c], o[2 * c + 1]));
}

int or_basefold_batch_verify_ext2(const u64 *roots, int num_comms, int n, int lr, const u64 *points, int num_points,
                                  const int *ev_poly, const int *ev_point, const u64 *ev_vals, int num_evals,
                                  const u64 *proof, int num_queries, const u64 *tab, const u64 *lvl_off,
                                  or_transcript *t) {
    if (n < 2 || num_comms < 1 || num_points < 1 || num_evals < 1) return 0;
    for (int i = 0; i < num_evals; i++)
        if (ev_poly[i] < 0 || ev_poly[i] >= num_comms || ev_point[i] < 0 || ev_point[i] >= num_points) return 0;
    const size_t L = (size_t)1 << (n + lr);
    const u64 *outer = proof;
    const u64 *croot = outer + (size_t)n * 6;
    const u64 *ieval = croot + 4;
    const u64 *inner = ieval + 2;
    const u64 *froots = inner + (size_t)n * 6;
    const u64 *final_cw = froots + (size_t)(n - 1) * 4;
    const u64 *cq = final_cw + ((size_t)2 << lr);
    const size_t per_q = 1 + (size_t)n * 4 + path_words_total(n, lr);
    const u64 *iq = cq + (size_t)num_queries * per_q;
    const size_t indiv = 2 + (size_t)(n + lr - 1) * 4;
    int ok = 1;

    for (int c = 0; c < num_comms; c++) bt_observe_hash(t, roots + 4 * c);
    for (int p = 0; p < num_points; p++)
        for (int i = 0; i < n; i++) bt_observe_ext2(t, e2_mk(points[((size_t)p * n + i) * 2], points[((size_t)p * n + i) * 2 + 1]));
    for (int i = 0; i < num_evals; i++) bt_observe_ext2(t, e2_mk(ev_vals[2 * i], ev_vals[2 * i + 1]));
    u64 *w = (u64 *)malloc(8 * (size_t)num_evals);
    batch_weights(t, num_evals, w);
    e2 claimed = e2_base(0);
    for (int i = 0; i < num_evals; i++) claimed = e2_add(claimed, e2_scale(e2_mk(ev_vals[2 * i], ev_vals[2 * i + 1]), w[i]));
    e2 *r = (e2 *)malloc(sizeof(e2) * n);
    e2 *ich = (e2 *)malloc(sizeof(e2) * n);
    e2 *sc = (e2 *)malloc(sizeof(e2) * num_evals);
    /* outer sumcheck */
    if (!e2_eq(oracle_sum(outer), claimed)) ok = 0;
    if (ok) {
        observe_oracle(t, outer);
        for (int rd = 0; rd + 1 < n && ok; rd++) {
            r[rd] = bt_sample_ext2(t);
            if (!e2_eq(oracle_at(outer + (size_t)rd * 6, r[rd]), oracle_sum(outer + (size_t)(rd + 1) * 6))) ok = 0;
            else observe_oracle(t, outer + (size_t)(rd + 1) * 6);
        }
    }
    if (ok) {
        r[n - 1] = bt_sample_ext2(t);
        if (!e2_eq(oracle_at(outer + (size_t)(n - 1) * 6, r[n - 1]), e2_mk(ieval[0], ieval[1]))) ok = 0;
    }
    /* inner sumcheck with the folded roots */
    if (ok) {
        bt_observe_hash(t, croot);
        if (!e2_eq(oracle_sum(inner), e2_mk(ieval[0], ieval[1]))) ok = 0;
    }
    if (ok) {
        observe_oracle(t, inner);
        for (int rd = 0; rd + 1 < n && ok; rd++) {
            ich[rd] = bt_sample_ext2(t);
            if (!e2_eq(oracle_at(inner + (size_t)rd * 6, ich[rd]), oracle_sum(inner + (size_t)(rd + 1) * 6))) ok = 0;
            else {
                observe_oracle(t, inner + (size_t)(rd + 1) * 6);
                bt_observe_hash(t, froots + 4 * rd);
            }
        }
    }
    if (ok) ich[n - 1] = bt_sample_ext2(t);
    /* queries */
    if (ok && num_queries > 0) {
        for (int i = 0; i < num_evals; i++)
            sc[i] = e2_mul(eq_eval_ext2(r, points + (size_t)ev_point[i] * n * 2, n), e2_base(w[i]));
        size_t *idx = (size_t *)malloc(sizeof(size_t) * num_queries);
        for (int q = 0; q < num_queries; q++) idx[q] = (size_t)(bt_sample(t) % (u64)(L / 2));
        for (int q = 0; q < num_queries && ok; q++) {
            const u64 *qq = cq + (size_t)q * per_q;
            size_t leaf = idx[q];
            if (qq[0] != leaf) {
                ok = 0;
                break;
            }
            const u64 *vals = qq + 1;
            const u64 *paths = vals + (size_t)n * 4;
            u64 lh[4];
            or_poseidon2_hash_ext2_leaf(vals, vals + 2, lh);
            if (!verify_path(lh, paths, n + lr - 1, leaf, croot)) {
                ok = 0;
                break;
            }
            const u64 *pth = paths + (size_t)(n + lr - 1) * 4;
            size_t fidx = leaf;
            for (int rd = 0; rd < n && ok; rd++) {
                e2 v0 = e2_mk(vals[4 * rd], vals[4 * rd + 1]), v1 = e2_mk(vals[4 * rd + 2], vals[4 * rd + 3]);
                const u64 *ent = tab + 2 * (lvl_off[rd] + fidx);
                e2 f = e2_add(v0, e2_mul(e2_mul(e2_sub(ich[rd], e2_base(ent[0])), e2_sub(v1, v0)), e2_base(ent[1])));
                if (rd < n - 1) {
                    const u64 *nv = vals + 4 * (rd + 1);
                    e2 exp = (fidx & 1) ? e2_mk(nv[2], nv[3]) : e2_mk(nv[0], nv[1]);
                    u64 nh[4];
                    or_poseidon2_hash_ext2_leaf(nv, nv + 2, nh);
                    int depth = n + lr - 2 - rd;
                    if (!e2_eq(f, exp) || !verify_path(nh, pth, depth, fidx / 2, froots + 4 * rd)) ok = 0;
                    pth += (size_t)depth * 4;
                } else {
                    const u64 *e = final_cw + ((fidx / 2) * 2 + (fidx & 1)) * 2;
                    if (!e2_eq(f, e2_mk(e[0], e[1]))) ok = 0;
                }
                fidx /= 2;
            }
            e2 a0 = e2_base(0), a1 = e2_base(0);
            for (int i = 0; i < num_evals && ok; i++) {
                const u64 *d = iq + ((size_t)q * num_evals + i) * indiv;
                u64 ih[4];
                or_poseidon2_hash_gl_leaf(d[0], d[1], ih);
                if (!verify_path(ih, d + 2, n + lr - 1, leaf, roots + 4 * ev_poly[i])) ok = 0;
                a0 = e2_add(a0, e2_scale(sc[i], d[0]));
                a1 = e2_add(a1, e2_scale(sc[i], d[1]));
            }
            if (ok && (!e2_eq(a0, e2_mk(vals[0], vals[1])) || !e2_eq(a1, e2_mk(vals[2], vals[3])))) ok = 0;
        }
        free(idx);
    }
    free(sc);
    free(ich);
    free(r);
    free(w);
    return ok;
}

/* ======================================================================
 * almost-Goldilocks q = 2^64 - 2^32 - 31, Ext2 = F_q[X]/(X^2 - 3)
 * (cuda_almost_goldilocks/almost_goldilocks.cuh, almost_extension.cuh)
 * ====================================================================== */
#define AGL_Q 0xFFFFFFFEFFFFFFE1ULL
static inline u64 agl_canon(u64 a) { return a >= AGL_Q ? a - AGL_Q : a; }
static inline u64 agl_add(u64 a, u64 b) { return (u64)(((u128)agl_canon(a) + agl_canon(b)) % AGL_Q); }
static inline u64 agl_sub(u64 a, u64 b) {
    a = agl_canon(a);
    b = agl_canon(b);
    return a >= b ? a - b : AGL_Q - (b - a);
}
static inline u64 agl_mul(u64 a, u64 b) { return (u64)(((u128)a * b) % AGL_Q); }
u64 or_agl_add(u64 a, u64 b) { return agl_add(a, b); }
u64 or_agl_sub(u64 a, u64 b) { return agl_sub(a, b); }
u64 or_agl_mul(u64 a, u64 b) { return agl_mul(a, b); }
void or_aext2_mul(const u64 a[2], const u64 b[2], u64 out[2]) {
    out[0] = agl_add(agl_mul(a[0], b[0]), agl_mul(3, agl_mul(a[1], b[1])));
    out[1] = agl_add(agl_mul(a[0], b[1]), agl_mul(a[1], b[0]));
}

/* ======================================================================
 * Partial evaluation, bit permutation, fused permute + partial evaluation
 * (cuda/partial_eval.cuh, goldilocks-cuda-rs/src/partial_eval.rs:406-520 CPU helpers;
 * cuda/fused_permute_peval.cuh; wrapper.cu:1824-1841; almost-goldilocks forms
 * cuda_almost_goldilocks/almost_partial_eval.cuh, almost_fused_permute_peval.cuh).
 * field 0: Goldilocks (Ext2 X^2 - 7), 1: almost-Goldilocks (Ext2 X^2 - 3).
 * ====================================================================== */
typedef struct { u64 c0, c1; } fe2;
static u64 f_add(int f, u64 a, u64 b) { return f ? agl_add(a, b) : gl_add(gl_canon(a), gl_canon(b)); }
static u64 f_sub(int f, u64 a, u64 b) { return f ? agl_sub(a, b) : gl_sub(gl_canon(a), gl_canon(b)); }
static u64 f_mul(int f, u64 a, u64 b) { return f ? agl_mul(a, b) : gl_mul(a, b); }
static u64 f_canon(int f, u64 a) { return f ? agl_canon(a) : gl_canon(a); }
static fe2 fe2_mul(int f, fe2 a, fe2 b) {
    fe2 r;
    u64 w = f ? 3 : 7;
    r.c0 = f_add(f, f_mul(f, a.c0, b.c0), f_mul(f, w, f_mul(f, a.c1, b.c1)));
    r.c1 = f_add(f, f_mul(f, a.c0, b.c1), f_mul(f, a.c1, b.c0));
    return r;
}

/* fix the low m variables at base r: out[j] = in[2j] + r_i (in[2j+1] - in[2j]) per level */
void or_partial_eval_base(int field, const u64 *evals, int log_n, const u64 *r, int m, u64 *out) {
    size_t sz = (size_t)1 << log_n;
    u64 *d = (u64 *)malloc(sz * 8);
    for (size_t k = 0; k < sz; k++) d[k] = f_canon(field, evals[k]);
    for (int i = 0; i < m; i++) {
        size_t half = sz / 2;
        for (size_t j = 0; j < half; j++)
            d[j] = f_add(field, d[2 * j], f_mul(field, r[i], f_sub(field, d[2 * j + 1], d[2 * j])));
        sz = half;
    }
    for (size_t k = 0; k < sz; k++) out[k] = f_canon(field, d[k]);
    free(d);
}

/* the same at Ext2 r (m >= 1): the first level mixed, then Ext2 levels; out: 2^(log_n-m) Ext2 */
void or_partial_eval_ext2(int field, const u64 *evals, int log_n, const u64 *r, int m, u64 *out) {
    size_t sz = (size_t)1 << log_n;
    fe2 *d = (fe2 *)malloc(sizeof(fe2) * (sz / 2 + 1));
    size_t half = sz / 2;
    for (size_t j = 0; j < half; j++) {
        u64 a = f_canon(field, evals[2 * j]), b = f_canon(field, evals[2 * j + 1]);
        u64 diff = f_sub(field, b, a);
        d[j].c0 = f_add(field, a, f_mul(field, r[0], diff));
        d[j].c1 = f_mul(field, r[1], diff);
    }
    sz = half;
    for (int i = 1; i < m; i++) {
        fe2 ri = {r[2 * i], r[2 * i + 1]};
        half = sz / 2;
        for (size_t j = 0; j < half; j++) {
            fe2 a = d[2 * j], b = d[2 * j + 1];
            fe2 diff = {f_sub(field, b.c0, a.c0), f_sub(field, b.c1, a.c1)};
            fe2 t = fe2_mul(field, ri, diff);
            d[j].c0 = f_add(field, a.c0, t.c0);
            d[j].c1 = f_add(field, a.c1, t.c1);
        }
        sz = half;
    }
    for (size_t k = 0; k < sz; k++) {
        out[2 * k] = f_canon(field, d[k].c0);
        out[2 * k + 1] = f_canon(field, d[k].c1);
    }
    free(d);
}

/* out[new] = in[old], old bit inv[k] <- new bit k  (wrapper.cu:1824-1841) */
void or_bit_permute(const u64 *in, u64 *out, const int *inv, int n_bits) {
    size_t total = (size_t)1 << n_bits;
    for (size_t nw = 0; nw < total; nw++) {
        size_t old = 0;
        for (int k = 0; k < n_bits; k++)
            if ((nw >> k) & 1) old |= (size_t)1 << inv[k];
        out[nw] = in[old];
    }
}

/* out[j] = sum_{b < 2^m} evals[lo[i & (2^half-1)] | hi[i >> half]] eq[b], i = j 2^m + b
 * (fused_permute_peval.cuh), for j < 2^(n-m) */
void or_fused_permute_peval(int field, const u64 *evals, int n, int m, int half, const u64 *eq, const uint32_t *lo,
                            const uint32_t *hi, u64 *out) {
    size_t outs = (size_t)1 << (n - m), inner = (size_t)1 << m, lo_mask = ((size_t)1 << half) - 1;
    for (size_t j = 0; j < outs; j++) {
        u64 a0 = 0, a1 = 0;
        for (size_t b = 0; b < inner; b++) {
            size_t i = (j << m) + b;
            u64 v = f_canon(field, evals[lo[i & lo_mask] | hi[i >> half]]);
            a0 = f_add(field, a0, f_mul(field, v, eq[2 * b]));
            a1 = f_add(field, a1, f_mul(field, v, eq[2 * b + 1]));
        }
        out[2 * j] = f_canon(field, a0);
        out[2 * j + 1] = f_canon(field, a1);
    }
}

/* ======================================================================
 * Ajtai: ChaCha8 matrix PRG (cuda_almost_goldilocks/ajtai_chacha8.cuh:60-178)
 * and the wide commitment (ajtai.cuh:216-275, ajtai_cpu_reference.cuh:57-186)
 * ====================================================================== */
#define ROTL32(x, n) (((x) << (n)) | ((x) >> (32 - (n))))
#define QR(a, b, c, d)                                                                              \
    do {                                                                                           \
        a += b; d ^= a; d = ROTL32(d, 16);                                                         \
        c += d; b ^= c; b = ROTL32(b, 12);                                                         \
        a += b; d ^= a; d = ROTL32(d, 8);                                                          \
        c += d; b ^= c; b = ROTL32(b, 7);                                                          \
    } while (0)

void or_chacha8_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3], uint32_t out[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                      key[4],      key[5],      key[6],      key[7],      counter, nonce[0], nonce[1], nonce[2]};
    uint32_t x[16];
    memcpy(x, s, sizeof(x));
    for (int dr = 0; dr < 4; dr++) {
        QR(x[0], x[4], x[8], x[12]);
        QR(x[1], x[5], x[9], x[13]);
        QR(x[2], x[6], x[10], x[14]);
        QR(x[3], x[7], x[11], x[15]);
        QR(x[0], x[5], x[10], x[15]);
        QR(x[1], x[6], x[11], x[12]);
        QR(x[2], x[7], x[8], x[13]);
        QR(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}

/* 8 coefficients for (row, j, block): accept the block's 8 words if all < q, else
 * scan counters block + 8k in order keeping words < q (ajtai_chacha8.cuh:115-178). */
static void prg_block(const uint32_t key[8], uint32_t row, u64 j, uint32_t blk, u64 out[8]) {
    uint32_t nonce[3] = {row, (uint32_t)(j & 0xFFFFFFFFu), (uint32_t)(j >> 32)};
    uint32_t buf[16];
    int written = 0;
    for (int k = 0; k < 8; k++) out[k] = 0;
    for (uint32_t retry = 0; retry < 16 && written < 8; retry++) {
        or_chacha8_block(key, blk + retry * 8u, nonce, buf);
        for (int k = 0; k < 8 && written < 8; k++) {
            u64 s = ((u64)buf[2 * k + 1] << 32) | buf[2 * k];
            if (s < AGL_Q) out[written++] = s;
        }
    }
}

void or_ajtai_ring_elem(const uint32_t key[8], uint32_t row, u64 j, u64 out[64]) {
    for (uint32_t b = 0; b < 8; b++) prg_block(key, row, j, b, out + 8 * b);
}

/* c[i][r] = sum_j sum_l sign * M_ij[(r - l) mod 64] * z_j[l], sign = -1 when l > r. */
void or_ajtai_commit_wide(const uint32_t key[8], const u64 *z, u64 N, u64 col_offset, int row_lo, int nrows,
                          u64 *out) {
    u64 M[64];
    for (int i = 0; i < nrows; i++) {
        u64 acc[64];
        memset(acc, 0, sizeof(acc));
        for (u64 j = 0; j < N; j++) {
            or_ajtai_ring_elem(key, (uint32_t)(row_lo + i), j + col_offset, M);
            const u64 *zj = z + j * 64;
            for (int r = 0; r < 64; r++) {
                u64 a = acc[r];
                for (int l = 0; l < 64; l++) {
                    u64 prod = agl_mul(M[(r - l) & 63], zj[l]);
                    a = (l <= r) ? agl_add(a, prod) : agl_sub(a, prod);
                }
                acc[r] = a;
            }
        }
        memcpy(out + (size_t)i * 64, acc, sizeof(acc));
    }
}

typedef struct { const uint32_t *key; int row_lo; u64 N; u64 *M; } ajtai_m_ctx;
static void ajtai_m_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    ajtai_m_ctx *c = (ajtai_m_ctx *)ctx;
    for (size_t k = lo; k < hi; k++)
        or_ajtai_ring_elem(c->key, (uint32_t)(c->row_lo + (int)(k / c->N)), k % c->N, c->M + k * 64);
}
typedef struct { const u64 *M; const uint8_t *z8; u64 N; int nrows; u64 *out; } ajtai_w_ctx;
static void ajtai_witness_range(void *ctx, size_t lo, size_t hi, int part) {
    (void)part;
    ajtai_w_ctx *c = (ajtai_w_ctx *)ctx;
    u64 N = c->N;
    for (size_t b = lo; b < hi; b++) {
        const uint8_t *zb = c->z8 + b * N * 64;
        for (int i = 0; i < c->nrows; i++) {
            /* positive and negative parts accumulated exactly in 128 bits:
             * each product < 2^72, at most N*64 <= 2^26 terms per coefficient */
            for (int r = 0; r < 64; r++) {
                u128 pos = 0, neg = 0;
                for (u64 j = 0; j < N; j++) {
                    const u64 *Mij = c->M + ((size_t)i * N + j) * 64;
                    const uint8_t *zj = zb + j * 64;
                    for (int l = 0; l <= r; l++) pos += (u128)Mij[r - l] * zj[l];
                    for (int l = r + 1; l < 64; l++) neg += (u128)Mij[r - l + 64] * zj[l];
                }
                u64 pm = (u64)(pos % AGL_Q), nm = (u64)(neg % AGL_Q);
                c->out[(b * (size_t)c->nrows + i) * 64 + r] = agl_sub(pm, nm);
            }
        }
    }
}
/* witnesses split over the host threads (one witness per part at least) */
void or_ajtai_commit_u8_batch(const uint32_t key[8], const uint8_t *z8, u64 N, int B, int row_lo, int nrows,
                              u64 *out) {
    u64 *M = (u64 *)malloc(sizeof(u64) * (size_t)nrows * N * 64);
    ajtai_m_ctx mc = {key, row_lo, N, M};
    par_for((size_t)nrows * N, 64, ajtai_m_range, &mc);
    ajtai_w_ctx wc = {M, z8, N, nrows, out};
    par_for((size_t)B, 1, ajtai_witness_range, &wc);
    free(M);
}

/* ======================================================================
 * Monolith-12 (goldilocks-cuda-rs/src/cpu_monolith.rs:13-139): concrete = circulant MDS with
 * first row MO_C plus round constants, fully reduced; bars = the byte-wise chi-like S-box on the
 * first 4 limbs; bricks = s[i] += s[i-1]^2 for i = 11 .. 1 (with the old s[i-1]).
 * The round constants are the published Monolith-64 ones (LOOKUP_BITS = 8).
 * ====================================================================== */
static const u64 MO_C[12] = {7, 23, 8, 26, 13, 10, 9, 7, 6, 22, 21, 8};
static const u64 MO_RC[7][12] = {
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
    {13596126580325903823ull, 5676126986831820406ull, 11349149288412960427ull, 3368797843020733411ull,
     16240671731749717664ull, 9273190757374900239ull, 14446552112110239438ull, 4033077683985131644ull,
     4291229347329361293ull, 13231607645683636062ull, 1383651072186713277ull, 8898815177417587567ull},
    {2383619671172821638ull, 6065528368924797662ull, 16737578966352303081ull, 2661700069680749654ull,
     7414030722730336790ull, 18124970299993404776ull, 9169923000283400738ull, 15832813151034110977ull,
     16245117847613094506ull, 11056181639108379773ull, 10546400734398052938ull, 8443860941261719174ull},
    {15799082741422909885ull, 13421235861052008152ull, 15448208253823605561ull, 2540286744040770964ull,
     2895626806801935918ull, 8644593510196221619ull, 17722491003064835823ull, 5166255496419771636ull,
     1015740739405252346ull, 4400043467547597488ull, 5176473243271652644ull, 4517904634837939508ull},
    {18341030605319882173ull, 13366339881666916534ull, 6291492342503367536ull, 10004214885638819819ull,
     4748655089269860551ull, 1520762444865670308ull, 8393589389936386108ull, 11025183333304586284ull,
     5993305003203422738ull, 458912836931247573ull, 5947003897778655410ull, 17184667486285295106ull},
    {15710528677110011358ull, 8929476121507374707ull, 2351989866172789037ull, 11264145846854799752ull,
     14924075362538455764ull, 10107004551857451916ull, 18325221206052792232ull, 16751515052585522105ull,
     15305034267720085905ull, 15639149412312342017ull, 14624541102106656564ull, 3542311898554959098ull},
    {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
};

static u64 mo_bar(u64 x) {
    u64 l1 = ((~x & 0x8080808080808080ull) >> 7) | ((~x & 0x7F7F7F7F7F7F7F7Full) << 1);
    u64 l2 = ((x & 0xC0C0C0C0C0C0C0C0ull) >> 6) | ((x & 0x3F3F3F3F3F3F3F3Full) << 2);
    u64 l3 = ((x & 0xE0E0E0E0E0E0E0E0ull) >> 5) | ((x & 0x1F1F1F1F1F1F1F1Full) << 3);
    u64 t = x ^ (l1 & l2 & l3);
    return ((t & 0x8080808080808080ull) >> 7) | ((t & 0x7F7F7F7F7F7F7F7Full) << 1);
}

static void mo_concrete(u64 s[12], int round) {
    u64 out[12];
    for (int r = 0; r < 12; r++) {
        u128 acc = MO_RC[round][r];
        for (int c = 0; c < 12; c++) acc += (u128)s[c] * MO_C[(c - r + 12) % 12];
        out[r] = gl_reduce128(acc);
    }
    memcpy(s, out, sizeof(out));
}

void or_monolith_permute(u64 s[12]) {
    for (int i = 0; i < 12; i++) s[i] = gl_canon(s[i]);
    mo_concrete(s, 0);
    for (int r = 1; r <= 6; r++) {
        for (int i = 0; i < 4; i++) s[i] = mo_bar(s[i]);
        for (int i = 11; i >= 1; i--) s[i] = gl_add(s[i], gl_mul(s[i - 1], s[i - 1]));
        mo_concrete(s, r);
    }
}

static void mo_tree_up(u64 *tree, size_t leaves) {
    size_t off = 0, nodes = leaves;
    while (nodes > 1) {
        u64 *layer = tree + 4 * off, *up = layer + 4 * nodes;
        for (size_t j = 0; j < nodes / 2; j++) {
            u64 st[12] = {0};
            memcpy(st, layer + 8 * j, 8 * sizeof(u64));
            or_monolith_permute(st);
            memcpy(up + 4 * j, st, 4 * sizeof(u64));
        }
        off += nodes;
        nodes /= 2;
    }
}

void or_monolith_tree_gl(const u64 *cw, size_t leaves, u64 *tree) {
    for (size_t i = 0; i < leaves; i++) {
        u64 st[12] = {0};
        st[0] = cw[2 * i];
        st[1] = cw[2 * i + 1];
        or_monolith_permute(st);
        memcpy(tree + 4 * i, st, 4 * sizeof(u64));
    }
    mo_tree_up(tree, leaves);
}

void or_monolith_tree_ext2(const u64 *cw, size_t leaves, u64 *tree) {
    for (size_t i = 0; i < leaves; i++) {
        u64 st[12] = {0};
        memcpy(st, cw + 4 * i, 4 * sizeof(u64));
        or_monolith_permute(st);
        memcpy(tree + 4 * i, st, 4 * sizeof(u64));
    }
    mo_tree_up(tree, leaves);
}
