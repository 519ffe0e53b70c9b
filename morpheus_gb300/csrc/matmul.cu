// Proof of one quantized matmul layer C = A B (A: M x K, B: K x N, int8-range values
// embedded in Goldilocks), the einsum step of the reference's DAG prover
// (zk-torch-3/src/basicblock/einsum.rs:807-1000) reduced to its field work:
//   1. embed A and B (v >= 0 -> v, v < 0 -> p + v) and commit both with Basefold (rate 1/2);
//   2. transcript "matmul" . master_seed . index . M . N . K . roots -> points r_i (log M Ext2
//      challenges) and r_j (log N);
//   3. partial evaluations a_k = sum_i eq(r_i, i) A[i][k], b_k = sum_j B[k][j] eq(r_j, j), so
//      that C~(r_i, r_j) = sum_k a_k b_k;
//   4. the degree-2 product sumcheck over the log K variables of k on (a, b) (Ext2 inputs,
//      CpuLinearSumcheckProverExt2 semantics) on the same transcript -> r_k;
//   5. open A at (r_k, r_i) and B at (r_j, r_k) (variable order = index bits, low first:
//      A[i][k] sits at i K + k, B[k][j] at k N + j), each on its own "bf-open" transcript
//      (master_seed, 8 index + 0 / 1); their evaluations equal the sumcheck's final values;
//   6. Ajtai commitment of the job's 2^16-coefficient witness, the first 2^16 entries of A
//      as bytes v + 128, under a resident key (rows of the almost-Goldilocks matrix).
#include <vector>

#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "../../include/goldilocks_cuda_wrapper.h"
#include "basefold.cuh"
#include "common.cuh"
#include "host_field.hpp"
#include "open_engine.cuh"

namespace gb {

constexpr int MM_WITNESS = 1 << 16;

__global__ void embed_i8_kernel(const int8_t* __restrict__ x, u64* __restrict__ out, size_t n) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    int v = x[t];
    out[t] = v >= 0 ? (u64)v : GL_P - (u64)(-v);
}

__global__ void i8_to_u8_kernel(const int8_t* __restrict__ x, uint8_t* __restrict__ out, size_t n) {
    size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (t >= n) return;
    out[t] = (uint8_t)((int)x[t] + 128);
}

// part[split][k] = sum_{i in split's rows} eq[i] A[i][k]  (Ext2 eq, base A; lazy sums, at most
// 4096 terms per split so the high parts stay small)
__global__ void pe_cols_kernel(const u64* __restrict__ A, const u64* __restrict__ eq, int M, int K, int rows_per_split,
                               u64* __restrict__ part) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    int split = blockIdx.y;
    if (k >= K) return;
    int i0 = split * rows_per_split, i1 = min(M, i0 + rows_per_split);
    glw s0 = glw_of(0), s1 = glw_of(0);
    for (int i = i0; i < i1; i++) {
        u64 x = __ldg(A + (size_t)i * K + k);
        u64 e0 = __ldg(eq + 2 * i), e1 = __ldg(eq + 2 * i + 1);
        s0 = glw_add(s0, gl_mul(e0, x));
        s1 = glw_add(s1, gl_mul(e1, x));
    }
    u64* o = part + ((size_t)split * K + k) * 2;
    o[0] = glw_reduce(s0);
    o[1] = glw_reduce(s1);
}

__global__ void pe_cols_sum_kernel(const u64* __restrict__ part, int splits, int K, u64* __restrict__ out) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    glw s0 = glw_of(0), s1 = glw_of(0);
    for (int s = 0; s < splits; s++) {
        s0 = glw_add(s0, part[((size_t)s * K + k) * 2]);
        s1 = glw_add(s1, part[((size_t)s * K + k) * 2 + 1]);
    }
    out[2 * k] = glw_reduce(s0);
    out[2 * k + 1] = glw_reduce(s1);
}

// out[k] = sum_j B[k][j] eq[j]: one warp per row k
__global__ void pe_rows_kernel(const u64* __restrict__ B, const u64* __restrict__ eq, int K, int N,
                               u64* __restrict__ out) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= K) return;
    const u64* row = B + (size_t)warp * N;
    glw s0 = glw_of(0), s1 = glw_of(0);
    for (int j = lane; j < N; j += 32) {
        u64 x = __ldg(row + j);
        s0 = glw_add(s0, gl_mul(__ldg(eq + 2 * j), x));
        s1 = glw_add(s1, gl_mul(__ldg(eq + 2 * j + 1), x));
    }
    u64 r0 = gl_warp_sum(glw_reduce(s0)), r1 = gl_warp_sum(glw_reduce(s1));
    if (lane == 0) {
        out[2 * warp] = r0;
        out[2 * warp + 1] = r1;
    }
}

static int log2_exact(int v) {
    if (v <= 0 || (v & (v - 1))) return -1;
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

size_t matmul_proof_len(int m, int n, int k, int q) {
    int lm = log2_exact(m), ln = log2_exact(n), lk = log2_exact(k);
    if (lm < 0 || ln < 0 || lk < 1) return 0;
    size_t sc = 2 + (size_t)lk * 3 * 2 + (size_t)lk * 2 + 4 + 2;
    return 8 + sc + gb_basefold_proof_len(lm + lk, 1, q) + gb_basefold_proof_len(lk + ln, 1, q) + 16 * 64;
}

size_t matmul_hbm_bytes(int m, int n, int k) {
    size_t a = (size_t)m * k, b = (size_t)k * n;
    return (a + b) * 130 + (a > b ? a : b) * 144 + ((size_t)8 << 20);
}

// Steps 1-4 and the Ajtai commitment of one job, on the calling thread's stream; on success the
// stream is idle and the two openings (A at (r_k, r_i), B at (r_j, r_k)) are returned as tasks with
// their commitments, for the caller to open and then destroy.
int matmul_prologue(void* table, void* ajtai_key, const u64 seed[2], int q, const gb_matmul_job* job,
                    std::vector<OpenTask>* tasks, std::vector<void*>* coms) {
    using namespace host;
    const int M = job->m, N = job->n, K = job->k;
    const int lm = log2_exact(M), ln = log2_exact(N), lk = log2_exact(K);
    if (!table || !ajtai_key || lm < 0 || ln < 0 || lk < 1 || lm + lk < 2 || lk + ln < 2 || lm + lk > 30 ||
        lk + ln > 30 || (size_t)M * K < (size_t)MM_WITNESS || !job->h_a || !job->h_b || !job->h_proof || q < 0) {
        set_error_msg("gb_prove_matmul: invalid job (M, N, K powers of two, M K >= 2^16, table and key set)");
        return GB_EINVAL;
    }
    {
        int rows = 0;
        uint64_t ring = 0;
        if (gb_ajtai_key_info(ajtai_key, nullptr, &rows, &ring) || rows != 16 || ring != MM_WITNESS / 64) {
            set_error_msg("gb_prove_matmul: the Ajtai key must hold 16 rows over 1024 ring columns");
            return GB_EINVAL;
        }
    }
    cudaStream_t s = stream();
    const size_t MK = (size_t)M * K, KN = (size_t)K * N;
    std::vector<void*> owned;
    auto dev = [&](size_t bytes, void** p) -> int {
        cudaError_t e = cudaMallocAsync(p, bytes < 16 ? 16 : bytes, s);
        if (e != cudaSuccess) {
            set_error("cudaMallocAsync", e);
            return GB_ECUDA;
        }
        owned.push_back(*p);
        return GB_OK;
    };
    auto cleanup = [&]() {
        for (void* p : owned) cudaFreeAsync(p, s);
    };
    int8_t *d_a8 = nullptr, *d_b8 = nullptr;
    u64 *d_A = nullptr, *d_B = nullptr, *d_ab = nullptr, *d_pt = nullptr, *d_eqm = nullptr, *d_eqn = nullptr,
        *d_part = nullptr, *d_aj = nullptr;
    uint8_t* d_w = nullptr;
    const int rps = 256;
    const int splits = (M + rps - 1) / rps;
    int rc = dev(MK, (void**)&d_a8);
    if (!rc) rc = dev(KN, (void**)&d_b8);
    if (!rc) rc = dev(MK * 8, (void**)&d_A);
    if (!rc) rc = dev(KN * 8, (void**)&d_B);
    if (!rc) rc = dev((size_t)K * 32, (void**)&d_ab);  // a | b, Ext2
    if (!rc) rc = dev((size_t)(lm + ln) * 16, (void**)&d_pt);
    if (!rc) rc = dev((size_t)M * 16, (void**)&d_eqm);
    if (!rc) rc = dev((size_t)N * 16, (void**)&d_eqn);
    if (!rc) rc = dev((size_t)splits * K * 16, (void**)&d_part);
    if (!rc) rc = dev(MM_WITNESS, (void**)&d_w);
    if (!rc) rc = dev(16 * 64 * 8, (void**)&d_aj);
    if (rc) {
        cleanup();
        return rc;
    }
    u64* out = job->h_proof;
    u64* roots = out;                              // A, B
    u64* claim = roots + 8;                        // 2
    u64* msgs = claim + 2;                         // lk x 3 x 2
    u64* chal = msgs + (size_t)lk * 6;             // lk x 2
    u64* finals = chal + (size_t)lk * 2;           // 2 x 2
    u64* fe = finals + 4;                          // 2
    u64* openA = fe + 2;
    u64* openB = openA + gb_basefold_proof_len(lm + lk, 1, q);
    u64* aj = openB + gb_basefold_proof_len(lk + ln, 1, q);

    void* comA = nullptr;
    void* comB = nullptr;
    auto finish = [&](int r) {
        cleanup();
        if (!r) {
            cudaError_t e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                set_error("cudaStreamSynchronize", e);
                r = GB_ECUDA;
            }
        }
        if (r) {
            if (comA) gb_basefold_commitment_destroy(comA);
            if (comB) gb_basefold_commitment_destroy(comB);
        }
        return r;
    };
#define MM_TRY(x)                    \
    do {                             \
        int _r = (x);                \
        if (_r) return finish(_r);   \
    } while (0)
#define MM_CUDA(x)                                 \
    do {                                           \
        cudaError_t _e = (x);                      \
        if (_e != cudaSuccess) {                   \
            set_error(#x, _e);                     \
            return finish(GB_ECUDA);               \
        }                                          \
    } while (0)

    // 1. inputs, embedding, Ajtai witness, commitments
    MM_CUDA(cudaMemcpyAsync(d_a8, job->h_a, MK, cudaMemcpyHostToDevice, s));
    MM_CUDA(cudaMemcpyAsync(d_b8, job->h_b, KN, cudaMemcpyHostToDevice, s));
    embed_i8_kernel<<<grid_for(MK, 256), 256, 0, s>>>(d_a8, d_A, MK);
    MM_TRY(check_launch("embed_i8_kernel"));
    embed_i8_kernel<<<grid_for(KN, 256), 256, 0, s>>>(d_b8, d_B, KN);
    MM_TRY(check_launch("embed_i8_kernel"));
    i8_to_u8_kernel<<<grid_for(MM_WITNESS, 256), 256, 0, s>>>(d_a8, d_w, MM_WITNESS);
    MM_TRY(check_launch("i8_to_u8_kernel"));
    MM_TRY(gb_ajtai_commit_u8_batched(ajtai_key, d_w, 1, d_aj));
    MM_CUDA(cudaMemcpyAsync(aj, d_aj, 16 * 64 * 8, cudaMemcpyDeviceToHost, s));
    MM_TRY(gb_basefold_commit(d_A, nullptr, lm + lk, 1, &comA, roots));
    MM_TRY(gb_basefold_commit(d_B, nullptr, lk + ln, 1, &comB, roots + 4));

    // 2. transcript -> r_i, r_j
    gb_transcript t;
    gb_transcript_new(&t, "matmul");
    tr_append_ext2(&t, "", E2{canon(seed[0]), canon(seed[1])});
    tr_append_u64(&t, "", job->index);
    tr_append_u64(&t, "", (u64)M);
    tr_append_u64(&t, "", (u64)N);
    tr_append_u64(&t, "", (u64)K);
    for (int w = 0; w < 8; w++) tr_append_u64(&t, "", roots[w]);
    std::vector<u64> pt(2 * (lm + ln));
    for (int v = 0; v < lm + ln; v++) {
        E2 c = tr_challenge_ext2(&t, "");
        pt[2 * v] = c.c0;
        pt[2 * v + 1] = c.c1;
    }
    MM_CUDA(cudaMemcpyAsync(d_pt, pt.data(), pt.size() * 8, cudaMemcpyHostToDevice, s));
    MM_TRY(eq_table(d_pt, lm, true, d_eqm));
    MM_TRY(eq_table(d_pt + 2 * lm, ln, true, d_eqn));

    // 3. partial evaluations
    pe_cols_kernel<<<dim3((unsigned)((K + 127) / 128), (unsigned)splits), 128, 0, s>>>(d_A, d_eqm, M, K, rps, d_part);
    MM_TRY(check_launch("pe_cols_kernel"));
    pe_cols_sum_kernel<<<grid_for(K, 128), 128, 0, s>>>(d_part, splits, K, d_ab);
    MM_TRY(check_launch("pe_cols_sum_kernel"));
    pe_rows_kernel<<<grid_for((size_t)K * 32, 256), 256, 0, s>>>(d_B, d_eqn, K, N, d_ab + 2 * (size_t)K);
    MM_TRY(check_launch("pe_rows_kernel"));

    // 4. sumcheck over k; the claim is s_0(0) + s_0(1)
    MM_TRY(gb_sumcheck_prove_ext2_polys(&t, lk, 2, d_ab, nullptr, msgs, chal, finals, fe));
    {
        E2 c = e2add(E2{msgs[0], msgs[1]}, E2{msgs[2], msgs[3]});
        claim[0] = c.c0;
        claim[1] = c.c1;
    }

    // 5. openings
    std::vector<u64> ptA(2 * (lk + lm)), ptB(2 * (ln + lk));
    for (int v = 0; v < lk; v++) {
        ptA[2 * v] = chal[2 * v];
        ptA[2 * v + 1] = chal[2 * v + 1];
        ptB[2 * (ln + v)] = chal[2 * v];
        ptB[2 * (ln + v) + 1] = chal[2 * v + 1];
    }
    for (int v = 0; v < lm; v++) {
        ptA[2 * (lk + v)] = pt[2 * v];
        ptA[2 * (lk + v) + 1] = pt[2 * v + 1];
    }
    for (int v = 0; v < ln; v++) {
        ptB[2 * v] = pt[2 * (lm + v)];
        ptB[2 * v + 1] = pt[2 * (lm + v) + 1];
    }
    {
        int r = finish(GB_OK);
        if (r) return r;
    }
    for (int which = 0; which < 2; which++) {
        OpenTask t;
        t.com = (BfCommitment*)(which ? comB : comA);
        t.point = which ? ptB : ptA;
        gb_transcript_new(&t.t, "bf-open");
        tr_append_ext2(&t.t, "", E2{canon(seed[0]), canon(seed[1])});
        tr_append_u64(&t.t, "", 8 * job->index + (u64)which);
        t.proof = which ? openB : openA;
        tasks->push_back(std::move(t));
        coms->push_back(which ? comB : comA);
    }
    return GB_OK;
#undef MM_TRY
#undef MM_CUDA
}

int prove_matmul(void* table, void* ajtai_key, const u64 seed[2], int q, const gb_matmul_job* job) {
    std::vector<OpenTask> tasks;
    std::vector<void*> coms;
    int rc = matmul_prologue(table, ajtai_key, seed, q, job, &tasks, &coms);
    if (rc) return rc;
    return open_tasks_inline(table, q, tasks, coms);
}

}  // namespace gb

using namespace gb;

extern "C" {

size_t gb_matmul_proof_len(int m, int n, int k, int num_queries) { return matmul_proof_len(m, n, k, num_queries); }

size_t gb_matmul_hbm_bytes(int m, int n, int k) { return matmul_hbm_bytes(m, n, k); }

int gb_prove_matmul(void* table, void* ajtai_key, const uint64_t master_seed[2], int num_queries,
                    const gb_matmul_job* job) {
    if (!master_seed || !job) return GB_EINVAL;
    return prove_matmul(table, ajtai_key, master_seed, num_queries, job);
}

}  // extern "C"
