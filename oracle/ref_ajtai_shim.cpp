// C entry points over the reference's own host-compilable Ajtai CPU reference
// (cuda_almost_goldilocks/ajtai_cpu_reference.cuh, ajtai_chacha8.cuh), compiled
// from the reference tree by oracle/Makefile into oracle/_ref/.  Test
// infrastructure: used only to pin the oracle's Ajtai restatement.
#include "ajtai_cpu_reference.cuh"

extern "C" {

void ref_chacha8_block(const uint32_t key[8], uint32_t counter, const uint32_t nonce[3], uint32_t out[16]) {
    chacha8_block(key, counter, nonce, out);
}

void ref_ring_elem(const uint32_t key[8], int row, uint64_t j, uint64_t out[64]) {
    auto r = ajtai_cpu::cpu_prg_ring_elem<64>(key, row, j);
    for (int i = 0; i < 64; i++) out[i] = r[i];
}

// Wide commitment composed from the reference's PRG and naive negacyclic ring
// product: c_i = sum_j M[i, j + col_offset] * z_j (ajtai_cpu_reference.cuh:57-160).
void ref_commit_wide(const uint32_t key[8], const uint64_t* z, uint64_t N, uint64_t col_offset,
                     int row_lo, int nrows, uint64_t* out) {
    for (int i = 0; i < nrows; i++) {
        ajtai_cpu::Ring<64> acc{};
        for (uint64_t j = 0; j < N; j++) {
            auto M = ajtai_cpu::cpu_prg_ring_elem<64>(key, row_lo + i, j + col_offset);
            ajtai_cpu::Ring<64> zj;
            for (int l = 0; l < 64; l++) zj[l] = z[j * 64 + l];
            auto prod = ajtai_cpu::cpu_ring_mul<64>(M, zj);
            for (int r = 0; r < 64; r++) acc[r] = ajtai_cpu::h_add(acc[r], prod[r]);
        }
        for (int r = 0; r < 64; r++) out[i * 64 + r] = ajtai_cpu::h_canon(acc[r]);
    }
}

// Binary commitment for KAPPA = 42 rows (cpu_ajtai_commit<64, 42>).
void ref_commit_binary(const uint32_t key[8], const uint64_t* z_bits, uint64_t N, uint64_t* out) {
    auto c = ajtai_cpu::cpu_ajtai_commit<64, 42>(key, z_bits, N);
    for (int i = 0; i < 42; i++)
        for (int r = 0; r < 64; r++) out[i * 64 + r] = c[i][r];
}

}
