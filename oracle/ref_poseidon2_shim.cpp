// C entry points over the reference's own Goldilocks / Poseidon2 device code
// (cuda/goldilocks.cuh, cuda/extension.cuh, cuda/poseidon2.cuh) compiled for the
// host by oracle/Makefile: the headers carry host fallbacks for the 64x64
// multiply, and the __constant__ round-constant tables become host globals that
// this shim fills from the reference's own host copies (what poseidon2_init()
// does with cudaMemcpyToSymbol).  Test infrastructure: it pins the oracle's
// Poseidon2 to the reference's code path.
#include <cstring>
#include "poseidon2.cuh"

extern "C" {

void ref_poseidon2_init() {
    std::memcpy((void*)d_RC_EXT_8, h_RC_EXT_8, sizeof(h_RC_EXT_8));
    std::memcpy((void*)d_RC_INT, h_RC_INT, sizeof(h_RC_INT));
    std::memcpy((void*)d_DIAG_8, h_DIAG_8, sizeof(h_DIAG_8));
}

void ref_poseidon2_permute(uint64_t s[8]) {
    GoldilocksField st[8];
    for (int i = 0; i < 8; i++) st[i] = GoldilocksField(s[i]);
    poseidon2_permute_8(st);
    for (int i = 0; i < 8; i++) s[i] = canonicalize(st[i].value);
}

// The device field ops as compiled on the host (non-canonical outputs canonicalised).
uint64_t ref_gl_mul(uint64_t a, uint64_t b) { return canonicalize(gl_mul(GoldilocksField(a), GoldilocksField(b)).value); }
uint64_t ref_gl_add(uint64_t a, uint64_t b) { return canonicalize(gl_add(GoldilocksField(a), GoldilocksField(b)).value); }
uint64_t ref_gl_sub(uint64_t a, uint64_t b) { return canonicalize(gl_sub(GoldilocksField(a), GoldilocksField(b)).value); }
void ref_ext2_mul(const uint64_t a[2], const uint64_t b[2], uint64_t out[2]) {
    GoldilocksExt2 r = ext2_mul(GoldilocksExt2(a[0], a[1]), GoldilocksExt2(b[0], b[1]));
    out[0] = canonicalize(r.c[0].value);
    out[1] = canonicalize(r.c[1].value);
}

}
