// Basefold polynomial commitment on the device: host-side objects shared by the
// drivers (basefold.cu) and the eq-table kernels (eq.cu).
#pragma once
#include <vector>

#include "common.cuh"
#include "gl.cuh"

namespace gb {

// eq(r, x) over {0,1}^n, variable i <-> bit i of x; out has 2^n entries (Ext2 if EXT).
// r is on the device (n values, Ext2 pairs if EXT).  Launches only.
int eq_table(const u64* d_r, int n, bool ext, u64* d_out);

// Folding table of BasefoldTable::generate (goldilocks-cuda-rs/src/basefold.rs:270-362):
// level i has 2^(num_vars + log_rate - i - 1) (point, weight) entries.
struct BfTable {
    int num_vars = 0, log_rate = 0, num_rounds = 0;
    uint64_t seed = 0;
    std::vector<size_t> level_offsets;  // in entries
    u64* d_entries = nullptr;           // [total][2]
    size_t total = 0;
};

// Device-resident commitment (BasefoldCommitment, basefold.rs:369-427).  evals are
// kept in natural order (the reference keeps their bit-reversed copy and reverses
// it again at open time).
struct BfCommitment {
    int num_vars = 0, log_rate = 0;
    u64* d_evals = nullptr;     // 2^n base field
    u64* d_codeword = nullptr;  // 2^(n+lr) base field
    u64* d_tree = nullptr;      // (2 * 2^(n+lr-1) - 1) digests
    u64 root[4] = {0, 0, 0, 0};
};

}  // namespace gb
