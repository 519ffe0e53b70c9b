// Device-side Fiat-Shamir challengers: batches of independent duplex sponges over Poseidon2
// (width 8, rate 4), the reference ABI of goldilocks-cuda-rs (src/ffi.rs:314-372, wrapper.cu:1004-1110,
// semantics of cuda/challenger.cuh:37-222):
//   observe: invalidate pending outputs, append to the input buffer, duplex when it holds 4;
//   duplex:  the input buffer overwrites the rate part (unused rate slots become 0), permute,
//            the rate part goes to the output buffer in reverse order (4 outputs);
//   sample:  duplex if no output is pending, then pop the last output.
// One thread per challenger.  The state layout is the reference's (8 + 4 + 4 field words, two
// int counters: 136 bytes), so that states copied to the host keep their meaning; the words
// are kept canonical.
#include "../../include/goldilocks_cuda_wrapper.h"
#include "common.cuh"
#include "poseidon2.cuh"

namespace gb {

struct ChallengerState {
    u64 sponge[8];
    u64 input[4];
    u64 output[4];
    int input_count;
    int output_count;
};
static_assert(sizeof(ChallengerState) == 136, "challenger state layout");

__device__ __forceinline__ void ch_duplex(ChallengerState* s) {
    u64 st[8];
#pragma unroll
    for (int i = 0; i < 4; i++) st[i] = i < s->input_count ? s->input[i] : 0;
#pragma unroll
    for (int i = 4; i < 8; i++) st[i] = s->sponge[i];
    s->input_count = 0;
    p2_permute(st);
#pragma unroll
    for (int i = 0; i < 8; i++) s->sponge[i] = gl_canon(st[i]);
#pragma unroll
    for (int i = 0; i < 4; i++) s->output[3 - i] = s->sponge[i];
    s->output_count = 4;
}

__device__ __forceinline__ void ch_observe(ChallengerState* s, u64 v) {
    s->output_count = 0;
    s->input[s->input_count++] = gl_canon(v);
    if (s->input_count == 4) ch_duplex(s);
}

__device__ __forceinline__ u64 ch_sample(ChallengerState* s) {
    if (s->output_count == 0) ch_duplex(s);
    return s->output[--s->output_count];
}

// op: 0 init, 1 observe `count` values each, 2 sample `count` values each
__global__ void challenger_kernel(ChallengerState* __restrict__ states, const u64* __restrict__ in,
                                  u64* __restrict__ out, int count, int n, int op) {
    int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    ChallengerState s = states[idx];
    if (op == 0) {
        for (int i = 0; i < 8; i++) s.sponge[i] = 0;
        for (int i = 0; i < 4; i++) s.input[i] = s.output[i] = 0;
        s.input_count = s.output_count = 0;
    } else if (op == 1) {
        for (int k = 0; k < count; k++) ch_observe(&s, in[(size_t)idx * count + k]);
    } else {
        for (int k = 0; k < count; k++) out[(size_t)idx * count + k] = ch_sample(&s);
    }
    states[idx] = s;
}

static int challenger_run(void* d_states, const u64* in, u64* out, int count, int n, int op, const char* name) {
    if (!d_states || n < 0 || count < 0 || (op == 1 && count && n && !in) || (op == 2 && count && n && !out))
        return GB_EINVAL;
    if (n == 0) return GB_OK;
    challenger_kernel<<<grid_for((size_t)n, 128), 128, 0, stream()>>>((ChallengerState*)d_states, in, out, count, n, op);
    return check_launch(name);
}

}  // namespace gb

using namespace gb;

extern "C" {

int challenger_state_size(void) { return (int)sizeof(ChallengerState); }

int challenger_alloc_states(void** d_states, int n) {
    if (!d_states || n <= 0) return GB_EINVAL;
    return cudaMalloc(d_states, (size_t)n * sizeof(ChallengerState)) == cudaSuccess ? 0 : GB_ECUDA;
}

int challenger_init_states(void* d_states, int n) {
    return challenger_run(d_states, nullptr, nullptr, 0, n, 0, "challenger_init_states");
}

int challenger_observe_ffi(void* d_states, const uint64_t* d_values, int n) {
    return challenger_run(d_states, d_values, nullptr, 1, n, 1, "challenger_observe_ffi");
}

int challenger_observe_slice_ffi(void* d_states, const uint64_t* d_values, int count, int n) {
    return challenger_run(d_states, d_values, nullptr, count, n, 1, "challenger_observe_slice_ffi");
}

int challenger_observe_ext2_ffi(void* d_states, const uint64_t* d_values, int n) {
    return challenger_run(d_states, d_values, nullptr, 2, n, 1, "challenger_observe_ext2_ffi");
}

int challenger_sample_ffi(void* d_states, uint64_t* d_outputs, int n) {
    return challenger_run(d_states, nullptr, d_outputs, 1, n, 2, "challenger_sample_ffi");
}

int challenger_sample_array_ffi(void* d_states, uint64_t* d_outputs, int count, int n) {
    return challenger_run(d_states, nullptr, d_outputs, count, n, 2, "challenger_sample_array_ffi");
}

int challenger_sample_ext2_ffi(void* d_states, uint64_t* d_outputs, int n) {
    return challenger_run(d_states, nullptr, d_outputs, 2, n, 2, "challenger_sample_ext2_ffi");
}

int challenger_sample_ext5_ffi(void* d_states, uint64_t* d_outputs, int n) {
    return challenger_run(d_states, nullptr, d_outputs, 5, n, 2, "challenger_sample_ext5_ffi");
}

int challenger_copy_state_to_host(void* h_state, const void* d_state) {
    cudaStream_t s = stream();
    if (cudaMemcpyAsync(h_state, d_state, sizeof(ChallengerState), cudaMemcpyDeviceToHost, s) != cudaSuccess) return -1;
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -1;
}

int challenger_copy_state_to_device(void* d_state, const void* h_state) {
    cudaStream_t s = stream();
    if (cudaMemcpyAsync(d_state, h_state, sizeof(ChallengerState), cudaMemcpyHostToDevice, s) != cudaSuccess) return -1;
    return cudaStreamSynchronize(s) == cudaSuccess ? 0 : -1;
}

}  // extern "C"
