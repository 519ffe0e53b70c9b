// Shared runtime plumbing for the C-ABI library: the launch stream, error
// reporting, launch-size helpers.
//
// Stream model: the reference wrappers launch on the per-thread default stream
// (both crates build with --default-stream per-thread, goldilocks-cuda-rs/build.rs:115-126).
// Here every launch goes to gb::stream(), which is the per-thread default stream
// unless the calling thread selected another one with gb_set_stream().
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

namespace gb {

cudaStream_t stream();
void set_error(const char* where, cudaError_t e);
void set_error_msg(const std::string& msg);
int num_sms();
// Pinned host staging of the calling thread: slot 0 sumcheck, slot 1 Basefold, slot 2 staged copies.
constexpr int PINNED_SLOTS = 3;
uint64_t* thread_pinned(int slot, size_t words);

// Return-code conventions of the reference C ABI (goldilocks-cuda-rs/cuda/wrapper.cu):
// 0 ok, -1 CUDA error; -2 invalid argument and -3 unsupported option are this
// library's refinements of the reference's -1 / -3.
constexpr int GB_OK = 0;
constexpr int GB_ECUDA = -1;
constexpr int GB_EINVAL = -2;
constexpr int GB_EUNSUPPORTED = -3;

void count_launch();

inline int check_launch(const char* where) {
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(where, e);
        return GB_ECUDA;
    }
    return GB_OK;
}

inline int sync_stream(const char* where) {
    cudaError_t e = cudaStreamSynchronize(stream());
    if (e != cudaSuccess) {
        set_error(where, e);
        return GB_ECUDA;
    }
    return GB_OK;
}

inline unsigned grid_for(size_t work, int block, int per_thread = 1) {
    size_t g = (work + (size_t)block * per_thread - 1) / ((size_t)block * per_thread);
    if (g < 1) g = 1;
    if (g > 0x7fffffffull) g = 0x7fffffffull;
    return (unsigned)g;
}

#define GB_CUDA_TRY(call)                        \
    do {                                         \
        cudaError_t _e = (call);                 \
        if (_e != cudaSuccess) {                 \
            ::gb::set_error(#call, _e);          \
            return ::gb::GB_ECUDA;               \
        }                                        \
    } while (0)

#define GB_LAUNCH_CHECK(name)                    \
    do {                                         \
        int _rc = ::gb::check_launch(name);      \
        if (_rc) return _rc;                     \
    } while (0)

}  // namespace gb
