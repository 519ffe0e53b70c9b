// Runtime plumbing of the C ABI: stream selection, error strings, the memory and
// device entry points (goldilocks-cuda-rs/src/ffi.rs:11-26, :306-309), batch
// field ops and host transcript helpers.
#include <atomic>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/almost_goldilocks_cuda_wrapper.h"
#include "../../include/goldilocks_cuda_wrapper.h"
#include "common.cuh"
#include "host_field.hpp"
#include <nvtx3/nvToolsExt.h>

namespace gb {

static thread_local cudaStream_t t_stream = cudaStreamPerThread;
static thread_local std::string t_err;

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

// The stream-ordered pool behind cudaMallocAsync defaults to a release threshold of 0: it
// hands its memory back to the driver at every synchronisation, and the next allocation maps
// it again.  Like the reference (almost-goldilocks-cuda-rs/cuda/wrapper.cu:151-166), let the
// pool keep what it holds; cuda_pool_trim releases it explicitly.  Done once per device, on
// the first launch-stream lookup with that device current.
static void keep_pool_memory() {
    constexpr int MAX_DEVICES = 64;
    static thread_local uint64_t t_done = 0;  // devices this thread has seen configured
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return;
    if (t_done & (1ull << dev)) return;
    static std::mutex mu;
    static bool done[MAX_DEVICES] = {};
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!done[dev]) {
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
                uint64_t thr = UINT64_MAX;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
            }
            done[dev] = true;
        }
    }
    t_done |= 1ull << dev;
}

cudaStream_t stream() {
    keep_pool_memory();
    return t_stream;
}

// Pinned host staging owned by the calling thread, one buffer per slot, released when the
// thread exits (worker threads of the prover service come and go).
namespace {
struct PinnedSlots {
    uint64_t* buf[PINNED_SLOTS] = {};
    size_t cap[PINNED_SLOTS] = {};
    ~PinnedSlots() {
        for (int i = 0; i < PINNED_SLOTS; i++)
            if (buf[i]) cudaFreeHost(buf[i]);
    }
};
}  // namespace

uint64_t* thread_pinned(int slot, size_t words) {
    static thread_local PinnedSlots t;
    if (slot < 0 || slot >= PINNED_SLOTS) return nullptr;
    if (words > t.cap[slot]) {
        if (t.buf[slot]) cudaFreeHost(t.buf[slot]);
        size_t c = words < 8192 ? 8192 : words;
        if (cudaMallocHost(&t.buf[slot], c * 8) != cudaSuccess) {
            t.buf[slot] = nullptr;
            t.cap[slot] = 0;
            return nullptr;
        }
        t.cap[slot] = c;
    }
    return t.buf[slot];
}

void set_error(const char* where, cudaError_t e) {
    t_err = std::string(where) + ": " + cudaGetErrorString(e);
}
void set_error_msg(const std::string& msg) { t_err = msg; }

int num_sms() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 148;
    return n;
}

// ---------------------------------------------------------------------------
// batch field kernels
// ---------------------------------------------------------------------------
template <int OP>
__global__ void gl_batch_kernel(const u64* __restrict__ a, const u64* __restrict__ b, u64* __restrict__ r, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    u64 x = a[i];
    u64 y = (OP == 3) ? 0 : b[i];
    u64 z;
    if (OP == 0) z = gl_add(x, y);
    else if (OP == 1) z = gl_sub(x, y);
    else if (OP == 2) z = gl_mul(x, y);
    else z = gl_inv(x);
    r[i] = z;
}

template <int OP>
__global__ void e2_batch_kernel(const u64* __restrict__ a, const u64* __restrict__ b, u64* __restrict__ r, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    e2 x = e2_ld(a + 2 * (size_t)i), y = e2_ld(b + 2 * (size_t)i), z;
    if (OP == 0) z = e2_add(x, y);
    else if (OP == 1) z = e2_sub(x, y);
    else z = e2_mul(x, y);
    e2_st(r + 2 * (size_t)i, z);
}

template <int OP>
static int gl_batch(const u64* a, const u64* b, u64* r, int n, const char* name) {
    if (n < 0) return GB_EINVAL;
    if (n == 0) return GB_OK;
    gl_batch_kernel<OP><<<grid_for(n, 256), 256, 0, stream()>>>(a, b, r, n);
    return check_launch(name);
}
template <int OP>
static int e2_batch(const u64* a, const u64* b, u64* r, int n, const char* name) {
    if (n < 0) return GB_EINVAL;
    if (n == 0) return GB_OK;
    e2_batch_kernel<OP><<<grid_for(n, 256), 256, 0, stream()>>>(a, b, r, n);
    return check_launch(name);
}

__global__ void i64_to_i32_kernel(const int64_t* __restrict__ s, int32_t* __restrict__ d, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        d[i] = (int32_t)s[i];
}
__global__ void add_i32_i64_kernel(int64_t* __restrict__ d, const int32_t* __restrict__ s, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        d[i] += (int64_t)s[i];
}

// Throughput ceiling of this file's Goldilocks multiplication: every thread runs
// 8 independent chains of `iters` multiplications (no memory traffic).
__global__ void __launch_bounds__(256) mulmod_probe_kernel(u64* out, int iters) {
    u64 a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = 0x9E3779B97F4A7C15ull * (threadIdx.x + 1 + j) + blockIdx.x;
    const u64 m = 0x0123456789ABCDEFull;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) a[j] = gl_mul(a[j], m);
    }
    u64 r = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) r ^= a[j];
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = r;
}

}  // namespace gb

using namespace gb;

extern "C" {

int gb_set_stream(void* s) {
    t_stream = s ? (cudaStream_t)s : cudaStreamPerThread;
    return 0;
}
void* gb_get_stream(void) { return (void*)t_stream; }
const char* gb_last_error(void) { return t_err.c_str(); }
int gb_device_sm_count(void) { return num_sms(); }
unsigned long long gb_launch_count(void) { return g_launches.load(); }

int gb_mulmod_probe(uint64_t* d_out, int blocks, int iters) {
    if (blocks <= 0 || iters <= 0) return GB_EINVAL;
    mulmod_probe_kernel<<<blocks, 256, 0, stream()>>>(d_out, iters);
    return check_launch("gb_mulmod_probe");
}

int gb_binary_version(void) {
    cudaFuncAttributes a;
    if (cudaFuncGetAttributes(&a, mulmod_probe_kernel) != cudaSuccess) return -1;
    return a.binaryVersion;
}

int goldilocks_cuda_init(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return -1;
    return cudaSetDevice(0) == cudaSuccess ? 0 : -1;
}
int poseidon2_cuda_init(void) { return 0; }

int cuda_malloc(void** ptr, size_t size) { return cudaMalloc(ptr, size) == cudaSuccess ? 0 : -1; }
int cuda_free(void* ptr) { return cudaFree(ptr) == cudaSuccess ? 0 : -1; }
int cuda_memcpy_htod(void* dst, const void* src, size_t size) {
    return cudaMemcpyAsync(dst, src, size, cudaMemcpyHostToDevice, stream()) == cudaSuccess &&
                   cudaStreamSynchronize(stream()) == cudaSuccess
               ? 0
               : -1;
}
int cuda_memcpy_dtoh(void* dst, const void* src, size_t size) {
    return cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToHost, stream()) == cudaSuccess &&
                   cudaStreamSynchronize(stream()) == cudaSuccess
               ? 0
               : -1;
}
int cuda_memcpy_dtod(void* dst, const void* src, size_t size) {
    return cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToDevice, stream()) == cudaSuccess &&
                   cudaStreamSynchronize(stream()) == cudaSuccess
               ? 0
               : -1;
}
int cuda_device_synchronize(void) { return cudaDeviceSynchronize() == cudaSuccess ? 0 : -1; }
int cuda_get_last_error(void) { return (int)cudaGetLastError(); }
int cuda_peek_at_last_error(void) { return (int)cudaPeekAtLastError(); }
int cuda_mem_get_info(size_t* f, size_t* t) { return cudaMemGetInfo(f, t) == cudaSuccess ? 0 : -1; }
const char* agl_cuda_error_string(int code) { return cudaGetErrorString((cudaError_t)code); }
// Peer access between devices (almost wrapper.cu:268-279): best effort, an already enabled peer is
// success.  A one-GPU process has no peer, so enabling one reports -1 as the reference does.
int cuda_memcpy_peer(void* dst, int dst_dev, const void* src, int src_dev, size_t size) {
    return cudaMemcpyPeer(dst, dst_dev, src, src_dev, size) == cudaSuccess ? 0 : -1;
}
int cuda_enable_peer_access(int peer) {
    const cudaError_t e = cudaDeviceEnablePeerAccess(peer, 0);
    if (e == cudaSuccess || e == cudaErrorPeerAccessAlreadyEnabled) {
        cudaGetLastError();
        return 0;
    }
    cudaGetLastError();
    return -1;
}
// Profiler ranges (almost wrapper.cu:327-328)
void agl_nvtx_push(const char* name) { nvtxRangePushA(name); }
void agl_nvtx_pop(void) { nvtxRangePop(); }
int cuda_memset(void* dst, int value, size_t size) {
    return cudaMemsetAsync(dst, value, size, stream()) == cudaSuccess && cudaStreamSynchronize(stream()) == cudaSuccess
               ? 0
               : -1;
}
int cuda_sync_mine(void) { return cudaStreamSynchronize(stream()) == cudaSuccess ? 0 : -1; }
int cuda_stream_create(void** s) {
    cudaStream_t st;
    if (!s || cudaStreamCreate(&st) != cudaSuccess) return -1;
    *s = (void*)st;
    return 0;
}
int cuda_stream_destroy(void* s) { return cudaStreamDestroy((cudaStream_t)s) == cudaSuccess ? 0 : -1; }
int cuda_stream_synchronize(void* s) { return cudaStreamSynchronize((cudaStream_t)s) == cudaSuccess ? 0 : -1; }
int cuda_memcpy_dtod_async(void* dst, const void* src, size_t size, void* s) {
    return cudaMemcpyAsync(dst, src, size, cudaMemcpyDeviceToDevice, (cudaStream_t)s) == cudaSuccess ? 0 : -1;
}
int cuda_memcpy_htod_async(void* dst, const void* src, size_t size, void* s) {
    return cudaMemcpyAsync(dst, src, size, cudaMemcpyHostToDevice, (cudaStream_t)s) == cudaSuccess ? 0 : -1;
}
size_t agl_cached_bytes(void) {
    int dev = 0;
    cudaMemPool_t pool;
    uint64_t reserved = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess)
        return 0;
    return (size_t)reserved;
}
size_t gb_pool_used_high(int reset) {
    int dev = 0;
    cudaMemPool_t pool;
    uint64_t high = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess ||
        cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &high) != cudaSuccess)
        return (size_t)-1;
    if (reset) {
        uint64_t zero = 0;  // resets the mark to the memory in use now
        if (cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero) != cudaSuccess) return (size_t)-1;
    }
    return (size_t)high;
}
// chunked copies through the thread's pinned staging buffer
static int staged_copy(void* dst, const void* src, size_t bytes, bool to_host) {
    constexpr size_t CH = (size_t)16 << 20;
    if (bytes == 0) return 0;
    uint64_t* buf = gb::thread_pinned(2, CH / 8);
    if (!buf) return -1;
    cudaStream_t s = stream();
    for (size_t o = 0; o < bytes; o += CH) {
        size_t n = bytes - o < CH ? bytes - o : CH;
        if (to_host) {
            if (cudaMemcpyAsync(buf, (const char*)src + o, n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                return -1;
            std::memcpy((char*)dst + o, buf, n);
        } else {
            std::memcpy(buf, (const char*)src + o, n);
            if (cudaMemcpyAsync((char*)dst + o, buf, n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                return -1;
        }
    }
    return 0;
}
int agl_d2h_staged(void* h_dst, const void* d_src, size_t bytes) { return staged_copy(h_dst, d_src, bytes, true); }
int agl_h2d_staged(void* d_dst, const void* h_src, size_t bytes) { return staged_copy(d_dst, h_src, bytes, false); }
int cuda_pool_trim(size_t min_bytes_to_keep) {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) return -1;
    return cudaMemPoolTrimTo(pool, min_bytes_to_keep) == cudaSuccess ? 0 : -1;
}
int cuda_set_device(int d) { return cudaSetDevice(d) == cudaSuccess ? 0 : -1; }
int cuda_get_device(int* d) { return cudaGetDevice(d) == cudaSuccess ? 0 : -1; }
int cuda_get_device_count(int* c) { return cudaGetDeviceCount(c) == cudaSuccess ? 0 : -1; }
int cuda_get_device_name(int device, char* name, int max_len) {
    cudaDeviceProp prop;
    if (max_len <= 0 || cudaGetDeviceProperties(&prop, device) != cudaSuccess) return -1;
    std::strncpy(name, prop.name, (size_t)max_len - 1);
    name[max_len - 1] = '\0';
    return 0;
}

int gl_batch_add(const uint64_t* a, const uint64_t* b, uint64_t* r, int n) { return gl_batch<0>(a, b, r, n, "gl_batch_add"); }
int gl_batch_sub(const uint64_t* a, const uint64_t* b, uint64_t* r, int n) { return gl_batch<1>(a, b, r, n, "gl_batch_sub"); }
int gl_batch_mul(const uint64_t* a, const uint64_t* b, uint64_t* r, int n) { return gl_batch<2>(a, b, r, n, "gl_batch_mul"); }
int gl_batch_inverse(const uint64_t* a, uint64_t* r, int n) { return gl_batch<3>(a, nullptr, r, n, "gl_batch_inverse"); }
int ext2_batch_add_ffi(const uint64_t* a, const uint64_t* b, uint64_t* r, int n) { return e2_batch<0>(a, b, r, n, "ext2_batch_add"); }
int ext2_batch_sub_ffi(const uint64_t* a, const uint64_t* b, uint64_t* r, int n) { return e2_batch<1>(a, b, r, n, "ext2_batch_sub"); }
int ext2_batch_mul_ffi(const uint64_t* a, const uint64_t* b, uint64_t* r, int n) { return e2_batch<2>(a, b, r, n, "ext2_batch_mul"); }

void gb_transcript_new(gb_transcript* t, const char* label) {
    std::memset(t, 0, sizeof(*t));
    for (const char* p = label; *p; p++) host::tr_absorb(t, (u64)(unsigned char)*p);
}
void gb_transcript_append_u64(gb_transcript* t, const char* label, uint64_t v) { host::tr_append_u64(t, label, v); }
void gb_transcript_append_ext2(gb_transcript* t, const char* label, const uint64_t v[2]) {
    host::tr_append_ext2(t, label, host::E2{v[0], v[1]});
}
void gb_transcript_challenge_ext2(gb_transcript* t, const char* label, uint64_t out[2]) {
    host::E2 c = host::tr_challenge_ext2(t, label);
    out[0] = c.c0;
    out[1] = c.c1;
}


// Integer helpers of the Morpheus authentication path (almost wrapper.cu:3943-3958): d = (i32) s,
// d += (i64) s.  Synchronising.
int agl_i64_to_i32(const int64_t* s, int32_t* d, uint64_t n) {
    if (!n) return 0;
    i64_to_i32_kernel<<<grid_for(n, 256), 256, 0, stream()>>>(s, d, n);
    const cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? (int)e : (int)cudaStreamSynchronize(stream());
}
int agl_add_i32_i64(int64_t* d, const int32_t* s, uint64_t n) {
    if (!n) return 0;
    add_i32_i64_kernel<<<grid_for(n, 256), 256, 0, stream()>>>(d, s, n);
    const cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? (int)e : (int)cudaStreamSynchronize(stream());
}
// The calling thread's low-priority stream toggle of the Gaussian sampler (almost wrapper.cu:2989-2997).
// The sampler itself is not part of this library; the toggle keeps its contract (0, or -1 when the
// stream cannot be created).
static thread_local cudaStream_t t_low_stream = nullptr;
int agl_gauss_low_priority(int on) {
    if (on && !t_low_stream) {
        int lo = 0, hi = 0;
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if (cudaStreamCreateWithPriority(&t_low_stream, cudaStreamNonBlocking, lo) != cudaSuccess) {
            t_low_stream = nullptr;
            return -1;
        }
    } else if (!on && t_low_stream) {
        cudaStreamDestroy(t_low_stream);
        t_low_stream = nullptr;
    }
    return 0;
}
}  // extern "C"
