// Host emulation of CUDA launches, for running the reference's own kernel source on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  The reference's device code (cuda/*.cuh, and the kernels of
// goldilocks-cuda-rs/cuda/wrapper.cu) is compiled as host C++ by oracle/Makefile with the CUDA
// qualifiers mapped away; this header supplies what those kernels read from the hardware:
//
//   * threadIdx / blockIdx / blockDim / gridDim, one copy per host thread;
//   * launches: the grid's blocks are split over host threads, and inside a block the threads
//     run one after another;
//   * __syncthreads(): kernels that call it are launched with sim::launch_sync, which runs each
//     CUDA thread of a block as a fiber (ucontext) and switches fibers at every barrier, so a
//     shared-memory reduction sees every write made before the barrier.  __shared__ arrays are
//     function statics, which is correct because one host thread runs one block at a time and
//     each host thread has its own copy (thread_local).
//
// The reference's kernels use no warp shuffles, votes or atomics on this path.
#pragma once

#include <ucontext.h>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <thread>
#include <vector>

#include <vector_types.h>

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

namespace sim {

struct FiberBlock;
extern thread_local FiberBlock* t_block;

// One block's threads as fibers.  The scheduler resumes every unfinished fiber in turn; a fiber
// returns to it at each barrier and when its kernel body ends.
struct FiberBlock {
    static constexpr size_t STACK = 64 << 10;
    std::vector<ucontext_t> ctx;
    std::vector<char> stacks;
    std::vector<uint8_t> done;
    ucontext_t sched;
    unsigned nthreads = 0, cur = 0;
    const std::function<void()>* body = nullptr;

    void prepare(unsigned n) {
        if (ctx.size() < n) {
            ctx.resize(n);
            stacks.resize((size_t)n * STACK);
            done.resize(n);
        }
        nthreads = n;
    }
    static void entry() {
        FiberBlock* b = t_block;
        (*b->body)();
        b->done[b->cur] = 1;
        swapcontext(&b->ctx[b->cur], &b->sched);
    }
    void set_thread(unsigned t) {
        threadIdx.x = t % blockDim.x;
        threadIdx.y = (t / blockDim.x) % blockDim.y;
        threadIdx.z = t / (blockDim.x * blockDim.y);
    }
    void run(const std::function<void()>& fn) {
        body = &fn;
        for (unsigned t = 0; t < nthreads; t++) {
            getcontext(&ctx[t]);
            ctx[t].uc_stack.ss_sp = stacks.data() + (size_t)t * STACK;
            ctx[t].uc_stack.ss_size = STACK;
            ctx[t].uc_link = nullptr;
            makecontext(&ctx[t], (void (*)())entry, 0);
            done[t] = 0;
        }
        for (unsigned left = nthreads; left;) {
            left = 0;
            for (unsigned t = 0; t < nthreads; t++) {
                if (done[t]) continue;
                cur = t;
                set_thread(t);
                swapcontext(&sched, &ctx[t]);
                if (!done[t]) left++;
            }
        }
    }
    void barrier() { swapcontext(&ctx[cur], &sched); }
};

inline int host_threads() {
    static int n = [] {
        unsigned h = std::thread::hardware_concurrency();
        return (int)(h ? h : 1);
    }();
    return n;
}

// Splits the grid's blocks over host threads; block_fn(b) runs block b of the grid.
inline void for_blocks(unsigned long long nblocks, const std::function<void(unsigned long long)>& block_fn) {
    int k = host_threads();
    if (nblocks < 4 || k == 1) {
        for (unsigned long long b = 0; b < nblocks; b++) block_fn(b);
        return;
    }
    if ((unsigned long long)k > nblocks) k = (int)nblocks;
    std::vector<std::thread> th;
    for (int t = 0; t < k; t++)
        th.emplace_back([&, t] {
            for (unsigned long long b = nblocks * t / k; b < nblocks * (t + 1) / k; b++) block_fn(b);
        });
    for (auto& x : th) x.join();
}

inline void set_block(dim3 grid, dim3 block, unsigned long long b) {
    gridDim = grid;
    blockDim = block;
    blockIdx.x = (unsigned)(b % grid.x);
    blockIdx.y = (unsigned)((b / grid.x) % grid.y);
    blockIdx.z = (unsigned)(b / ((unsigned long long)grid.x * grid.y));
}

// A kernel with no barrier: the threads of each block run one after another.
inline void launch(dim3 grid, dim3 block, const std::function<void()>& kernel) {
    unsigned long long nb = (unsigned long long)grid.x * grid.y * grid.z;
    unsigned nt = block.x * block.y * block.z;
    for_blocks(nb, [&](unsigned long long b) {
        set_block(grid, block, b);
        for (unsigned t = 0; t < nt; t++) {
            threadIdx.x = t % block.x;
            threadIdx.y = (t / block.x) % block.y;
            threadIdx.z = t / (block.x * block.y);
            kernel();
        }
    });
}

// A kernel that calls __syncthreads(): each block's threads run as fibers.
inline void launch_sync(dim3 grid, dim3 block, const std::function<void()>& kernel) {
    unsigned long long nb = (unsigned long long)grid.x * grid.y * grid.z;
    unsigned nt = block.x * block.y * block.z;
    for_blocks(nb, [&](unsigned long long b) {
        static thread_local FiberBlock fb;
        t_block = &fb;
        set_block(grid, block, b);
        fb.prepare(nt);
        fb.run(kernel);
        t_block = nullptr;
    });
}

inline void syncthreads() {
    if (!t_block) {
        std::fprintf(stderr, "ref_sim: __syncthreads() in a kernel launched without launch_sync\n");
        std::abort();
    }
    t_block->barrier();
}

}  // namespace sim

#define SIM_DEFINE_BUILTINS                  \
    thread_local uint3 threadIdx;            \
    thread_local uint3 blockIdx;             \
    thread_local dim3 blockDim;              \
    thread_local dim3 gridDim;               \
    namespace sim {                          \
    thread_local FiberBlock* t_block = nullptr; \
    }
