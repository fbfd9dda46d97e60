/* Host emulation of whole CUDA kernel launches with one host thread per CUDA
 * thread, for host builds of kernels that synchronise inside a block
 * (tests/test_process_host.py).  Include after cuda_runtime.h (this
 * directory), whose thread and block indices are per host thread and whose
 * atomics are host atomics.
 *
 * Blocks run one after another on a pool of host threads; the threads of a
 * block run at the same time.  __syncthreads is a barrier of the block's
 * threads; a warp shuffle writes the caller's value into the warp's exchange
 * slots, waits at a barrier of the warp's lanes and reads its source lane's
 * slot.  __shared__ variables become statics, which is sound
 * because one block runs at a time.  A thread that returns leaves its
 * block's and its warp's barriers, as an exited CUDA thread stops counting
 * at a block barrier.  Kernels whose shuffles run with lanes missing (a lane
 * that returned) are outside what this emulates.  Not part of the library. */
#pragma once
#include <algorithm>
#include <barrier>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

#define __shared__ static

struct dim3 {
    unsigned x, y, z;
    constexpr dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

namespace block_threads {

constexpr int kPoolThreads = 1024;  // the largest block this emulates

struct BlockState {
    std::unique_ptr<std::barrier<>> bar;
    std::vector<std::unique_ptr<std::barrier<>>> warp;
    unsigned long long xchg[2][kPoolThreads];  // by shuffle parity
    explicit BlockState(int nt) : bar(new std::barrier<>(nt)) {
        for (int w = 0; w * 32 < nt; w++) warp.emplace_back(new std::barrier<>(std::min(32, nt - w * 32)));
    }
};
inline BlockState *cur = nullptr;
inline thread_local unsigned parity = 0;  // the calling thread's shuffles so far, mod 2

inline int linear_tid() { return (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)); }

// value of lane `src` of the caller's warp (`take`), else the caller's own.
// One barrier per shuffle: consecutive shuffles use alternate slot arrays,
// and a lane can reach the next shuffle of the same parity only after every
// lane has passed the barrier of the shuffle in between, that is, after
// every lane has read this one.
template <class T>
inline T exchange(T v, int src, bool take) {
    static_assert(sizeof(T) <= 8, "shuffles move at most 8 bytes");
    const int t = linear_tid(), w = t >> 5;
    unsigned long long *x = cur->xchg[parity];
    parity ^= 1u;
    unsigned long long b = 0;
    std::memcpy(&b, &v, sizeof(T));
    x[t] = b;
    cur->warp[w]->arrive_and_wait();
    T r = v;
    if (take) std::memcpy(&r, &x[(w << 5) + src], sizeof(T));
    return r;
}

// as many host threads as the blocks it runs have threads
class Pool {
public:
    explicit Pool(int n) : go_(n + 1), done_(n + 1) {
        for (int i = 0; i < n; i++) th_.emplace_back([this, i] { run(i); });
    }
    // runs block `idx` of the launch; returns when its threads have finished
    void block(dim3 grid, dim3 blk, dim3 idx, const std::function<void()> *fn) {
        grid_ = grid;
        blk_ = blk;
        idx_ = idx;
        fn_ = fn;
        go_.arrive_and_wait();
        done_.arrive_and_wait();
    }

private:
    void run(int i) {
        for (;;) {
            go_.arrive_and_wait();
            const int nt = (int)(blk_.x * blk_.y * blk_.z);
            if (i < nt) {
                threadIdx = {i % blk_.x, (i / blk_.x) % blk_.y, i / (blk_.x * blk_.y)};
                parity = 0;
                blockIdx = {idx_.x, idx_.y, idx_.z};
                blockDim = {blk_.x, blk_.y, blk_.z};
                gridDim = {grid_.x, grid_.y, grid_.z};
                (*fn_)();
                cur->bar->arrive_and_drop();
                cur->warp[i >> 5]->arrive_and_drop();
            }
            done_.arrive_and_wait();
        }
    }
    std::barrier<> go_, done_;
    std::vector<std::thread> th_;
    dim3 grid_, blk_, idx_;
    const std::function<void()> *fn_ = nullptr;
};

// Every block of the grid, x fastest, on the pool of the block's size.  The
// pools live for the process (their threads wait between launches).
inline void launch(dim3 grid, dim3 blk, const std::function<void()> &fn) {
    static Pool *pools[kPoolThreads + 1] = {};
    const int nt = (int)(blk.x * blk.y * blk.z);
    if (nt < 1 || nt > kPoolThreads) std::abort();
    if (!pools[nt]) pools[nt] = new Pool(nt);
    Pool *pool = pools[nt];
    for (unsigned z = 0; z < grid.z; z++)
        for (unsigned y = 0; y < grid.y; y++)
            for (unsigned x = 0; x < grid.x; x++) {
                BlockState st(nt);
                cur = &st;
                pool->block(grid, blk, dim3(x, y, z), &fn);
                cur = nullptr;
            }
}

}  // namespace block_threads

static inline void __syncthreads() { block_threads::cur->bar->arrive_and_wait(); }

static inline void __syncwarp(unsigned = 0xffffffffu) {
    block_threads::cur->warp[block_threads::linear_tid() >> 5]->arrive_and_wait();
}

// the lanes of the caller's warp whose predicate is non-zero (every lane
// of the warp takes part)
static inline unsigned __ballot_sync(unsigned, int pred) {
    using namespace block_threads;
    const int t = linear_tid(), w = t >> 5;
    unsigned long long *x = cur->xchg[parity];
    parity ^= 1u;
    x[t] = pred != 0;
    cur->warp[w]->arrive_and_wait();
    unsigned m = 0;
    for (int l = 0; l < 32; l++)
        if (x[(w << 5) + l]) m |= 1u << l;
    return m;
}

// lane `src` of the caller's `width`-lane segment of the warp
template <class T>
static inline T __shfl_sync(unsigned, T v, int src, int width = 32) {
    const int lane = block_threads::linear_tid() & 31;
    return block_threads::exchange(v, (lane & ~(width - 1)) + (src & (width - 1)), true);
}
template <class T>
static inline T __shfl_up_sync(unsigned, T v, unsigned d) {
    const int lane = block_threads::linear_tid() & 31;
    return block_threads::exchange(v, lane - (int)d, lane >= (int)d);
}
template <class T>
static inline T __shfl_down_sync(unsigned, T v, unsigned d) {
    const int lane = block_threads::linear_tid() & 31;
    return block_threads::exchange(v, lane + (int)d, lane + (int)d < 32);
}
template <class T>
static inline T __shfl_xor_sync(unsigned, T v, int m) {
    const int lane = block_threads::linear_tid() & 31;
    return block_threads::exchange(v, lane ^ m, true);
}
