/* Host emulation of whole CUDA kernel launches, one fiber per CUDA thread,
 * for host builds of kernels that synchronise inside a block
 * (tests/test_process_host.py, tests/test_pipeline_host.py).  Include after
 * cuda_runtime.h (this directory).
 *
 * Blocks run one after another on the calling thread.  Each CUDA thread of a
 * block is a fiber with its own stack, entered once through a POSIX ucontext
 * and afterwards switched with _setjmp / _longjmp; a fiber runs until it
 * waits at a barrier or returns, and a scheduler then resumes the next ready
 * fiber.  __syncthreads is a barrier of the block's live threads; a warp
 * shuffle writes the caller's value into the warp's exchange slots, waits at
 * a barrier of the warp's live lanes and reads its source lane's slot.  A
 * barrier's waiters become ready again when its last live participant
 * arrives; a thread that returns leaves its block's and its warp's barriers,
 * as an exited CUDA thread stops counting at a block barrier.  __shared__
 * variables become statics (one block runs at a time).  The schedule is
 * deterministic, so atomics resolve in the same order on every run, unless
 * shuffle_seed is set: then blocks run in a random order and a random ready
 * fiber resumes next, so that a read which only a missing barrier separates
 * from its write, or an assumption about block order, shows.  Kernels
 * whose shuffles run with lanes missing (a lane that returned) and kernels
 * that spin on memory another thread writes are outside what this emulates;
 * a block whose fibers all wait ends the program.  Not part of the library. */
#pragma once
#include <setjmp.h>
#include <ucontext.h>

#if defined(_FORTIFY_SOURCE) && _FORTIFY_SOURCE > 0
#error "build without _FORTIFY_SOURCE: fibers switch stacks with _longjmp, which its check refuses"
#endif

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <vector>

#define __shared__ static

struct dim3 {
    unsigned x, y, z;
    constexpr dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};

namespace block_threads {

constexpr int kMaxThreads = 1024;          // the largest block this emulates
constexpr size_t kStackBytes = 256 << 10;  // per fiber

struct Barrier {
    int expected = 0, arrived = 0;
    std::vector<int> waiters;
};

struct JmpBuf {
    jmp_buf b;
};

struct Sched {
    ucontext_t main_ctx;  // the scheduler, as a fiber's first entry left it
    jmp_buf main_jb;      // the scheduler, as the last resume left it
    std::vector<ucontext_t> ctx;
    std::vector<JmpBuf> jb;  // each started fiber, as it last waited
    std::vector<char> started;
    std::vector<char *> stacks;
    std::vector<HostDim3> tidx;
    std::vector<unsigned> par;
    std::vector<char> done;
    std::deque<int> ready;
    int cur = -1;
    const std::function<void()> *fn = nullptr;
    Barrier bar;
    std::vector<Barrier> warp;
    unsigned long long xchg[2][kMaxThreads];  // by shuffle parity
};
inline Sched *sched = nullptr;
inline unsigned parity = 0;  // the running fiber's shuffles so far, mod 2
// 0: blocks in grid order and ready fibers first in, first out; otherwise
// the seed of a shuffled schedule
inline unsigned long long shuffle_seed = 0;
inline unsigned long long shuffle_state = 0;
inline unsigned long long shuffle_next() {  // splitmix64
    unsigned long long z = (shuffle_state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

inline int linear_tid() { return (int)(threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z)); }

inline void release(Barrier &b) {
    b.arrived = 0;
    for (int w : b.waiters) sched->ready.push_back(w);
    b.waiters.clear();
}

inline void arrive_and_wait(Barrier &b) {
    Sched &s = *sched;
    if (b.arrived + 1 == b.expected) {
        release(b);
        return;
    }
    b.arrived++;
    const int me = s.cur;
    b.waiters.push_back(me);
    if (!_setjmp(s.jb[me].b)) _longjmp(s.main_jb, 1);  // back here when the barrier is complete
}

inline void arrive_and_drop(Barrier &b) {
    b.expected--;
    if (b.arrived > 0 && b.arrived == b.expected) release(b);
}

inline void fiber_entry() {
    Sched &s = *sched;
    const int me = s.cur;
    (*s.fn)();
    arrive_and_drop(s.bar);
    arrive_and_drop(s.warp[me >> 5]);
    s.done[me] = 1;
    _longjmp(s.main_jb, 1);  // never returns
}

// value of lane `src` of the caller's warp (`take`), else the caller's own.
// One barrier per shuffle: consecutive shuffles use alternate slot arrays,
// and a lane reaches the next shuffle of the same parity only after every
// lane has passed the barrier of the shuffle in between, that is, after
// every lane has read this one.
template <class T>
inline T exchange(T v, int src, bool take) {
    static_assert(sizeof(T) <= 8, "shuffles move at most 8 bytes");
    const int t = linear_tid(), w = t >> 5;
    unsigned long long *x = sched->xchg[parity];
    parity ^= 1u;
    unsigned long long b = 0;
    std::memcpy(&b, &v, sizeof(T));
    x[t] = b;
    arrive_and_wait(sched->warp[w]);
    T r = v;
    if (take) std::memcpy(&r, &x[(w << 5) + src], sizeof(T));
    return r;
}

// Every block of the grid, x fastest (or shuffled, see shuffle_seed).
inline void launch(dim3 grid, dim3 blk, const std::function<void()> &fn) {
    static Sched *s = new Sched();
    sched = s;
    const int nt = (int)(blk.x * blk.y * blk.z);
    if (nt < 1 || nt > kMaxThreads) std::abort();
    while ((int)s->stacks.size() < nt) s->stacks.push_back(static_cast<char *>(std::malloc(kStackBytes)));
    s->ctx.resize(nt);
    s->jb.resize(nt);
    s->started.resize(nt);
    s->tidx.resize(nt);
    s->par.resize(nt);
    s->done.resize(nt);
    s->fn = &fn;
    blockDim = {blk.x, blk.y, blk.z};
    gridDim = {grid.x, grid.y, grid.z};
    const unsigned long long nb = (unsigned long long)grid.x * grid.y * grid.z;
    std::vector<unsigned long long> order(nb);
    for (unsigned long long b = 0; b < nb; b++) order[b] = b;
    if (shuffle_seed) {
        if (!shuffle_state) shuffle_state = shuffle_seed;
        for (unsigned long long b = nb; b > 1; b--) std::swap(order[b - 1], order[shuffle_next() % b]);
    }
    for (unsigned long long ob : order) {
        const unsigned bx = (unsigned)(ob % grid.x), by = (unsigned)(ob / grid.x % grid.y),
                       bz = (unsigned)(ob / grid.x / grid.y);
        blockIdx = {bx, by, bz};
        s->bar = Barrier{nt, 0, {}};
        s->warp.assign((nt + 31) / 32, Barrier{});
        for (int w = 0; w * 32 < nt; w++) s->warp[w].expected = std::min(32, nt - w * 32);
        s->ready.clear();
        for (int i = 0; i < nt; i++) {
            getcontext(&s->ctx[i]);
            s->ctx[i].uc_stack.ss_sp = s->stacks[i];
            s->ctx[i].uc_stack.ss_size = kStackBytes;
            s->ctx[i].uc_link = &s->main_ctx;
            makecontext(&s->ctx[i], fiber_entry, 0);
            s->tidx[i] = {i % blk.x, (i / blk.x) % blk.y, i / (blk.x * blk.y)};
            s->par[i] = 0;
            s->done[i] = 0;
            s->started[i] = 0;
            s->ready.push_back(i);
        }
        while (!s->ready.empty()) {
            int i;
            if (shuffle_seed) {
                const size_t j = (size_t)(shuffle_next() % s->ready.size());
                i = s->ready[j];
                s->ready.erase(s->ready.begin() + (long)j);
            } else {
                i = s->ready.front();
                s->ready.pop_front();
            }
            s->cur = i;
            threadIdx = s->tidx[i];
            parity = s->par[i];
            // a started fiber resumes where it waited (no signal-mask system
            // call, unlike swapcontext); a new one enters once through its
            // ucontext; either comes back here with _longjmp
            if (!_setjmp(s->main_jb)) {
                if (s->started[i]) _longjmp(s->jb[i].b, 1);
                s->started[i] = 1;
                swapcontext(&s->main_ctx, &s->ctx[i]);
            }
            s->par[i] = parity;
        }
        for (int i = 0; i < nt; i++)
            if (!s->done[i]) {
                std::fprintf(stderr, "block_threads: block (%u, %u, %u): thread %d waits forever\n", bx, by,
                             bz, i);
                std::abort();
            }
    }
    s->cur = -1;
}

}  // namespace block_threads

static inline void __syncthreads() { block_threads::arrive_and_wait(block_threads::sched->bar); }

static inline void __syncwarp(unsigned = 0xffffffffu) {
    block_threads::arrive_and_wait(block_threads::sched->warp[block_threads::linear_tid() >> 5]);
}

// the lanes of the caller's warp whose predicate is non-zero (every lane
// of the warp takes part)
static inline unsigned __ballot_sync(unsigned, int pred) {
    using namespace block_threads;
    const int t = linear_tid(), w = t >> 5;
    unsigned long long *x = sched->xchg[parity];
    parity ^= 1u;
    x[t] = pred != 0;
    arrive_and_wait(sched->warp[w]);
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
