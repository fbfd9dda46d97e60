// Host emulation of one eight-lane group of a warp, for host builds of
// warp-cooperative kernel code whose shuffles all lie outside divergent
// branches (every lane makes the same sequence of __shfl_sync calls).
//
// run_group(f, out) runs f(g) for g = 0..7 one lane after another, in
// passes.  Within a pass, __shfl_sync records the calling lane's value and
// returns the value its source lane recorded at the same call in the
// previous pass.  Passes repeat until every call returned what its source
// lane recorded in the same pass (a fixpoint).  A shuffle's value depends
// only on earlier calls, so the fixpoint is reached after at most as many
// passes as the longest chain of dependent shuffles, and the lanes' results
// are then those of lockstep execution.
#pragma once
#include <cstdlib>
#include <cstring>

namespace group_lanes {
constexpr int kLanes = 8, kMaxCalls = 2048;
inline int lane = 0, call = 0;
inline double rec[kLanes][kMaxCalls], prev[kLanes][kMaxCalls];
}  // namespace group_lanes

static inline double __shfl_sync(unsigned, double v, int src, int width) {
    using namespace group_lanes;
    const int k = call++;
    if (k >= kMaxCalls || width != kLanes) std::abort();
    rec[lane][k] = v;
    return prev[src & (width - 1)][k];
}

// false if the lanes disagree on the number of calls or no fixpoint is reached
template <class F>
static bool run_group(F f, double out[group_lanes::kLanes], int max_passes = 100) {
    using namespace group_lanes;
    std::memset(prev, 0, sizeof prev);
    for (int p = 0; p < max_passes; p++) {
        int calls = -1;
        for (int g = 0; g < kLanes; g++) {
            lane = g;
            call = 0;
            out[g] = f(g);
            if (calls >= 0 && call != calls) return false;
            calls = call;
        }
        bool fixed = true;
        for (int g = 0; g < kLanes && fixed; g++)
            fixed = std::memcmp(rec[g], prev[g], sizeof(double) * calls) == 0;
        if (fixed) return true;
        for (int g = 0; g < kLanes; g++) std::memcpy(prev[g], rec[g], sizeof(double) * calls);
    }
    return false;
}
