// Allocation-free variant of the debug voxel export (make_debug_voxel_map,
// scripts/gvom.py:395-410, 481-503).
//
// The regular export (gvom_debug_voxel_map) allocates its block-offset table
// and its output buffer with cudaMalloc / cudaFree.  Some callers cannot let
// that happen: a debug publisher that shares the GPU with a latency-bound
// mapping loop (cudaFree synchronises the whole device, so it stalls every
// other map instance's in-flight scan), or a process that must keep its device
// memory footprint fixed after start-up.  This variant writes into a device
// buffer the caller owns and keeps its only scratch, the per-block row counts
// and offsets, in a fixed-size file-scope device array.
//
// Scratch contents: words [0, nblocks) receive each block's count of occupied
// voxels (k_debug_count), are turned into exclusive row offsets in place
// (k_debug_offsets), and word [nblocks] receives the total.  Every word that a
// kernel reads was written earlier in the same call, so nothing has to start
// at zero.  The array is shared by every instance in the process on a device:
// two calls that overlap in time would race on it, so the host entry point
// holds a process-wide lock per device until the call's device work is done.
#include <cuda_runtime.h>

#include "gvom_internal.cuh"

namespace gvom {

// kStaticDebugBlocks blocks of 1024 voxels cover grids up to 32M voxels
// (e.g. 512 x 512 x 128); 128 KB of device memory.
static __device__ __align__(256) int g_debug_scratch[kStaticDebugBlocks + 1];

namespace {

// counts -> exclusive offsets, in place, and the total at [n]; one block of
// 1024 threads, each owning a run of up to kStaticDebugBlocks / 1024 words
constexpr int kScanThreads = 1024;

__global__ void __launch_bounds__(kScanThreads) k_debug_offsets(int *__restrict__ words, int n) {
    __shared__ int warp_sum[kScanThreads / 32];
    const int per = (n + kScanThreads - 1) / kScanThreads;
    const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
    int own = 0;
    for (int k = lo; k < hi; k++) own += words[k];
    // block-wide exclusive scan of `own`
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int incl = own;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sum[w] = incl;
    __syncthreads();
    if (w == 0) {
        int v = warp_sum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += t;
        }
        warp_sum[lane] = v;  // inclusive over warps
    }
    __syncthreads();
    int run = (w > 0 ? warp_sum[w - 1] : 0) + incl - own;
    for (int k = lo; k < hi; k++) {
        const int c = words[k];
        words[k] = run;
        run += c;
    }
    if (threadIdx.x == kScanThreads - 1) words[n] = warp_sum[kScanThreads / 32 - 1];
}

}  // namespace

cudaError_t debug_static_scratch(int **ptr) {
    return cudaGetSymbolAddress(reinterpret_cast<void **>(ptr), g_debug_scratch);
}

cudaError_t launch_debug_offsets(int *words, int n, cudaStream_t st) {
    k_debug_offsets<<<1, kScanThreads, 0, st>>>(words, n);
    return cudaGetLastError();
}

}  // namespace gvom
