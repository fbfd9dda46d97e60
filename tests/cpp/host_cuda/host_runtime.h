/* A host stand-in for the CUDA runtime calls of the library's host code
 * (gvom_gb300/csrc/gvom_capi.cu), so that the C ABI itself runs on the CPU
 * over kernels run by block_threads.h (tests/test_capi_host.py).  Include after
 * cuda_runtime.h (this directory).
 *
 * Device memory is host memory: allocations are tracked (a pointer query
 * tells them from other memory) against a settable device total, so the
 * library's free-memory admission can be driven; fresh allocations hold a
 * junk pattern, as device memory holds whatever was there.  Each allocation
 * (rounded up to 256 bytes, the alignment cudaMalloc gives) ends against an
 * inaccessible page and starts after one, so a read or write past its end
 * stops the process; the bytes between the requested size and those pages
 * hold a guard pattern checked when the allocation is freed and on request,
 * so a write just past either end is counted (guard_faults).  Kernels run to
 * completion when they are launched, so work is done in issue order and
 * streams and events need no state.  Graph capture is refused.  Not part of
 * the library. */
#pragma once
#include <sys/mman.h>
#include <unistd.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "block_threads.h"

typedef struct CUgraph_st *cudaGraph_t;
typedef struct CUgraphExec_st *cudaGraphExec_t;
typedef struct CUgraphNode_st *cudaGraphNode_t;
struct cudaGraphEdgeData;

enum cudaMemcpyKind {
    cudaMemcpyHostToHost = 0,
    cudaMemcpyHostToDevice = 1,
    cudaMemcpyDeviceToHost = 2,
    cudaMemcpyDeviceToDevice = 3,
    cudaMemcpyDefault = 4
};
enum cudaStreamCaptureStatus { cudaStreamCaptureStatusNone = 0, cudaStreamCaptureStatusActive = 1 };
enum cudaStreamCaptureMode { cudaStreamCaptureModeGlobal = 0, cudaStreamCaptureModeThreadLocal = 1 };
enum cudaDeviceAttr { cudaDevAttrMultiProcessorCount = 16, cudaDevAttrPageableMemoryAccess = 88 };
enum cudaMemoryType { cudaMemoryTypeUnregistered = 0, cudaMemoryTypeHost = 1, cudaMemoryTypeDevice = 2 };

struct cudaMemsetParams {
    void *dst;
    size_t pitch;
    unsigned int value;
    unsigned int elementSize;
    size_t width;
    size_t height;
};
struct cudaKernelNodeParams {
    void *func;
    dim3 gridDim;
    dim3 blockDim;
    unsigned int sharedMemBytes;
    void **kernelParams;
    void **extra;
};
struct cudaPointerAttributes {
    cudaMemoryType type;
    int device;
    void *devicePointer;
    void *hostPointer;
};

constexpr unsigned cudaEventDisableTiming = 2;
constexpr unsigned cudaStreamNonBlocking = 1;
constexpr unsigned cudaEventRecordExternal = 1;
constexpr unsigned long long cudaGraphInstantiateFlagUseNodePriority = 8;
constexpr cudaError_t cudaSuccess = 0;
constexpr cudaError_t cudaErrorMemoryAllocation = 2;
constexpr cudaError_t cudaErrorNotSupported = 801;

namespace host_runtime {
inline std::mutex mu;
inline std::map<const char *, size_t> allocs;  // device allocations: address -> bytes
inline size_t total = (size_t)8 << 30;         // the device's memory
inline size_t used = 0;
inline int num_sms = 4;
inline char handle_bytes[1];  // streams and events: any non-null address
inline unsigned char junk = 0xa5;  // the contents of a fresh allocation
constexpr unsigned char kGuardByte = 0x5a;
inline unsigned long long guard_faults = 0;
struct Mapping {
    char *base;   // start of the mapping (an inaccessible page)
    size_t len;   // bytes mapped
    char *lo;     // first byte of the readable pages
    char *end;    // one past the readable pages (an inaccessible page follows)
};
inline std::map<const char *, Mapping> maps;  // allocation -> its mapping
// the guard bytes around [p, p + bytes) within the readable pages
inline bool guards_intact(const char *p, size_t bytes) {
    const Mapping &m = maps.at(p);
    for (const char *q = m.lo; q < p; q++)
        if ((unsigned char)*q != kGuardByte) return false;
    for (const char *q = p + bytes; q < m.end; q++)
        if ((unsigned char)*q != kGuardByte) return false;
    return true;
}
// live allocations whose guard zones were overwritten (counted in guard_faults)
inline unsigned long long check_live() {
    std::lock_guard<std::mutex> lk(mu);
    unsigned long long bad = 0;
    for (auto &a : allocs)
        if (!guards_intact(a.first, a.second)) bad++;
    guard_faults += bad;
    return bad;
}
}  // namespace host_runtime

static inline cudaError_t cudaMalloc(void **p, size_t bytes) {
    std::lock_guard<std::mutex> lk(host_runtime::mu);
    *p = nullptr;
    if (host_runtime::used + bytes > host_runtime::total) return cudaErrorMemoryAllocation;
    const size_t pg = (size_t)sysconf(_SC_PAGESIZE);
    const size_t rounded = bytes ? (bytes + 255) & ~(size_t)255 : 256;
    const size_t data = (rounded + pg - 1) / pg * pg;
    char *base = static_cast<char *>(mmap(nullptr, data + 2 * pg, PROT_READ | PROT_WRITE,
                                          MAP_PRIVATE | MAP_ANONYMOUS, -1, 0));
    if (base == MAP_FAILED) return cudaErrorMemoryAllocation;
    mprotect(base, pg, PROT_NONE);
    mprotect(base + pg + data, pg, PROT_NONE);
    char *lo = base + pg, *end = base + pg + data;
    char *m = end - rounded;  // the rounded allocation ends against the inaccessible page
    std::memset(lo, host_runtime::kGuardByte, (size_t)(m - lo));
    std::memset(m, host_runtime::junk, bytes);
    std::memset(m + bytes, host_runtime::kGuardByte, rounded - bytes);
    host_runtime::allocs[m] = bytes;
    host_runtime::maps[m] = host_runtime::Mapping{base, data + 2 * pg, lo, end};
    host_runtime::used += bytes;
    *p = m;
    return cudaSuccess;
}
static inline cudaError_t cudaFree(void *p) {
    if (!p) return cudaSuccess;
    std::lock_guard<std::mutex> lk(host_runtime::mu);
    auto it = host_runtime::allocs.find(static_cast<const char *>(p));
    if (it == host_runtime::allocs.end()) std::abort();  // not a device allocation
    if (!host_runtime::guards_intact(it->first, it->second)) host_runtime::guard_faults++;
    host_runtime::used -= it->second;
    const host_runtime::Mapping mp = host_runtime::maps.at(it->first);
    host_runtime::maps.erase(it->first);
    host_runtime::allocs.erase(it);
    munmap(mp.base, mp.len);
    return cudaSuccess;
}
static inline cudaError_t cudaMemGetInfo(size_t *fr, size_t *tot) {
    std::lock_guard<std::mutex> lk(host_runtime::mu);
    *fr = host_runtime::total - host_runtime::used;
    *tot = host_runtime::total;
    return cudaSuccess;
}
static inline cudaError_t cudaPointerGetAttributes(cudaPointerAttributes *a, const void *p) {
    std::lock_guard<std::mutex> lk(host_runtime::mu);
    std::memset(a, 0, sizeof *a);
    const char *c = static_cast<const char *>(p);
    auto it = host_runtime::allocs.upper_bound(c);
    if (it != host_runtime::allocs.begin()) {
        --it;
        if (c < it->first + it->second) {
            a->type = cudaMemoryTypeDevice;
            a->devicePointer = const_cast<void *>(p);
            return cudaSuccess;
        }
    }
    a->type = cudaMemoryTypeUnregistered;
    a->hostPointer = const_cast<void *>(p);
    return cudaSuccess;
}
static inline cudaError_t cudaMemcpyAsync(void *dst, const void *src, size_t n, cudaMemcpyKind, cudaStream_t) {
    if (n) std::memmove(dst, src, n);
    return cudaSuccess;
}
static inline cudaError_t cudaMemsetAsync(void *p, int v, size_t n, cudaStream_t = nullptr) {
    if (n) std::memset(p, v, n);
    return cudaSuccess;
}
static inline cudaError_t cudaGetDevice(int *d) {
    *d = 0;
    return cudaSuccess;
}
static inline cudaError_t cudaSetDevice(int) { return cudaSuccess; }
static inline cudaError_t cudaDeviceGetAttribute(int *v, cudaDeviceAttr a, int) {
    *v = a == cudaDevAttrMultiProcessorCount ? host_runtime::num_sms : 0;
    return cudaSuccess;
}
static inline cudaError_t cudaDeviceGetStreamPriorityRange(int *least, int *greatest) {
    *least = 0;
    *greatest = -1;
    return cudaSuccess;
}
static inline cudaError_t cudaStreamCreateWithPriority(cudaStream_t *s, unsigned, int) {
    *s = reinterpret_cast<cudaStream_t>(host_runtime::handle_bytes);
    return cudaSuccess;
}
static inline cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
static inline cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
static inline cudaError_t cudaStreamWaitEvent(cudaStream_t, cudaEvent_t, unsigned = 0) { return cudaSuccess; }
static inline cudaError_t cudaEventCreate(cudaEvent_t *e) {
    *e = reinterpret_cast<cudaEvent_t>(host_runtime::handle_bytes);
    return cudaSuccess;
}
static inline cudaError_t cudaEventCreateWithFlags(cudaEvent_t *e, unsigned) { return cudaEventCreate(e); }
static inline cudaError_t cudaEventDestroy(cudaEvent_t) { return cudaSuccess; }
static inline cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t = nullptr) { return cudaSuccess; }
static inline cudaError_t cudaEventRecordWithFlags(cudaEvent_t, cudaStream_t, unsigned) { return cudaSuccess; }
static inline cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
static inline cudaError_t cudaEventElapsedTime(float *ms, cudaEvent_t, cudaEvent_t) {
    *ms = 0.f;
    return cudaSuccess;
}
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
static inline const char *cudaGetErrorString(cudaError_t e) {
    return e == cudaErrorMemoryAllocation ? "out of memory (host runtime)" : "not supported by the host runtime";
}
struct cudaFuncAttributes {
    int unused;
};
static inline cudaError_t cudaFuncGetAttributes(cudaFuncAttributes *, const void *) { return cudaSuccess; }
// graphs: refused (the library's graph mode stays off)
static inline cudaError_t cudaStreamBeginCapture(cudaStream_t, cudaStreamCaptureMode) { return cudaErrorNotSupported; }
static inline cudaError_t cudaStreamEndCapture(cudaStream_t, cudaGraph_t *g) {
    *g = nullptr;
    return cudaErrorNotSupported;
}
static inline cudaError_t cudaStreamGetCaptureInfo(cudaStream_t, cudaStreamCaptureStatus *s, unsigned long long *,
                                                   cudaGraph_t *, const cudaGraphNode_t **, const cudaGraphEdgeData **,
                                                   size_t *n) {
    *s = cudaStreamCaptureStatusNone;
    if (n) *n = 0;
    return cudaSuccess;
}
static inline cudaError_t cudaGraphInstantiate(cudaGraphExec_t *, cudaGraph_t, unsigned long long) {
    return cudaErrorNotSupported;
}
static inline cudaError_t cudaGraphLaunch(cudaGraphExec_t, cudaStream_t) { return cudaErrorNotSupported; }
static inline cudaError_t cudaGraphDestroy(cudaGraph_t) { return cudaSuccess; }
static inline cudaError_t cudaGraphExecDestroy(cudaGraphExec_t) { return cudaSuccess; }
static inline cudaError_t cudaGraphExecKernelNodeSetParams(cudaGraphExec_t, cudaGraphNode_t,
                                                           const cudaKernelNodeParams *) {
    return cudaErrorNotSupported;
}
static inline cudaError_t cudaGraphExecMemsetNodeSetParams(cudaGraphExec_t, cudaGraphNode_t, const cudaMemsetParams *) {
    return cudaErrorNotSupported;
}
static inline cudaError_t cudaGraphExecMemcpyNodeSetParams1D(cudaGraphExec_t, cudaGraphNode_t, void *, const void *,
                                                             size_t, cudaMemcpyKind) {
    return cudaErrorNotSupported;
}
static inline cudaError_t cudaGraphExecEventRecordNodeSetEvent(cudaGraphExec_t, cudaGraphNode_t, cudaEvent_t) {
    return cudaErrorNotSupported;
}
static inline cudaError_t cudaGraphMemsetNodeGetParams(cudaGraphNode_t, cudaMemsetParams *) {
    return cudaErrorNotSupported;
}
static inline cudaError_t cudaLaunchKernel(const void *, dim3, dim3, void **, size_t, cudaStream_t) {
    return cudaErrorNotSupported;  // kernels launch through the host launchers
}
