"""Host builds of whole kernel files for the CPU tests: the preamble that
stands in for the CUDA runtime around the library's launchers (block
emulation in tests/cpp/host_cuda/block_threads.h, CUDA's by-value integer
min / max, the intrinsics the kernels call), the rewrites a host compiler
needs (`<<<...>>>` launches, dynamic shared memory), and the compile step.
Test infrastructure only."""
import os
import re
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "gvom_gb300", "csrc")
HOST_CUDA = os.path.join(HERE, "cpp", "host_cuda")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

PRELUDE = r"""
#include <algorithm>
#include <cmath>
using std::isfinite; using std::isnan; using std::max; using std::min;
#include "cuda_runtime.h"
#include "block_threads.h"
// CUDA's integer min / max take their operands by value (a volatile read
// included)
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int max(int a, int b) { return a > b ? a : b; }
static inline long long min(long long a, long long b) { return a < b ? a : b; }
static inline long long max(long long a, long long b) { return a > b ? a : b; }
template <class T> static inline T __ldg(const T *p) { return *p; }
static inline unsigned long long __umul64hi(unsigned long long a, unsigned long long b) {
    return (unsigned long long)(((unsigned __int128)a * b) >> 64);
}
static inline float __fdividef(float a, float b) { return a / b; }
static inline float __frcp_rn(float x) { return 1.0f / x; }
static inline float rsqrtf(float x) { return 1.0f / std::sqrt(x); }
static inline int __ffs(int x) { return __builtin_ffs(x); }
constexpr cudaError_t cudaSuccess = 0;
static inline cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
static inline cudaError_t cudaGetLastError() { return cudaSuccess; }
struct cudaFuncAttributes { int unused; };
static inline cudaError_t cudaFuncGetAttributes(cudaFuncAttributes *, const void *) { return cudaSuccess; }
template <class T> static inline cudaError_t cudaGetSymbolAddress(void **p, const T &symbol) {
    *p = (void *)&symbol;  // a file-scope device array is a host array here
    return cudaSuccess;
}
#include "gvom_internal.cuh"
namespace gvom {
// a launch runs every block of the grid under the block emulator
template <typename... P>
cudaError_t rec_kernel(void (*fn)(P...), dim3 grid, dim3 block, size_t, cudaStream_t, std::decay_t<P>... args) {
    block_threads::launch(grid, block, [&] { fn(args...); });
    return cudaSuccess;
}
static inline cudaError_t rec_event_external(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
static inline cudaError_t rec_event_internal(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
}  // namespace gvom
"""


def _split_top(s):
    """Split at the commas outside parentheses."""
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
            continue
        depth += ch == "("
        depth -= ch == ")"
        cur += ch
    parts.append(cur.strip())
    return parts


def host_source(src):
    """A kernel file's text as a host compiler takes it: each direct launch
    `k<<<grid, block, smem, stream>>>(args)` becomes
    `rec_kernel(k, dim3(grid), dim3(block), smem, stream, args)`, and each
    dynamic shared array `extern __shared__ T a[];` a static of the file's
    kMaxStage bytes."""
    def launch(m):
        parts = _split_top(m.group(2))
        assert len(parts) == 4, m.group(0)
        return f"rec_kernel({m.group(1)}, dim3({parts[0]}), dim3({parts[1]}), {parts[2]}, {parts[3]}, "
    out = re.sub(r"(\w+(?:<[^<>;]*>)?)<<<(.*?)>>>\(", launch, src)
    out = re.sub(r"extern __shared__ (\w+) (\w+)\[\];", r"static \1 \2[kMaxStage / sizeof(\1)];", out)
    return out


def compile_units(units, out_dir, name):
    """Compile {file name: source text} in parallel and link them into one
    shared library; returns its path."""
    # (no _FORTIFY_SOURCE: the block emulator's fibers switch stacks with _longjmp)
    flags = ["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-frounding-math", "-fPIC", "-Wno-unknown-pragmas",
             "-U_FORTIFY_SOURCE", "-I", HOST_CUDA, "-I", CSRC, "-I", INCLUDE]
    for fname, text in units.items():
        (out_dir / fname).write_text(text)

    def one(fname):
        subprocess.run(flags + ["-c", str(out_dir / fname), "-o", str(out_dir / (fname + ".o"))], check=True)

    with ThreadPoolExecutor(len(units)) as ex:
        list(ex.map(one, units))
    so = out_dir / name
    subprocess.run(["g++", "-shared", "-o", str(so)] + [str(out_dir / (f + ".o")) for f in units], check=True)
    return so
