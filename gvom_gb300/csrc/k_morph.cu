// 2-D image kernels of the reference that no caller launches
// (scripts/gvom.py:807-885): __expand_binary, __lowpass_binary and
// __convolve, over [x][y] images of xy_size x xy_size (y fastest, the layout
// of the 2-D maps), on the caller's device buffers and stream.
//
// Each block takes a 32 x 8 tile of output cells and stages the tile plus
// its halo (the kernel's reach) in shared memory when that fits, so every
// input cell is read from global memory once per block; otherwise the reads
// go through the read-only cache.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "gvom_internal.cuh"

namespace gvom {
namespace {

constexpr int kTX = 8, kTY = 32;      // output tile: 8 x-rows of 32 y-cells
constexpr int kMaxStage = 48 * 1024;  // shared staging, bytes

// the tile [x0 - h, x0 + kTX + h) x [y0 - h, y0 + kTY + h) of `in`, or
// `fill` outside the image
template <typename T>
__device__ void stage(const T *__restrict__ in, T *sm, int X, int x0, int y0, int h, T fill) {
    const int sx = kTX + 2 * h, sy = kTY + 2 * h;
    for (int k = threadIdx.y * kTY + threadIdx.x; k < sx * sy; k += kTX * kTY) {
        const int gx = x0 - h + k / sy, gy = y0 - h + k % sy;
        sm[k] = (gx >= 0 && gx < X && gy >= 0 && gy < X) ? __ldg(&in[(long long)gx * X + gy]) : fill;
    }
}

// __expand_binary (scripts/gvom.py:807-831): 1 where a cell equal to 1 lies
// in the disc of radius r -- rows i in [-floor(r), floor(r)], and in row i
// the columns j with |j| <= floor(sqrt(r r - i i)) (float64, as the
// reference); cells outside the image are skipped.
__global__ void __launch_bounds__(kTX * kTY) k_expand_binary(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                                            int X, double r, int h, int staged) {
    extern __shared__ int32_t sm_i[];
    const int x0 = blockIdx.y * kTX, y0 = blockIdx.x * kTY;
    if (staged) {
        stage<int32_t>(in, sm_i, X, x0, y0, h, 0);
        __syncthreads();
    }
    const int x = x0 + threadIdx.y, y = y0 + threadIdx.x;
    if (x >= X || y >= X) return;
    const int ri = (int)floor(r);
    const int sy = kTY + 2 * h;
    int v = 0;
    for (int i = -ri; i <= ri && !v; i++) {
        if (x + i < 0 || x + i >= X) continue;
        const int dy = (int)floor(sqrt(__dsub_rn(__dmul_rn(r, r), (double)(i * i))));
        for (int j = -dy; j <= dy; j++) {
            if (y + j < 0 || y + j >= X) continue;
            const int c = staged ? sm_i[(threadIdx.y + h + i) * sy + (threadIdx.x + h + j)]
                                 : __ldg(&in[(long long)(x + i) * X + (y + j)]);
            if (c == 1) {
                v = 1;
                break;
            }
        }
    }
    out[(long long)x * X + y] = v;
}

// __lowpass_binary (scripts/gvom.py:833-861): a cell equal to 0 stays 0;
// otherwise 1 where the mean of the (2 fs + 1)^2 window, clipped to the
// image, is >= filter_fraction (float64 sum and count, one division).
__global__ void __launch_bounds__(kTX * kTY) k_lowpass_binary(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                                             int X, int fs, double frac, int staged) {
    extern __shared__ int32_t sm_i[];
    const int x0 = blockIdx.y * kTX, y0 = blockIdx.x * kTY;
    if (staged) {
        stage<int32_t>(in, sm_i, X, x0, y0, fs, 0);
        __syncthreads();
    }
    const int x = x0 + threadIdx.y, y = y0 + threadIdx.x;
    if (x >= X || y >= X) return;
    const int sy = kTY + 2 * fs;
    const int self = staged ? sm_i[(threadIdx.y + fs) * sy + threadIdx.x + fs] : __ldg(&in[(long long)x * X + y]);
    int v = 0;
    if (self != 0) {
        // the reference adds the cells one by one in float64; for int32 cells
        // every partial sum of a window of at most 2^21 cells is an integer
        // below 2^53, exact in float64, so the integer sum is the same value
        long long sum = 0, cnt = 0;
        for (int i = -fs; i <= fs; i++) {
            if (x + i < 0 || x + i >= X) continue;
            for (int j = -fs; j <= fs; j++) {
                if (y + j < 0 || y + j >= X) continue;
                sum += staged ? sm_i[(threadIdx.y + fs + i) * sy + (threadIdx.x + fs + j)]
                              : __ldg(&in[(long long)(x + i) * X + (y + j)]);
                cnt++;
            }
        }
        v = __ddiv_rn((double)sum, (double)cnt) >= frac ? 1 : 0;
    }
    out[(long long)x * X + y] = v;
}

// __convolve (scripts/gvom.py:863-885) with its indexing as written: every
// term reads input[x + r, y + r] (not x + i, y + j), so an in-image cell
// sums input[x + r, y + r] times each kernel entry [0, 2r] x [0, 2r] in row
// order, and a cell whose (x + r, y + r) lies outside the image gives 0.  The
// reference computes r as a float ((kernel_size - 1) / 2) and passes it to
// range(), which cannot run; the radius here is the integer
// (kernel_size - 1) / 2 that range() would need.
__global__ void __launch_bounds__(kTX * kTY) k_convolve(const double *__restrict__ in, double *__restrict__ out,
                                                       const double *__restrict__ kern, int X, int ks) {
    const int x = blockIdx.y * kTX + threadIdx.y, y = blockIdx.x * kTY + threadIdx.x;
    if (x >= X || y >= X) return;
    const int r = (ks - 1) / 2;
    double acc = 0.0;
    if (x + r >= 0 && x + r < X && y + r >= 0 && y + r < X) {
        const double p = __ldg(&in[(long long)(x + r) * X + (y + r)]);
        for (int i = -r; i <= r; i++)
            for (int j = -r; j <= r; j++) acc = __dadd_rn(acc, __dmul_rn(p, __ldg(&kern[(i + r) * ks + (j + r)])));
    }
    out[(long long)x * X + y] = acc;
}

dim3 grid_of(int X) { return dim3((unsigned)((X + kTY - 1) / kTY), (unsigned)((X + kTX - 1) / kTX)); }

}  // namespace

cudaError_t launch_expand_binary(const int32_t *in, int32_t *out, int X, double r, cudaStream_t st) {
    const int h = r >= 0.0 ? (int)floor(r) : 0;
    const size_t smem = (size_t)(kTX + 2 * h) * (kTY + 2 * h) * sizeof(int32_t);
    const int staged = smem <= (size_t)kMaxStage;
    k_expand_binary<<<grid_of(X), dim3(kTY, kTX), staged ? smem : 0, st>>>(in, out, X, r, h, staged);
    return cudaGetLastError();
}

cudaError_t launch_lowpass_binary(const int32_t *in, int32_t *out, int X, int fs, double frac, cudaStream_t st) {
    const size_t smem = (size_t)(kTX + 2 * fs) * (kTY + 2 * fs) * sizeof(int32_t);
    const int staged = smem <= (size_t)kMaxStage;
    k_lowpass_binary<<<grid_of(X), dim3(kTY, kTX), staged ? smem : 0, st>>>(in, out, X, fs, frac, staged);
    return cudaGetLastError();
}

cudaError_t launch_convolve(const double *in, double *out, const double *kern, int X, int ks, cudaStream_t st) {
    k_convolve<<<grid_of(X), dim3(kTY, kTX), 0, st>>>(in, out, kern, X, ks);
    return cudaGetLastError();
}

}  // namespace gvom
