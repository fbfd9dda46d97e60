// Internal types and device helpers of the GB300 G-VOM path.
//
// Data layout in device memory (one map instance):
//   per ring slot   idx  int32[V]        voxel id -> compact index (>=0), -1 unknown,
//                                        <= -2 free with -(v+1) pass-throughs
//                   rec  VoxelRec[cap]   per occupied voxel statistics (64 B)
//   combined (x2)   cidx int32[V], crec VoxelRec[V] (double-buffered: current / previous)
//   per scan scratch cnt  u64[Vext]      dense (hit << 32 | total) over the grid plus the
//                                        eigen-neighbourhood halo; zero between scans
//                   prec float4[N]       per point: voxel fraction xyz + extended cell id
//                   prank int32[N]       per point: rank inside its cell
//                   sorted float4[N]     points grouped by cell
//   2-D maps        height/inferred/slope/roughness/guess f64[X*X], pos/neg/vis int32[X*X]
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#ifdef __CUDACC__
#include <type_traits>
#include <vector>
#endif

#include "gvom_exact.cuh"

namespace gvom {

#ifdef __CUDACC__  // (the host-compiled kernel tests include this header without the CUDA runtime)
// ---------------------------------------------------------------------------
// Stream-ordered work in graph mode.  The launch sequences of a process,
// combine or step call go through the rec_* helpers below.  Without graphs
// they launch directly.  The first time a sequence runs in graph mode it is
// captured (the helpers launch into the capture and note each node they
// add, in order); later calls of the same shape do not capture again: the
// helpers write the new parameters (kernel arguments and grid, memset and
// copy addresses, events) into the executable graph's nodes in the same
// order.  A call whose sequence differs (another kernel at a position, more
// or fewer nodes) is captured anew.
// ---------------------------------------------------------------------------
struct GraphNodes {
    cudaGraph_t graph = nullptr;      // the graph `exec` was instantiated from (owns the nodes)
    cudaGraphExec_t exec = nullptr;
    std::vector<cudaGraphNode_t> nodes;
    std::vector<const void *> tags;   // per node: kernel function, or the kind of operation
    std::vector<cudaMemsetParams> mset;  // per node: memset parameters at capture (other nodes: unused)
    std::vector<long long> arg;       // per node: memset size and value, copy size, or recorded event
};

struct Recorder {
    int mode = 0;             // 0 launch directly, 1 capture (and note nodes), 2 write into g's nodes
    GraphNodes *g = nullptr;
    size_t next = 0;          // next node (mode 2)
    bool ok = true;           // mode 2: every operation matched its node and was written
};

// the recorder of the calling thread (calls on one instance are serialised)
Recorder &recorder();

// capture mode: notes the node the last operation on `st` added
cudaError_t rec_note(cudaStream_t st, const void *tag);
// update mode: the next node if it carries `tag`, else nullptr (and the update fails)
cudaGraphNode_t rec_take(const void *tag);

template <typename... P>
cudaError_t rec_kernel(void (*fn)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       std::decay_t<P>... args) {
    void *ptrs[] = {static_cast<void *>(&args)...};
    Recorder &r = recorder();
    if (r.mode == 2) {
        cudaGraphNode_t n = rec_take(reinterpret_cast<const void *>(fn));
        if (!n) return cudaSuccess;
        cudaKernelNodeParams kp = {};
        kp.func = reinterpret_cast<void *>(fn);
        kp.gridDim = grid;
        kp.blockDim = block;
        kp.sharedMemBytes = (unsigned)smem;
        kp.kernelParams = ptrs;
        if (cudaGraphExecKernelNodeSetParams(r.g->exec, n, &kp) != cudaSuccess) {
            cudaGetLastError();
            r.ok = false;
        }
        return cudaSuccess;
    }
    cudaError_t e = cudaLaunchKernel(reinterpret_cast<const void *>(fn), grid, block, ptrs, smem, st);
    if (e == cudaSuccess && r.mode == 1) e = rec_note(st, reinterpret_cast<const void *>(fn));
    return e;
}

cudaError_t rec_memset(void *p, int value, size_t bytes, cudaStream_t st);
cudaError_t rec_memcpy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st);
// an event recorded for waits outside the graph (an event-record node in graph mode)
cudaError_t rec_event_external(cudaEvent_t ev, cudaStream_t st);
// a fork / join inside one sequence (edges of the graph, nothing to write in update mode)
cudaError_t rec_event_internal(cudaEvent_t ev, cudaStream_t st);
cudaError_t rec_wait_internal(cudaStream_t st, cudaEvent_t ev);
#endif


constexpr int kMaxBatch = 16;         // scans per batched launch

// Launch-shape choices of the autotuner (each affects its own kernels only).
struct Tuning {
    int pts_block;      // points per block of the point-parallel kernels: 128 or 256
    int merge_planes;   // z planes per k_merge thread: 4, 8 or 16
    int stats_bpsm;     // k_merge_stats blocks per multiprocessor: 2, 4 or 8
    int step_overlap;   // gvom_step runs the index merge beside the statistics kernels: 0 or 1
    int maps_tile;      // k_maps2d tile: 256 (8 x 32), 224 (14 x 16), 128 (8 x 16) or 64 (4 x 16) cells
    int step_pipeline;  // gvom_step: 0 one stream; 1 the trace beside the previous step's combine; 2 also the
                        // rest of the process and the merge beside the previous step's columns and maps
};
constexpr Tuning kDefaultTuning = {256, 8, 4, 1, 224, 2};
constexpr int kCube = 16;             // shared-memory cube of ray-step counts (cells per axis)
constexpr int kCubeCells = kCube * kCube * kCube;
constexpr int kMaxSources = 17;       // ring slots (<= 16) + previous combined map
// physical slots of an instance: the ring's B plus spares, so that a step's
// scans are traced into slots that the combines still in flight do not read
constexpr int kMaxPhysSlots = (kMaxSources - 1) + 2 * kMaxBatch;

// Per-voxel record.  Ring slots store aux[0] = voxel id (int bits); the
// combined map stores the three eigenvalues (descending) in aux.
struct __align__(16) VoxelRec {
    float mean[3];   // mean of the neighbourhood points, voxel units, relative to the voxel corner
    float cov[6];    // xx xy xz yy yz zz
    float count;     // points in the neighbourhood
    int hit;
    int total;
    float min_h;     // lowest point height inside the voxel, fraction of a voxel
    float aux[3];
};
static_assert(sizeof(VoxelRec) == 64, "VoxelRec must be 64 bytes");

struct Geom {
    int X, Z;      // grid
    int exy, ez;   // neighbourhood half-widths (xy_eigen_dist, z_eigen_dist)
    int Xe, Ze;    // extended grid X + 2 exy, Z + 2 ez
    long long V, Vext;
};

struct __align__(8) ScanCounters {
    int C;                      // occupied voxels allocated (k_assign reserves C and pts with one 64-bit atomic)
    int pts;                    // points placed into cell groups
    int overflow;               // capacity exceeded (should never happen)
    int pad;
    unsigned long long valid;   // points passing the finite / min-distance filter
    unsigned long long hits;    // in-grid hits
    unsigned long long steps;   // ray-march increments
};

struct ScanDesc {
    const void *pts;       // device points
    long long n, stride;   // rows, elements per row (bytes per point for PointCloud2 data)
    int pc2;               // PointCloud2 data: x, y, z at byte offsets off[] of each point, 1 float32, 2 float64
    int off[3];
    int tmode;             // 0 none, 1 float32 transform, 2 float64 transform
    int fast_floor;        // |origin| + grid < 2^22: float32 ray voxel indices (see ray_index)
    int exact_ok;          // |origin| < 2^31: integer hit-voxel arithmetic (gx_coord)
    double T[12];          // transform rows 0..2 (a float32 transform is stored exactly)
    float Tf[12];          // the same rows as float32 (exact for a float32 transform)
    double od[3];          // voxel origin (integer-valued doubles)
    int oi[3];             // the same as int (valid when exact_ok)
    float pt0[3];          // ray start: (float)(ego / resolution)
    int cube0[3];          // grid voxel of the shared-memory cube's low corner
    int cube_on;           // the cube lies inside the grid (grid >= kCube per axis)
    int slot;
    int block_begin;       // first block of this scan in point-parallel launches
    int nblocks;
    long long pt_base;     // offset of this scan in prec / prank / sorted
    unsigned long long *cnt;
    int *idx;              // slot index map
    VoxelRec *rec;         // slot records
    long long rec_cap;
    ScanCounters *ctr;
};

template <int NS>
struct ScanTable {
    ScanDesc s[NS];
};

struct ProcessConst {
    Geom g;
    double xy_res, z_res;
    double md2;            // min_distance^2
    float md2_f32;         // smallest float32 >= md2 (float32 points compare in float32)
    ExactRes rxy, rz;      // exact-division constants of xy_res / z_res
    int step_cap;          // upper bound on ray steps inside the grid
    int nscans;
    int num_sms;           // multiprocessors of the device (persistent grids)
    unsigned long long xe_magic;  // floor((2^64 - 1) / Xe) + 1 (divisions by the extended row length)
};

struct MergeSrc {
    const int *idx;
    const VoxelRec *rec;
    int dx, dy, dz;        // combined origin - source origin (voxels)
    int is_last;           // previous combined map: clearing rule (scripts/gvom.py:1058)
};

struct MergeParams {
    Geom g;
    MergeSrc src[kMaxSources];
    int nsrc;
    int *out_idx;
    VoxelRec *out_rec;     // indexed by voxel id
    int *out_count;        // occupied voxels
    int *list;             // voxel ids of the occupied voxels (capacity V)
    int num_sms;
    int planes;            // Tuning::merge_planes (z planes per k_merge thread = colinfo chunk)
    int stats_bpsm;        // Tuning::stats_bpsm
    int2 *colinfo;         // per (z chunk, y, x): lowest occupied z, lowest known-free z (Z if none)
    double co[3];          // combined origin (voxels)
};

struct ColumnParams {
    int X, Z;
    int planes;            // z planes per colinfo chunk
    const int *idx;        // combined index map
    const VoxelRec *rec;   // combined records (by voxel id)
    const int2 *colinfo;
    double co[3];          // combined origin (voxels)
    double xy_res, z_res;
    double ego[3];
    double robot_r2;       // robot_radius^2
    double disc_h;         // ego z - ground_to_lidar_height
    double pos_thr, robot_h;
    float pthr_v, robh_v;  // pos_thr / z_res, robot_height / z_res
    float base_xf, base_yf, res_f, r2_f;  // robot disc in float32: x_world - ego = base + x * res
    double *height, *inferred;
    int *pos_density;
    int *zlow;             // lowest occupied z per column (-1 if none)
    float *mlow;           // its in-voxel minimum height fraction
};

struct Maps2DParams {
    int X;
    double xy_res, z_res;
    double slope_thr, neg_thr;
    float slope_thr_f;
    const double *height, *inferred;
    const int *pos_density;
    const int *zlow;
    const float *mlow;
    double *slope_x, *slope_y, *rough, *guess;
    int *pos, *neg, *vis;
    int tile_cells;        // Tuning::maps_tile_cells: 256 (8 x 32), 224 (14 x 16), 128 (8 x 16) or 64 (4 x 16)
};

struct RosGridParams {
    int X;
    const int *pos, *neg, *vis;
    const double *rough;
    double density_thr, min_r, max_r;
    signed char *hard, *soft, *certainty, *negative, *roughness;  // X * X each, x fastest; nullable
};

struct DebugVoxParams {
    const int *idx;
    const VoxelRec *rec;
    const int *block_off;
    long long V;
    int X;
    double co[3];
    double xy_res, z_res;
    float *out;
    long long cap;
};

struct DebugMapParams {
    int X;
    double co[3];
    double xy_res, z_res;
    const double *height, *rough, *slope_x, *slope_y, *guess;
    float *out_h;   // (X*X, 7) or NULL
    float *out_i;   // (X*X, 3) or NULL
};

// host launchers (k_process.cu, k_combine.cu)
// `ev` (nullable): kProcessKernels + 1 (resp. kCombineKernels + 1) events,
// recorded before the first kernel and after each kernel.
constexpr int kProcessKernels = 6;  // voxelize_trace, assign, scatter, cell_moments, voxel_stats, cleanup
constexpr int kCombineKernels = 5;  // merge, merge_counts, merge_stats, columns, maps2d
constexpr int kCellMomBytes = 48;  // per point slot (moments stored at each cell's first slot)
// `part`: 0 every kernel, 1 k_voxelize_trace only, 2 the kernels after it
// (parts are launched without stage events).  `after_assign` (nullable) is
// recorded once the slots' index maps are complete, `after_moments`
// (nullable) once the slots' records hold hit, total and min height (what
// the count merge reads); `external`: as external events (graph capture: for
// a wait outside the captured graph).  The slots' index maps must already
// hold -1 when the trace starts.
cudaError_t launch_process(const ProcessConst &pc, const ScanDesc *table, int nscans, int total_blocks, int max_n,
                           int dtype, float4 *prec, int *prank, float4 *sorted, void *moments, cudaStream_t st,
                           cudaEvent_t *ev, int pts_block, cudaEvent_t after_assign, cudaEvent_t after_moments,
                           int part = 0, bool external = false);
// load every kernel of the process / combine path now instead of at its
// first launch (CUDA's lazy module loading)
cudaError_t preload_process_kernels();
cudaError_t preload_combine_kernels();
cudaError_t launch_gather_records(const VoxelRec *rec, const int *vids, int n, VoxelRec *out, cudaStream_t st);
cudaError_t launch_merge_index(const MergeParams &mp, cudaStream_t st);
// `part`: 0 counts, statistics, columns, maps2d in sequence; 1 the count
// merge; 4 the statistics merge; 2 columns; 3 maps2d (parts are launched
// without stage events)
cudaError_t launch_combine_rest(const MergeParams &mp, const ColumnParams &cp, const Maps2DParams &m2, cudaStream_t st,
                                cudaEvent_t *ev, int part = 0);
cudaError_t launch_combine(const MergeParams &mp, const ColumnParams &cp, const Maps2DParams &m2, cudaStream_t st,
                           cudaEvent_t *ev = nullptr);
cudaError_t launch_debug_count(const int *idx, long long V, int *counts, int nblocks, cudaStream_t st);
cudaError_t launch_debug_voxels(const DebugVoxParams &p, int nblocks, cudaStream_t st);
cudaError_t launch_debug_maps(const DebugMapParams &p, cudaStream_t st);
int debug_chunk();
cudaError_t launch_ros_grids(const RosGridParams &p, cudaStream_t st);

// 2-D image kernels with no caller on the path (k_morph.cu)
cudaError_t launch_expand_binary(const int32_t *in, int32_t *out, int X, double r, cudaStream_t st);
cudaError_t launch_lowpass_binary(const int32_t *in, int32_t *out, int X, int fs, double frac, cudaStream_t st);
cudaError_t launch_convolve(const double *in, double *out, const double *kern, int X, int ks, cudaStream_t st);

// allocation-free debug voxel export (k_debug_static.cu): per-block scratch of
// kStaticDebugBlocks + 1 words in a fixed device array
constexpr int kStaticDebugBlocks = 32768;
cudaError_t debug_static_scratch(int **ptr);
cudaError_t launch_debug_offsets(int *words, int n, cudaStream_t st);

// ---------------------------------------------------------------------------
// exact arithmetic helpers
// ---------------------------------------------------------------------------

// floor((double)p - od) for an integer-valued od, as the reference computes a
// ray voxel index (scripts/gvom.py:1215-1223).  For |od| < 2^24 this equals
// floor(p) - oi, except for p in (-2^-20, 0): there p - od may round to the
// integer -od itself (the float64 spacing near |od| < 2^24 is at most 2^-29,
// so for p <= -2^-20 the rounded difference stays below -od and the float32
// answer holds); that sliver takes the double path.  floor(p) for |p| < 2^22
// is read off the bits of p + 1.5 * 2^23 rounded down (the sum lies in
// [2^23, 2^24], where float32 spacing is 1).
// Returns INT_MIN for values far outside any grid (and NaN).
__device__ __forceinline__ int ray_index(float p, int oi, double od, int fast) {
    if (fast && fabsf(p) < 4194304.0f && !(p > -9.5367431640625e-07f && p < 0.0f))
        return __float_as_int(__fadd_rd(p, 12582912.0f)) - 0x4B400000 - oi;
    if (!(fabsf(p) < 1073741824.0f)) return INT32_MIN;
    if (fast && !(p > -9.5367431640625e-07f && p < 0.0f)) return __float2int_rd(p) - oi;
    double t = __dsub_rn((double)p, od);
    double f = floor(t);
    if (!(fabs(f) < 1.0e9)) return INT32_MIN;
    return (int)f;
}

// p in (-2^-20, 0): the one range where floor(p) - origin can differ from the
// reference's floor((double)p - origin) (see ray_index).  -0.0 is excluded:
// both formulas give -origin there.
__device__ __forceinline__ bool in_sliver(float p) {
    return (unsigned)__float_as_int(p) - 0x80000001u < 0x357FFFFFu;
}

// Number of iterations of `while (length < R) { ...; length += inc; }` with
// a float64 accumulator starting at 0, R = (double)rl - 1 and
// inc = |1.0 / (double)sk| (scripts/gvom.py:1206-1231), capped at `cap`.
// The accumulated rounding error of length stays below k * 2^-41 for the
// lengths that occur (< 2^11 voxels), so when R / inc is clear of an integer
// the count is ceil(R / inc).  R / inc = R |sk| (1 + O(2^-53)); R = rl - 1 is
// exact in float32 for 1 < rl < 2^23 and the float32 product adds at most
// 2^-24 relative error, so a 2^-18 relative margin decides it; otherwise the
// float64 loop's count is computed exactly in integer arithmetic
// (gx_step_count), or replayed in float64 where that declines.
__device__ __forceinline__ int ray_step_count(float rl, float sk, int cap) {
    if (!(rl > 1.0f)) return 0;  // R <= 0 (or NaN)
    if (rl < 8388608.0f) {
        const float est = __fmul_rn(__fsub_rn(rl, 1.0f), fabsf(sk));
        if (!(est < (float)cap)) return cap;
        const float fl = floorf(est);
        const float margin = 3.8147e-6f * fmaxf(est, 1.0f);  // 2^-18
        if (est - fl > margin && fl + 1.0f - est > margin) return (int)fl + 1;
    }
    const double R = __dsub_rn((double)rl, 1.0);
    const double inc = fabs(__ddiv_rn(1.0, (double)sk));
    const int Kx = gx_step_count(R, inc, cap);  // the float64 loop's count in integer arithmetic
    if (Kx >= 0) return Kx;
    double L = 0.0;
    int K = 0;
    while (L < R && K < cap) {
        K++;
        L = __dadd_rn(L, inc);
    }
    return K;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Kahan-compensated float32 accumulator.
struct KSum {
    float s, c;
    __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float v) {
        float y = __fsub_rn(v, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};

}  // namespace gvom
