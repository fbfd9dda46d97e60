// C ABI of the GB300 G-VOM path (include/gvom_gb300.h): instance state,
// device memory, stream ordering and the host side of Gvom.__init__,
// Process_pointcloud and combine_maps (scripts/gvom.py:21-442).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gvom_gb300.h"
#include "gvom_internal.cuh"


namespace gvom {

namespace {
thread_local Recorder t_rec;
// tags of the non-kernel nodes: the addresses of three distinct bytes
const char kTags[3] = {0, 1, 2};
const void *const kTagMemset = &kTags[0];
const void *const kTagMemcpy = &kTags[1];
const void *const kTagEvent = &kTags[2];
}  // namespace

Recorder &recorder() { return t_rec; }

cudaError_t rec_note(cudaStream_t st, const void *tag) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    const cudaError_t e = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd);
    if (e != cudaSuccess) return e;
    GraphNodes &g = *t_rec.g;
    if (cs != cudaStreamCaptureStatusActive || nd != 1) {
        t_rec.ok = false;  // the sequence cannot be replayed node by node: it is captured every time
        return cudaSuccess;
    }
    g.nodes.push_back(deps[0]);
    g.tags.push_back(tag);
    g.mset.push_back(cudaMemsetParams{});
    g.arg.push_back(0);
    return cudaSuccess;
}

cudaGraphNode_t rec_take(const void *tag) {
    Recorder &r = t_rec;
    if (!r.ok || r.next >= r.g->nodes.size() || r.g->tags[r.next] != tag) {
        r.ok = false;
        return nullptr;
    }
    return r.g->nodes[r.next++];
}

cudaError_t rec_memset(void *p, int value, size_t bytes, cudaStream_t st) {
    Recorder &r = t_rec;
    if (r.mode == 2) {
        const size_t i = r.next;
        cudaGraphNode_t n = rec_take(kTagMemset);
        if (!n) return cudaSuccess;
        // the same value and size as at capture: only the address changes
        if (r.g->arg[i] != (long long)(((unsigned long long)bytes << 8) | (unsigned)(value & 0xff))) {
            r.ok = false;
            return cudaSuccess;
        }
        cudaMemsetParams mp = r.g->mset[i];
        mp.dst = p;
        if (cudaGraphExecMemsetNodeSetParams(r.g->exec, n, &mp) != cudaSuccess) {
            cudaGetLastError();
            r.ok = false;
        }
        return cudaSuccess;
    }
    cudaError_t e = cudaMemsetAsync(p, value, bytes, st);
    if (e != cudaSuccess || r.mode != 1) return e;
    const size_t before = r.g->nodes.size();
    if ((e = rec_note(st, kTagMemset)) != cudaSuccess) return e;
    if (r.g->nodes.size() > before) {
        if (cudaGraphMemsetNodeGetParams(r.g->nodes.back(), &r.g->mset.back()) != cudaSuccess) {
            cudaGetLastError();
            r.ok = false;
        }
        r.g->arg.back() = (long long)(((unsigned long long)bytes << 8) | (unsigned)(value & 0xff));
    }
    return cudaSuccess;
}

cudaError_t rec_memcpy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
    Recorder &r = t_rec;
    if (r.mode == 2) {
        const size_t i = r.next;
        cudaGraphNode_t n = rec_take(kTagMemcpy);
        if (!n) return cudaSuccess;
        if (r.g->arg[i] != (long long)bytes ||
            cudaGraphExecMemcpyNodeSetParams1D(r.g->exec, n, dst, src, bytes, kind) != cudaSuccess) {
            cudaGetLastError();
            r.ok = false;
        }
        return cudaSuccess;
    }
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, st);
    if (e != cudaSuccess || r.mode != 1) return e;
    const size_t before = r.g->nodes.size();
    if ((e = rec_note(st, kTagMemcpy)) != cudaSuccess) return e;
    if (r.g->nodes.size() > before) r.g->arg.back() = (long long)bytes;
    return cudaSuccess;
}

cudaError_t rec_event_external(cudaEvent_t ev, cudaStream_t st) {
    Recorder &r = t_rec;
    if (r.mode == 2) {
        const size_t i = r.next;
        cudaGraphNode_t n = rec_take(kTagEvent);
        if (!n) return cudaSuccess;
        // the node's event as last written (it alternates between calls for
        // double-buffered state): rewrite it only when it changes
        if (r.g->arg[i] != (long long)(uintptr_t)ev) {
            if (cudaGraphExecEventRecordNodeSetEvent(r.g->exec, n, ev) != cudaSuccess) {
                cudaGetLastError();
                r.ok = false;
            } else {
                r.g->arg[i] = (long long)(uintptr_t)ev;
            }
        }
        return cudaSuccess;
    }
    if (r.mode == 0) return cudaEventRecord(ev, st);
    cudaError_t e = cudaEventRecordWithFlags(ev, st, cudaEventRecordExternal);
    if (e != cudaSuccess) return e;
    const size_t before = r.g->nodes.size();
    if ((e = rec_note(st, kTagEvent)) != cudaSuccess) return e;
    if (r.g->nodes.size() > before) r.g->arg.back() = (long long)(uintptr_t)ev;
    return cudaSuccess;
}

cudaError_t rec_event_internal(cudaEvent_t ev, cudaStream_t st) {
    return t_rec.mode == 2 ? cudaSuccess : cudaEventRecord(ev, st);
}

cudaError_t rec_wait_internal(cudaStream_t st, cudaEvent_t ev) {
    return t_rec.mode == 2 ? cudaSuccess : cudaStreamWaitEvent(st, ev, 0);
}

}  // namespace gvom

using namespace gvom;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

// combine_maps' four outputs, one block on the device (see gvom_create)
constexpr size_t kOutBytesPerCell = 8 + 3 * 4;  // roughness (f64), positive, negative, visibility (i32)

#define CUDA_TRY(expr)                                                                         \
    do {                                                                                       \
        cudaError_t e__ = (expr);                                                              \
        if (e__ != cudaSuccess)                                                                \
            return fail(GVOM_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e__));   \
    } while (0)

constexpr int kStages = kProcessKernels + kCombineKernels;
const char *kStageNames[kStages] = {"k_voxelize_trace", "k_assign", "k_scatter",     "k_cell_moments",
                                    "k_voxel_stats",    "k_cleanup", "k_merge",       "k_merge_counts",
                                    "k_merge_stats",    "k_columns", "k_maps2d"};

// CUDA events around each kernel launch, harvested when the host waits.
struct StageTimer {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    struct Pending {
        int first, nk;
        cudaEvent_t ev[kProcessKernels + 1];
    };
    std::vector<Pending> pending;
    double ms[kStages] = {0};
    long long n[kStages] = {0};

    cudaEvent_t get() {
        if (pool.empty()) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
            return e;
        }
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    // returns an event array for `nk` kernels starting at stage `first`, or nullptr when off
    cudaEvent_t *begin(int first, int nk) {
        if (!on) return nullptr;
        if (pending.size() >= 512) harvest();
        Pending p;
        p.first = first;
        p.nk = nk;
        for (int i = 0; i <= nk; i++) {
            p.ev[i] = get();
            if (!p.ev[i]) return nullptr;
        }
        pending.push_back(p);
        return pending.back().ev;
    }
    void harvest() {
        for (auto &p : pending) {
            cudaEventSynchronize(p.ev[p.nk]);
            for (int i = 0; i < p.nk; i++) {
                float t = 0.f;
                if (cudaEventElapsedTime(&t, p.ev[i], p.ev[i + 1]) == cudaSuccess) {
                    ms[p.first + i] += t;
                    n[p.first + i] += 1;
                }
            }
            for (int i = 0; i <= p.nk; i++) pool.push_back(p.ev[i]);
        }
        pending.clear();
        cudaGetLastError();
    }
    void reset() {
        harvest();
        for (int i = 0; i < kStages; i++) {
            ms[i] = 0;
            n[i] = 0;
        }
    }
    ~StageTimer() {
        for (auto &p : pending)
            for (int i = 0; i <= p.nk; i++) cudaEventDestroy(p.ev[i]);
        for (auto e : pool) cudaEventDestroy(e);
    }
};

struct Slot {
    int *idx = nullptr;
    VoxelRec *rec = nullptr;
    long long cap = 0;
    double od[3] = {0, 0, 0};
    bool valid = false;
};

// combine-done events kept per instance (a ring): event e % kCombEvents marks
// the end of combine e's last reader of the ring slots (its statistics merge)
constexpr int kCombEvents = 8;

// Makes the instance's device current for the duration of an entry point and
// restores the caller's device afterwards.
struct DeviceScope {
    int prev = -1;
    bool switched = false;
    explicit DeviceScope(int dev) {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) switched = cudaSetDevice(dev) == cudaSuccess;
        cudaGetLastError();
    }
    ~DeviceScope() {
        if (switched) cudaSetDevice(prev);
    }
};

}  // namespace

struct GvomHandle {
    GvomParams p;
    Geom g;
    int B = 0;
    int dev = 0;  // the device the instance was created on
    cudaStream_t own = nullptr, st = nullptr;
    std::mutex mu;
    // physical slots: the B the ring needs plus spares (up to kMaxPhysSlots).
    // phys_of maps a ring position to the physical slot of its scan (-1: none
    // yet); free_q holds the physical slots the ring does not reference, the
    // longest unreferenced first.  A scan takes the head of free_q, so with
    // enough spares it is traced into a slot that no combine still in flight
    // reads; slot_epoch (the last combine that read a slot) and ev_cdone make
    // that ordering explicit whatever the number of spares.
    std::vector<Slot> slots;
    long long buffer_index = 0, last_buffer_index = 0;  // the reference's ring positions (mod B)
    std::vector<int> phys_of;
    std::deque<int> free_q;
    std::vector<long long> slot_epoch;
    long long n_comb = 0;                // combines submitted
    cudaEvent_t ev_cdone[kCombEvents] = {};
    long long scans_total = 0;
    double ego[3] = {0, 0, 0};
    // combined map, double buffered (current / previous)
    int *cidx[2] = {nullptr, nullptr};
    VoxelRec *crec[2] = {nullptr, nullptr};
    double cod[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int cur = 0;
    bool have_comb = false;
    // per-scan scratch, in two sets used by alternate process calls (a step's
    // trace fills one set while the previous step's process reads the other)
    std::vector<unsigned long long *> cnt[2];  // one dense count array per concurrent scan
    float4 *prec[2] = {nullptr, nullptr};
    int *prank[2] = {nullptr, nullptr};
    float4 *sorted = nullptr;
    int sset = 0;  // scratch set of the next process call
    char *moments = nullptr;  // per point slot, kCellMomBytes each
    long long pcap = 0;
    void *dpts = nullptr;
    size_t dpts_bytes = 0;
    ScanCounters *d_ctr = nullptr;  // 2 x kMaxBatch (one block per scratch set)
    int *d_slotC = nullptr;         // per ring slot occupied count
    int *d_combC = nullptr;         // [0..1] occupied count per combined buffer, [2] float64 eigen refinements
    int last_ctr = -1;              // counters of the last processed scan
    // 2-D maps
    double *height = nullptr, *inferred = nullptr, *slope_x = nullptr, *slope_y = nullptr, *rough = nullptr,
           *guess = nullptr;
    int *pos_density = nullptr, *pos = nullptr, *neg = nullptr, *vis = nullptr;
    int *zlow = nullptr;
    float *mlow = nullptr;
    int2 *colinfo[2] = {nullptr, nullptr};  // (Z / 8 chunks) x X x X, one per combined buffer
    int *occ_list[2] = {nullptr, nullptr};  // occupied voxel ids of each combined buffer (V)
    bool have_maps = false;
    // debug
    int *d_dbg = nullptr;
    int8_t *d_ros = nullptr;  // staging of the five OccupancyGrid payloads
    long long bytes = 0;
    int pageable_access = 0;
    int num_sms = 1;
    Tuning tun = kDefaultTuning;
    StageTimer timer;
    // CUDA graphs: each process / combine launch sequence is captured once
    // per shape and replayed through an executable graph whose nodes take
    // the parameters of each later call (see Recorder)
    bool graphs = false;
    // [0] process, [1] combine, [2] step, [3] a pipelined step's trace, [4] its process rest (+ the combine
    // at level 1), [5] its columns and maps, [6] its count merge (level 2), [7] its index merge (level 2),
    // [8] its statistics merge (level 2); each up to kGraphCache executables, one per shape (number of
    // scans, merge source count), most recently used first
    std::vector<GraphNodes> gn[9];
    // a step forks the index merge onto `side` once the index maps are done
    // (ev_idx), and the count merge once the records' hit, total and min
    // height are (ev_mom, after the cell moments)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_idx = nullptr, ev_mom = nullptr, ev_join = nullptr;
    // the last call was a process that recorded ev_idx and ev_mom, so a
    // combine that follows may overlap its tail
    bool proc_events = false;
    // step pipeline (Tuning::step_pipeline): a step stages its points and
    // runs k_voxelize_trace on `tr` as soon as the process call that last used
    // its scratch set (the one before the previous call) is done with it
    // (ev_scratch[set]).  At level 1 the rest of the step follows on the
    // instance stream after ev_traced.  At level 2 the rest of the process
    // runs on `bs` after ev_traced; on `side`, the index merge after ev_idx
    // (and after the columns pass that last read the combined buffer it
    // writes, ev_cols[buffer]), the count merge after ev_mom and the
    // statistics merge after ev_scratch[set]; the columns and maps on the
    // instance stream after ev_merged, beside the next step's process.  Work
    // queued on the instance stream by other calls sets st_dirty: the next
    // level-2 step first orders `tr`, `bs` and `side` after it (ev_host).
    cudaStream_t tr = nullptr, bs = nullptr;
    // the statistics merge runs beside the columns and maps: on `side` after
    // the count merge (ev_ms) and joined at the end of a combine (ev_msj), or
    // at level 2 as its own graph, ev_stats[buffer] marking its end.  A
    // combine that follows a process swaps the roles (launch_comb): `side`
    // runs the merges, columns and maps, and ev_msj joins them back.
    cudaEvent_t ev_ms = nullptr, ev_msj = nullptr, ev_stats[2] = {nullptr, nullptr};
    cudaEvent_t ev_scratch[2] = {nullptr, nullptr};  // the process call that last used the set is done with it
    cudaEvent_t ev_traced = nullptr, ev_merged = nullptr, ev_host = nullptr;
    cudaEvent_t ev_cols[2] = {nullptr, nullptr};
    bool st_dirty = false;
};

namespace {

int dalloc(GvomHandle *h, void **p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(GVOM_ERR_OOM, std::string("device allocation of ") + std::to_string(bytes) +
                                      " bytes failed: " + cudaGetErrorString(e));
    }
    h->bytes += (long long)bytes;
    return GVOM_OK;
}

template <typename T>
int dalloc_t(GvomHandle *h, T **p, size_t n) {
    return dalloc(h, reinterpret_cast<void **>(p), n * sizeof(T));
}

void dfree(GvomHandle *h, void *p, size_t bytes) {
    if (p) {
        cudaFree(p);
        h->bytes -= (long long)bytes;
    }
}

long long ext_cells(const Geom &g) { return (long long)g.Xe * g.Xe * g.Ze; }

// Runs `enqueue` (stream-ordered work through the rec_* helpers, no
// allocation and no host synchronisation) directly, or in graph mode as the
// executable graph `which`: when that graph exists, `enqueue` writes this
// call's parameters into its nodes and the graph is launched; when it does
// not, or the sequence differs in shape, `enqueue` is captured into a new
// executable graph, which replaces the old one.
// executables kept per launch sequence: a step's trace and process graphs hold
// one fill or copy node per scan, so each batch size (1-16) is its own shape
constexpr size_t kGraphCache = 16;

template <class F>
int run_graphed(GvomHandle *h, int which, F &&enqueue, cudaStream_t st = nullptr) {
    if (!st) st = h->st;
    Recorder &r = recorder();
    if (!h->graphs) {
        r = Recorder{};
        return enqueue();
    }
    // the first cached executable whose nodes take this call's operations in
    // order is updated in place and launched (a request loop alternating
    // between batch sizes keeps one executable per size instead of capturing
    // again at every change)
    std::vector<GraphNodes> &cache = h->gn[which];
    for (size_t i = 0; i < cache.size(); i++) {
        GraphNodes &G = cache[i];
        r = Recorder{};
        r.mode = 2;
        r.g = &G;
        const int rc = enqueue();
        const bool done = r.ok && r.next == G.nodes.size();
        r = Recorder{};
        if (rc) return rc;
        if (done) {
            if (i) std::rotate(cache.begin(), cache.begin() + (long)i, cache.begin() + (long)i + 1);
            CUDA_TRY(cudaGraphLaunch(cache[0].exec, st));
            return GVOM_OK;
        }
    }
    GraphNodes fresh;
    r = Recorder{};
    r.mode = 1;
    r.g = &fresh;
    const cudaError_t eb = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (eb != cudaSuccess) {
        r = Recorder{};
        cudaGetLastError();
        return fail(GVOM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(eb));
    }
    const int rc = enqueue();
    const bool noted = r.ok;
    r = Recorder{};
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(st, &g);
    if (rc || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return rc ? rc : fail(GVOM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    }
    cudaGraphExec_t x = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&x, g, cudaGraphInstantiateFlagUseNodePriority);
    if (ei != cudaSuccess) {
        cudaGraphDestroy(g);
        cudaGetLastError();
        return fail(GVOM_ERR_CUDA, std::string("graph instantiation: ") + cudaGetErrorString(ei));
    }
    // the least recently used executable beyond the cache's size is freed (an
    // executable graph still running is freed when it completes)
    if (cache.size() >= kGraphCache) {
        if (cache.back().exec) cudaGraphExecDestroy(cache.back().exec);
        if (cache.back().graph) cudaGraphDestroy(cache.back().graph);
        cache.pop_back();
    }
    cache.insert(cache.begin(), std::move(fresh));
    GraphNodes &G = cache[0];
    G.graph = g;
    G.exec = x;
    if (!noted) {  // nodes not all noted: later calls capture again
        G.nodes.clear();
        G.tags.clear();
        G.mset.clear();
        G.arg.clear();
        G.nodes.push_back(nullptr);
        G.tags.push_back(nullptr);
    }
    CUDA_TRY(cudaGraphLaunch(G.exec, st));
    return GVOM_OK;
}

int check_params(const GvomParams *p) {
    if (!p) return fail(GVOM_ERR_ARG, "params is NULL");
    if (p->xy_size <= 0 || p->z_size <= 0 || p->buffer_size <= 0)
        return fail(GVOM_ERR_ARG, "xy_size, z_size and buffer_size must be positive");
    if (p->buffer_size > kMaxSources - 1)
        return fail(GVOM_ERR_ARG, "buffer_size above " + std::to_string(kMaxSources - 1) + " is not supported");
    if (!(p->xy_resolution > 0) || !(p->z_resolution > 0))
        return fail(GVOM_ERR_ARG, "resolutions must be positive");
    if (p->xy_eigen_dist < 0 || p->z_eigen_dist < 0 || p->xy_eigen_dist > 8 || p->z_eigen_dist > 8)
        return fail(GVOM_ERR_ARG, "eigen distances must be in [0, 8]");
    const long long V = (long long)p->xy_size * p->xy_size * p->z_size;
    const long long Vext = (long long)(p->xy_size + 2 * p->xy_eigen_dist) * (p->xy_size + 2 * p->xy_eigen_dist) *
                           (p->z_size + 2 * p->z_eigen_dist);
    if (V >= (1LL << 31) - 1 || Vext >= (1LL << 31) - 1)
        return fail(GVOM_ERR_ARG, "grid too large (voxel count must fit int32)");
    return GVOM_OK;
}

// grow the point scratch so that `n` points fit
int ensure_points(GvomHandle *h, long long n) {
    if (n <= h->pcap) return GVOM_OK;
    long long cap = std::max<long long>(n, h->pcap * 2);
    cap = std::max<long long>(cap, 4096);
    if (cap >= (1LL << 31)) return fail(GVOM_ERR_ARG, "too many points");
    CUDA_TRY(cudaStreamSynchronize(h->st));
    for (int b = 0; b < 2; b++) {
        dfree(h, h->prec[b], h->pcap * sizeof(float4));
        dfree(h, h->prank[b], h->pcap * sizeof(int));
        h->prec[b] = nullptr;
        h->prank[b] = nullptr;
    }
    dfree(h, h->sorted, h->pcap * sizeof(float4));
    dfree(h, h->moments, h->pcap * kCellMomBytes);
    h->sorted = nullptr;
    h->moments = nullptr;
    h->pcap = 0;
    int rc;
    for (int b = 0; b < 2; b++)
        if ((rc = dalloc_t(h, &h->prec[b], cap)) || (rc = dalloc_t(h, &h->prank[b], cap))) return rc;
    if ((rc = dalloc_t(h, &h->sorted, cap)) || (rc = dalloc(h, reinterpret_cast<void **>(&h->moments), (size_t)cap * kCellMomBytes)))
        return rc;
    h->pcap = cap;
    return GVOM_OK;
}

int ensure_dpts(GvomHandle *h, size_t bytes) {
    if (bytes <= h->dpts_bytes) return GVOM_OK;
    size_t cap = std::max(bytes, h->dpts_bytes * 2);
    CUDA_TRY(cudaStreamSynchronize(h->st));
    dfree(h, h->dpts, h->dpts_bytes);
    h->dpts = nullptr;
    h->dpts_bytes = 0;
    int rc = dalloc(h, &h->dpts, cap);
    if (rc) return rc;
    h->dpts_bytes = cap;
    return GVOM_OK;
}

int ensure_cnt(GvomHandle *h, int nscans, int set) {
    while ((int)h->cnt[set].size() < nscans) {
        unsigned long long *c = nullptr;
        const long long ve = ext_cells(h->g);
        int rc = dalloc_t(h, &c, (size_t)ve);
        if (rc) return rc;
        CUDA_TRY(cudaMemsetAsync(c, 0, (size_t)ve * 8, h->st));
        // complete before a pipelined trace on another stream adds into it
        CUDA_TRY(cudaStreamSynchronize(h->st));
        h->cnt[set].push_back(c);
    }
    return GVOM_OK;
}

int ensure_slot(GvomHandle *h, int s, long long need) {
    Slot &sl = h->slots[s];
    need = std::min<long long>(need, h->g.V);
    need = std::max<long long>(need, 1);
    if (sl.cap >= need) return GVOM_OK;
    long long cap = std::min<long long>(h->g.V, std::max<long long>(need, sl.cap * 2));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    dfree(h, sl.rec, sl.cap * sizeof(VoxelRec));
    sl.rec = nullptr;
    sl.cap = 0;
    int rc = dalloc_t(h, &sl.rec, (size_t)cap);
    if (rc) return rc;
    sl.cap = cap;
    return GVOM_OK;
}

// a spare physical slot (its index map; records grow on demand), first in
// the free queue: it has never been read
int add_slot(GvomHandle *h) {
    Slot s;
    int rc = dalloc_t(h, &s.idx, (size_t)h->g.V);
    if (rc) return rc;
    h->slots.push_back(s);
    h->slot_epoch.push_back(-1);
    h->free_q.push_front((int)h->slots.size() - 1);
    return GVOM_OK;
}

// Stream `s` waits until no combine still reads the physical slots `slot_of`
// (the end of the last combine that read each, ev_cdone).  A slot read by
// combine e was read by no later combine than the one that last recorded
// ev_cdone[e % kCombEvents], so the wait is never short.
int wait_slots_free(GvomHandle *h, const int *slot_of, int k, cudaStream_t s) {
    for (int i = 0; i < k; i++) {
        const long long e = h->slot_epoch[slot_of[i]];
        if (e >= 0) CUDA_TRY(cudaStreamWaitEvent(s, h->ev_cdone[e % kCombEvents], 0));
    }
    return GVOM_OK;
}

// marks the end of the combine just submitted on stream `s` (after its
// statistics merge, the last kernel that reads the ring slots)
int comb_done(GvomHandle *h, cudaStream_t s) {
    CUDA_TRY(cudaEventRecord(h->ev_cdone[h->n_comb % kCombEvents], s));
    h->n_comb++;
    return GVOM_OK;
}

void ray_origin(const GvomHandle *h, const double ego[3], double od[3]) {
    // scripts/gvom.py:138-141
    od[0] = std::floor((ego[0] / h->p.xy_resolution) - (double)h->g.X / 2.0);
    od[1] = std::floor((ego[1] / h->p.xy_resolution) - (double)h->g.X / 2.0);
    od[2] = std::floor((ego[2] / h->p.z_resolution) - (double)h->g.Z / 2.0);
}

int bytes_of(int dtype) { return dtype == GVOM_F64 ? 8 : 4; }

// Constants for the exact integer division by a voxel size r > 0:
// r = mr 2^er (53-bit mr), W = floor(2^116 / mr) (gvom_exact.cuh).
ExactRes exact_res(double r) {
    int e;
    const double f = std::frexp(r, &e);
    ExactRes R;
    R.mr = (unsigned long long)std::ldexp(f, 53);
    R.er = e - 53;
    unsigned __int128 w = ((unsigned __int128)1 << 116) / R.mr;
    if (w >> 64) w = ~0ull;
    R.W = (unsigned long long)w;
    R.pad = 0;
    return R;
}

struct ScanIn {
    const void *dev_pts;
    int dtype, tdtype;
    long long n, stride;
    double ego[3];
    double T[16];
    int pc2 = 0;           // PointCloud2 bytes: stride = point step in bytes, float32 fields at off[]
    int off[3] = {0, 0, 0};
};

// Enqueue the per-scan pipeline for `k` scans whose points are in device memory.
// A process call in three parts: host preparation (allocation, scan table),
// the stream-ordered launches, and the host ring bookkeeping.
struct ProcPlan {
    ProcessConst pc;
    ScanDesc table[kMaxBatch];
    int k = 0, block = 0, max_n = 0, dtype = GVOM_F32;
    int set = 0;  // scratch set
    // ring positions of a batch's dropped scans (those a later scan of the
    // same batch overwrites): the plan's scans take the positions after them,
    // where one call per scan would have put them
    int skip = 0;
    int slot_of[kMaxBatch];
    double last_ego[3];
    std::deque<int> free_before;  // the free queue before this plan took its slots
};

// Physical slots for the plan's scans.  Scan i overwrites ring position
// (buffer_index + skip + i) mod B: the slot that position held joins the back of
// the free queue, and the scan takes the head (the slot unreferenced the
// longest).  While fewer than `spare` + 1 slots are free, a spare slot is
// added first (up to kMaxPhysSlots; without memory the plan goes on with
// fewer spares, still correct through wait_slots_free).  Pipelined steps ask
// for two steps' worth of spares, so the head was last read two combines back.
void take_slots(GvomHandle *h, ProcPlan &pl, int spare) {
    pl.free_before = h->free_q;
    for (int i = 0; i < pl.k; i++) {
        const int pos = (int)((h->buffer_index + pl.skip + i) % h->B);
        if (h->phys_of[pos] >= 0) h->free_q.push_back(h->phys_of[pos]);
        while ((int)h->free_q.size() < spare + 1 && (int)h->slots.size() < kMaxPhysSlots) {
            if (add_slot(h)) {
                cudaGetLastError();
                break;
            }
        }
        pl.slot_of[i] = h->free_q.front();
        h->free_q.pop_front();
    }
}

// undoes take_slots when the plan is dropped before commit_scans
void release_slots(GvomHandle *h, ProcPlan &pl) { h->free_q = pl.free_before; }

int prepare_scans(GvomHandle *h, const std::vector<ScanIn> &scans, ProcPlan &pl, int spare = 0, int skip = 0) {
    const int k = (int)scans.size();
    pl.k = k;
    pl.skip = skip;
    if (k == 0) return GVOM_OK;
    int rc;
    pl.set = h->sset;
    if ((rc = ensure_cnt(h, k, pl.set))) return rc;
    long long total_pts = 0, max_n = 0;
    for (auto &s : scans) {
        total_pts += s.n;
        max_n = std::max(max_n, s.n);
    }
    if ((rc = ensure_points(h, std::max<long long>(total_pts, 1)))) return rc;
    ProcessConst &pc = pl.pc;
    pc.g = h->g;
    pc.xy_res = h->p.xy_resolution;
    pc.z_res = h->p.z_resolution;
    pc.md2 = h->p.min_distance * h->p.min_distance;
    {
        // smallest float32 whose value is >= md2
        float f = (float)pc.md2;
        if ((double)f < pc.md2) f = std::nextafter(f, INFINITY);
        while ((double)std::nextafter(f, -INFINITY) >= pc.md2) f = std::nextafter(f, -INFINITY);
        pc.md2_f32 = f;
        pc.rxy = exact_res(h->p.xy_resolution);
        pc.rz = exact_res(h->p.z_resolution);
    }
    pc.step_cap = 2 * std::max(h->g.X, h->g.Z) + 8;
    pc.num_sms = h->num_sms;
    pc.xe_magic = ~0ull / (unsigned long long)h->g.Xe + 1ull;
    pc.nscans = k;
    ScanDesc *table = pl.table;
    std::memset(pl.table, 0, sizeof(pl.table));
    int block = 0;
    long long base = 0;
    take_slots(h, pl, spare);
    int *slot_of = pl.slot_of;
    for (int i = 0; i < k; i++) {
        const ScanIn &s = scans[i];
        const int slot = slot_of[i];
        if ((rc = ensure_slot(h, slot, s.n))) {
            release_slots(h, pl);
            return rc;
        }
        ScanDesc &d = table[i];
        d.pts = s.dev_pts;
        d.n = s.n;
        d.stride = s.stride;
        d.pc2 = s.pc2;
        for (int a = 0; a < 3; a++) d.off[a] = s.off[a];
        d.tmode = s.tdtype == GVOM_NONE ? 0 : (s.tdtype == GVOM_F32 ? 1 : 2);
        for (int r = 0; r < 12; r++) {
            d.T[r] = s.T[r];
            d.Tf[r] = (float)s.T[r];
        }
        ray_origin(h, s.ego, d.od);
        // ray positions stay within one step of the grid, so for
        // |origin| + grid + 2 < 2^22 every position the march visits is below
        // 2^22 in magnitude (the float32 floor of ray_index applies)
        bool fast = true, exact = true;
        const double lim = 4194304.0 - (double)std::max(h->g.X, h->g.Z) - 2.0;
        for (int a = 0; a < 3; a++) {
            if (!(std::fabs(d.od[a]) < 2147483648.0)) exact = false;
            if (!(std::fabs(d.od[a]) < lim)) fast = false;
        }
        for (int a = 0; a < 3; a++) d.oi[a] = exact ? (int)d.od[a] : 0;
        d.fast_floor = fast ? 1 : 0;
        d.exact_ok = exact ? 1 : 0;
        d.pt0[0] = (float)(s.ego[0] / h->p.xy_resolution);
        d.pt0[1] = (float)(s.ego[1] / h->p.xy_resolution);
        d.pt0[2] = (float)(s.ego[2] / h->p.z_resolution);
        // shared-memory cube of ray-step counts around the ego voxel, clamped
        // into the grid (any placement is valid; near the ego is where every
        // ray passes)
        d.cube_on = (fast && h->g.X >= kCube && h->g.Z >= kCube) ? 1 : 0;
        for (int a = 0; a < 3; a++) {
            const int dim = a < 2 ? h->g.X : h->g.Z;
            int c = 0;
            if (d.cube_on) {
                const double ev = std::floor((double)d.pt0[a] - d.od[a]);
                c = (int)std::min(std::max(ev - kCube / 2, 0.0), (double)(dim - kCube));
            }
            d.cube0[a] = c;
        }
        d.slot = slot;
        d.block_begin = block;
        d.nblocks = (int)((s.n + h->tun.pts_block - 1) / h->tun.pts_block);
        block += d.nblocks;
        d.pt_base = base;
        base += s.n;
        d.cnt = h->cnt[pl.set][i];
        d.idx = h->slots[slot].idx;
        d.rec = h->slots[slot].rec;
        d.rec_cap = h->slots[slot].cap;
        d.ctr = h->d_ctr + pl.set * kMaxBatch + i;
    }
    pl.block = block;
    pl.max_n = (int)std::min<long long>(max_n, h->g.V);
    pl.dtype = scans[0].dtype;
    for (int a = 0; a < 3; a++) pl.last_ego[a] = scans[k - 1].ego[a];
    return GVOM_OK;
}

// stream-ordered work of a prepared process call on stream `st` (default
// h->st); `after_assign` (nullable) is recorded once the ring slots' index
// maps are complete (as an external event with `assign_external`).  `part`
// as in launch_process: 1 (the trace) and 2 (the rest) split one process
// call in two.  The trace part first fills the slots' index maps with -1
// (unknown): the trace counts pass-throughs down from there.
int launch_scans(GvomHandle *h, const ProcPlan &pl, cudaEvent_t after_assign, bool timing, int part = 0,
                 cudaStream_t st = nullptr, bool external = false, cudaEvent_t after_moments = nullptr) {
    if (!st) st = h->st;
    ScanCounters *ctr = h->d_ctr + pl.set * kMaxBatch;
    if (part == 0 || part == 1) {
        CUDA_TRY(rec_memset(ctr, 0, sizeof(ScanCounters) * pl.k, st));
        for (int i = 0; i < pl.k; i++)
            CUDA_TRY(rec_memset(h->slots[pl.slot_of[i]].idx, 0xff, sizeof(int) * (size_t)h->g.V, st));
    }
    CUDA_TRY(launch_process(pl.pc, pl.table, pl.k, pl.block, pl.max_n, pl.dtype, h->prec[pl.set], h->prank[pl.set], h->sorted,
                            h->moments, st, (timing && !part) ? h->timer.begin(0, kProcessKernels) : nullptr,
                            h->tun.pts_block, after_assign, after_moments, part, external));
    if (part == 1) return GVOM_OK;
    for (int i = 0; i < pl.k; i++)
        CUDA_TRY(rec_memcpy(h->d_slotC + pl.slot_of[i], &ctr[i].C, sizeof(int), cudaMemcpyDeviceToDevice, st));
    return GVOM_OK;
}

// ring bookkeeping (scripts/gvom.py:198-216) and the latest ego (:110-112)
void commit_scans(GvomHandle *h, const ProcPlan &pl) {
    for (int i = 0; i < pl.k; i++) {
        Slot &sl = h->slots[pl.slot_of[i]];
        for (int a = 0; a < 3; a++) sl.od[a] = pl.table[i].od[a];
        sl.valid = true;
    }
    for (int a = 0; a < 3; a++) h->ego[a] = pl.last_ego[a];
    const long long b0 = h->buffer_index + pl.skip;
    for (int i = 0; i < pl.k; i++) h->phys_of[(b0 + i) % h->B] = pl.slot_of[i];
    h->last_buffer_index = (b0 + pl.k - 1) % h->B;
    h->buffer_index = (b0 + pl.k) % h->B;
    h->scans_total += pl.skip + pl.k;
    h->last_ctr = pl.set * kMaxBatch + pl.k - 1;
    h->sset = pl.set ^ 1;
}

int enqueue_scans(GvomHandle *h, const std::vector<ScanIn> &scans, int skip = 0) {
    h->st_dirty = true;  // work on the instance stream: see the step pipeline
    if (scans.empty()) return GVOM_OK;
    ProcPlan pl;
    int rc = prepare_scans(h, scans, pl, 0, skip);
    if (rc) return rc;
    if (!rc) rc = wait_slots_free(h, pl.slot_of, pl.k, h->st);
    // events for a combine that follows (see combine_impl)
    const bool events = h->tun.step_overlap && !h->timer.on;
    if (!rc)
        rc = run_graphed(h, 0, [&]() -> int {
            return launch_scans(h, pl, events ? h->ev_idx : nullptr, !h->graphs, 0, nullptr, true,
                                events ? h->ev_mom : nullptr);
        });
    if (rc) {
        release_slots(h, pl);
        return rc;
    }
    CUDA_TRY(cudaEventRecord(h->ev_scratch[pl.set], h->st));  // a later pipelined trace may reuse the set
    commit_scans(h, pl);
    h->proc_events = events;
    return GVOM_OK;
}

int fill_scan(GvomHandle *h, ScanIn &s, int dtype, long long n, long long stride, const double ego[3],
              const void *T, int tdtype) {
    if (dtype != GVOM_F32 && dtype != GVOM_F64) return fail(GVOM_ERR_ARG, "points dtype must be float32 or float64");
    if (n < 0) return fail(GVOM_ERR_ARG, "negative point count");
    if (stride < 3) return fail(GVOM_ERR_ARG, "row_stride must be >= 3");
    if (!ego) return fail(GVOM_ERR_ARG, "ego position is NULL");
    if (T && tdtype != GVOM_F32 && tdtype != GVOM_F64) return fail(GVOM_ERR_ARG, "transform dtype must be float32 or float64");
    s.dtype = dtype;
    s.n = n;
    s.stride = stride;
    for (int a = 0; a < 3; a++) s.ego[a] = ego[a];
    s.tdtype = T ? tdtype : GVOM_NONE;
    for (int r = 0; r < 16; r++) s.T[r] = 0.0;
    if (T) {
        for (int r = 0; r < 16; r++)
            s.T[r] = tdtype == GVOM_F64 ? static_cast<const double *>(T)[r] : (double)static_cast<const float *>(T)[r];
    }
    (void)h;
    return GVOM_OK;
}

bool is_pinned_host(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char *gvom_last_error(void) { return g_err.c_str(); }

const char *gvom_version(void) { return "gvom_gb300 0.1 (sm_103a)"; }

int gvom_create(const GvomParams *params, GvomHandle **out) {
    if (!out) return fail(GVOM_ERR_ARG, "out is NULL");
    *out = nullptr;
    int rc = check_params(params);
    if (rc) return rc;
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    GvomHandle *h = new GvomHandle();
    h->dev = dev;
    h->p = *params;
    Geom &g = h->g;
    g.X = params->xy_size;
    g.Z = params->z_size;
    g.exy = params->xy_eigen_dist;
    g.ez = params->z_eigen_dist;
    g.Xe = g.X + 2 * g.exy;
    g.Ze = g.Z + 2 * g.ez;
    g.V = (long long)g.X * g.X * g.Z;
    g.Vext = ext_cells(g);
    h->B = params->buffer_size;
    h->slots.resize(h->B);
    h->slot_epoch.assign(h->B, -1);
    for (int s = 0; s < h->B; s++) h->free_q.push_back(s);
    h->phys_of.assign(h->B, -1);
    cudaDeviceGetAttribute(&h->pageable_access, cudaDevAttrPageableMemoryAccess, dev);
    if (cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || h->num_sms < 1)
        h->num_sms = 1;
    // admission: the resident footprint must fit in free device memory with margin
    const long long X2 = (long long)g.X * g.X;
    const long long need = (long long)h->B * g.V * 4 + 2 * g.V * (4 + (long long)sizeof(VoxelRec)) + g.V * 4 +
                           g.Vext * 8 +
                           X2 * (6 * 8 + 4 * 4) + (64LL << 20);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return fail(GVOM_ERR_CUDA, "cudaMemGetInfo failed");
    }
    if ((long long)fr < need) {
        delete h;
        return fail(GVOM_ERR_OOM, "admission refused: instance needs " + std::to_string(need) + " bytes, " +
                                      std::to_string((long long)fr) + " free");
    }
    // the instance stream at the highest priority, the side stream (index merge
    // of a step) at the lowest: the step's critical path keeps the SMs it needs
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if (cudaStreamCreateWithPriority(&h->own, cudaStreamNonBlocking, prio_greatest) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return fail(GVOM_ERR_CUDA, "stream creation failed");
    }
    h->st = h->own;
    if (cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, prio_least) != cudaSuccess ||
        cudaStreamCreateWithPriority(&h->tr, cudaStreamNonBlocking, prio_least) != cudaSuccess ||
        cudaStreamCreateWithPriority(&h->bs, cudaStreamNonBlocking, prio_greatest) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_ms, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_msj, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_stats[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_stats[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_merged, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_host, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_cols[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_cols[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_idx, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_mom, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_scratch[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_scratch[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_traced, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        gvom_destroy(h);
        return fail(GVOM_ERR_CUDA, "stream / event creation failed");
    }
    for (auto &e : h->ev_cdone) {
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            e = nullptr;
            cudaGetLastError();
            gvom_destroy(h);
            return fail(GVOM_ERR_CUDA, "event creation failed");
        }
    }
    auto bail = [&](int code) {
        gvom_destroy(h);
        return code;
    };
    for (int s = 0; s < h->B; s++) {
        if ((rc = dalloc_t(h, &h->slots[s].idx, (size_t)g.V))) return bail(rc);
    }
    for (int b = 0; b < 2; b++) {
        if ((rc = dalloc_t(h, &h->cidx[b], (size_t)g.V))) return bail(rc);
        if ((rc = dalloc_t(h, &h->crec[b], (size_t)g.V))) return bail(rc);
    }
    // counters + scan table
    if ((rc = dalloc(h, reinterpret_cast<void **>(&h->d_ctr), sizeof(ScanCounters) * 2 * kMaxBatch)))
        return bail(rc);
    if ((rc = dalloc_t(h, &h->d_slotC, (size_t)kMaxPhysSlots))) return bail(rc);
    if ((rc = dalloc_t(h, &h->d_combC, 4))) return bail(rc);
    double **maps[5] = {&h->height, &h->inferred, &h->slope_x, &h->slope_y, &h->guess};
    for (auto m : maps)
        if ((rc = dalloc_t(h, m, (size_t)X2))) return bail(rc);
    int **imaps[2] = {&h->pos_density, &h->zlow};
    for (auto m : imaps)
        if ((rc = dalloc_t(h, m, (size_t)X2))) return bail(rc);
    // combine_maps' four outputs in one block, roughness | positive | negative |
    // visibility (kOutBytesPerCell bytes a cell), so that a caller whose host
    // buffers follow the same layout gets them in one copy
    if ((rc = dalloc(h, reinterpret_cast<void **>(&h->rough), (size_t)X2 * kOutBytesPerCell))) return bail(rc);
    h->pos = reinterpret_cast<int *>(h->rough + X2);
    h->neg = h->pos + X2;
    h->vis = h->neg + X2;
    if ((rc = dalloc_t(h, &h->mlow, (size_t)X2))) return bail(rc);
    for (int b = 0; b < 2; b++)  // chunks of >= 4 planes
        if ((rc = dalloc_t(h, &h->colinfo[b], (size_t)X2 * ((g.Z + 3) / 4)))) return bail(rc);
    for (int b = 0; b < 2; b++)
        if ((rc = dalloc_t(h, &h->occ_list[b], (size_t)g.V))) return bail(rc);
    if (cudaMemsetAsync(h->d_slotC, 0, sizeof(int) * kMaxPhysSlots, h->st) != cudaSuccess ||
        cudaMemsetAsync(h->d_combC, 0, sizeof(int) * 4, h->st) != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(GVOM_ERR_CUDA, "memset failed"));
    }
    if ((rc = ensure_cnt(h, 1, 0)) || (rc = ensure_cnt(h, 1, 1))) return bail(rc);
    // every kernel loaded now, not at its first launch inside a later call
    if (preload_process_kernels() != cudaSuccess || preload_combine_kernels() != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(GVOM_ERR_CUDA, "kernel loading failed"));
    }
    if (cudaStreamSynchronize(h->st) != cudaSuccess) {
        cudaGetLastError();
        return bail(fail(GVOM_ERR_CUDA, "initialisation failed"));
    }
    *out = h;
    return GVOM_OK;
}

int gvom_destroy(GvomHandle *h) {
    if (!h) return GVOM_OK;
    DeviceScope ds(h->dev);
    if (h->st) cudaStreamSynchronize(h->st);
    if (h->own) cudaStreamSynchronize(h->own);
    for (auto &c : h->gn)
        for (auto &x : c) {
            if (x.exec) cudaGraphExecDestroy(x.exec);
            if (x.graph) cudaGraphDestroy(x.graph);
        }
    if (h->side) {
        cudaStreamSynchronize(h->side);
        cudaStreamDestroy(h->side);
    }
    for (cudaStream_t s : {h->tr, h->bs})
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    for (cudaEvent_t e : {h->ev_merged, h->ev_host, h->ev_cols[0], h->ev_cols[1], h->ev_ms, h->ev_msj, h->ev_stats[0],
                          h->ev_stats[1]})
        if (e) cudaEventDestroy(e);
    if (h->ev_idx) cudaEventDestroy(h->ev_idx);
    if (h->ev_mom) cudaEventDestroy(h->ev_mom);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    for (cudaEvent_t e : h->ev_scratch)
        if (e) cudaEventDestroy(e);
    if (h->ev_traced) cudaEventDestroy(h->ev_traced);
    for (cudaEvent_t e : h->ev_cdone)
        if (e) cudaEventDestroy(e);
    for (auto &s : h->slots) {
        cudaFree(s.idx);
        cudaFree(s.rec);
    }
    for (int b = 0; b < 2; b++) {
        cudaFree(h->cidx[b]);
        cudaFree(h->crec[b]);
    }
    for (int b = 0; b < 2; b++) {
        for (auto c : h->cnt[b]) cudaFree(c);
        cudaFree(h->prec[b]);
        cudaFree(h->prank[b]);
    }
    cudaFree(h->sorted);
    cudaFree(h->moments);
    cudaFree(h->dpts);
    cudaFree(h->d_ctr);
    cudaFree(h->d_slotC);
    cudaFree(h->d_combC);
    cudaFree(h->height);
    cudaFree(h->inferred);
    cudaFree(h->slope_x);
    cudaFree(h->slope_y);
    cudaFree(h->rough);  // also the positive, negative and visibility maps
    cudaFree(h->guess);
    cudaFree(h->pos_density);
    cudaFree(h->zlow);
    cudaFree(h->mlow);
    cudaFree(h->colinfo[0]);
    cudaFree(h->colinfo[1]);
    cudaFree(h->occ_list[0]);
    cudaFree(h->occ_list[1]);
    cudaFree(h->d_dbg);
    cudaFree(h->d_ros);
    if (h->own) cudaStreamDestroy(h->own);
    delete h;
    return GVOM_OK;
}

int gvom_process(GvomHandle *h, const void *points, int32_t dtype, int64_t n, int64_t row_stride,
                 const double ego[3], const void *transform, int32_t transform_dtype) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    if (n > 0 && !points) return fail(GVOM_ERR_ARG, "points is NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    ScanIn s;
    int rc = fill_scan(h, s, dtype, n, row_stride, ego, transform, transform_dtype);
    if (rc) return rc;
    const size_t bytes = (size_t)n * (size_t)row_stride * (size_t)bytes_of(dtype);
    if ((rc = ensure_dpts(h, bytes))) return rc;
    if (bytes) {
        CUDA_TRY(cudaMemcpyAsync(h->dpts, points, bytes, cudaMemcpyHostToDevice, h->st));
    }
    s.dev_pts = h->dpts;
    std::vector<ScanIn> v{s};
    if ((rc = enqueue_scans(h, v))) return rc;
    if (bytes && is_pinned_host(points)) CUDA_TRY(cudaStreamSynchronize(h->st));  // caller may reuse its buffer
    return GVOM_OK;
}

// tf's fromTranslationRotation (ROS tf 1.13, tf/listener.py: the product of
// transformations.translation_matrix and transformations.quaternion_matrix):
// the quaternion q = (x, y, z, w) scaled by sqrt(2 / q.q), its outer product
// Q, R = [[1-Q11-Q22, Q01-Q23, Q02+Q13], [Q01+Q23, 1-Q00-Q22, Q12-Q03],
// [Q02-Q13, Q12+Q03, 1-Q00-Q11]] evaluated left to right, translation in the
// last column; identity rotation when q.q is below 4 machine epsilons.  q.q
// accumulates with fused multiply-adds in index order, as numpy's dot of two
// float64 4-vectors does (OpenBLAS ddot).
static void pose_matrix(const double t[3], const double qin[4], double T[16]) {
    double q[4] = {qin[0], qin[1], qin[2], qin[3]};
    double nq = 0.0;
    for (int k = 0; k < 4; k++) nq = std::fma(q[k], q[k], nq);
    for (int r = 0; r < 16; r++) T[r] = (r % 5 == 0) ? 1.0 : 0.0;
    if (!(nq < 4.0 * 2.220446049250313e-16)) {
        const double sc = std::sqrt(2.0 / nq);
        for (int k = 0; k < 4; k++) q[k] *= sc;
        double Q[4][4];
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++) Q[a][b] = q[a] * q[b];
        T[0] = (1.0 - Q[1][1]) - Q[2][2];
        T[1] = Q[0][1] - Q[2][3];
        T[2] = Q[0][2] + Q[1][3];
        T[4] = Q[0][1] + Q[2][3];
        T[5] = (1.0 - Q[0][0]) - Q[2][2];
        T[6] = Q[1][2] - Q[0][3];
        T[8] = Q[0][2] - Q[1][3];
        T[9] = Q[1][2] + Q[0][3];
        T[10] = (1.0 - Q[0][0]) - Q[1][1];
    }
    T[3] = t[0];
    T[7] = t[1];
    T[11] = t[2];
}

int gvom_process_device(GvomHandle *h, const void *d_points, int32_t dtype, int64_t n, int64_t row_stride,
                        const double ego[3], const void *transform, int32_t transform_dtype) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    if (n > 0 && !d_points) return fail(GVOM_ERR_ARG, "points is NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    ScanIn s;
    int rc = fill_scan(h, s, dtype, n, row_stride, ego, transform, transform_dtype);
    if (rc) return rc;
    s.dev_pts = d_points;
    std::vector<ScanIn> v{s};
    return enqueue_scans(h, v);
}

// Validates a scan list and stages host points into the device staging
// buffer (stream-ordered on h->st).  Scans that a later scan of the same batch
// overwrites (ring wrap) are dropped, their count in `skipped` (the kept
// scans go to the ring positions after theirs); `pinned` tells whether a host
// buffer was page-locked (the copy must then finish before the call returns).
static int stage_batch(GvomHandle *h, const GvomScan *scans, int n_scans, int points_on_device,
                       std::vector<ScanIn> &v, bool &pinned, int &skipped, cudaStream_t st = nullptr) {
    if (!st) st = h->st;
    const int first = std::max(0, n_scans - std::min(h->B, kMaxBatch));
    skipped = first;
    const int dt = scans[first].dtype;
    size_t total_bytes = 0;
    pinned = false;
    for (int i = first; i < n_scans; i++) {
        ScanIn s;
        int rc = fill_scan(h, s, scans[i].dtype, scans[i].n, scans[i].row_stride, scans[i].ego, scans[i].transform,
                           scans[i].transform_dtype);
        if (rc) return rc;
        if (s.dtype != dt) return fail(GVOM_ERR_ARG, "all scans of a batch must share one points dtype");
        if (s.n > 0 && !scans[i].points) return fail(GVOM_ERR_ARG, "points is NULL");
        total_bytes += (size_t)s.n * (size_t)s.stride * (size_t)bytes_of(s.dtype);
        total_bytes = (total_bytes + 255) & ~(size_t)255;
        v.push_back(s);
    }
    if (points_on_device) {
        for (size_t j = 0; j < v.size(); j++) v[j].dev_pts = scans[first + (int)j].points;
        return GVOM_OK;
    }
    int rc;
    if ((rc = ensure_dpts(h, total_bytes))) return rc;
    size_t off = 0;
    for (size_t j = 0; j < v.size(); j++) {
        const GvomScan &sc = scans[first + (int)j];
        const size_t b = (size_t)v[j].n * (size_t)v[j].stride * (size_t)bytes_of(v[j].dtype);
        if (b) {
            CUDA_TRY(cudaMemcpyAsync(static_cast<char *>(h->dpts) + off, sc.points, b, cudaMemcpyHostToDevice, st));
            pinned = pinned || is_pinned_host(sc.points);
        }
        v[j].dev_pts = static_cast<char *>(h->dpts) + off;
        off = (off + b + 255) & ~(size_t)255;
    }
    return GVOM_OK;
}

int gvom_pose_to_transform(const double translation[3], const double rotation_xyzw[4], double out[16]) {
    if (!translation || !rotation_xyzw || !out) return fail(GVOM_ERR_ARG, "NULL argument");
    pose_matrix(translation, rotation_xyzw, out);
    return GVOM_OK;
}

int gvom_process_pointcloud2(GvomHandle *h, const void *data, int64_t n_points, int32_t point_step,
                             const int32_t xyz_offsets[3], int32_t field_dtype, int32_t data_on_device,
                             const double ego[3], const double translation[3], const double rotation_xyzw[4]) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    if (!xyz_offsets || !ego || !translation || !rotation_xyzw) return fail(GVOM_ERR_ARG, "NULL argument");
    if (field_dtype != GVOM_F32 && field_dtype != GVOM_F64)
        return fail(GVOM_ERR_ARG, "x / y / z fields must be float32 or float64");
    const int fb = bytes_of(field_dtype);
    if (n_points < 0) return fail(GVOM_ERR_ARG, "negative point count");
    if (n_points > 0 && !data) return fail(GVOM_ERR_ARG, "data is NULL");
    if (point_step <= 0 || point_step % fb) return fail(GVOM_ERR_ARG, "point_step must be a positive multiple of the field size");
    for (int a = 0; a < 3; a++)
        if (xyz_offsets[a] < 0 || xyz_offsets[a] % fb || xyz_offsets[a] + fb > point_step)
            return fail(GVOM_ERR_ARG, "x / y / z offsets must be aligned to the field size and inside the point");
    if (data_on_device && n_points > 0 && ((uintptr_t)data % (uintptr_t)fb))
        return fail(GVOM_ERR_ARG, "device data must be aligned to the field size");
    std::lock_guard<std::mutex> lk(h->mu);
    ScanIn s;
    double T[16];
    pose_matrix(translation, rotation_xyzw, T);
    int rc = fill_scan(h, s, GVOM_F64, n_points, 3, ego, T, GVOM_F64);
    if (rc) return rc;
    s.pc2 = field_dtype == GVOM_F32 ? 1 : 2;
    s.stride = point_step;
    for (int a = 0; a < 3; a++) s.off[a] = xyz_offsets[a];
    const size_t bytes = (size_t)n_points * (size_t)point_step;
    if (data_on_device) {
        s.dev_pts = data;
    } else {
        if ((rc = ensure_dpts(h, bytes))) return rc;
        if (bytes) CUDA_TRY(cudaMemcpyAsync(h->dpts, data, bytes, cudaMemcpyHostToDevice, h->st));
        s.dev_pts = h->dpts;
    }
    std::vector<ScanIn> v{s};
    if ((rc = enqueue_scans(h, v))) return rc;
    if (!data_on_device && bytes && is_pinned_host(data)) CUDA_TRY(cudaStreamSynchronize(h->st));
    return GVOM_OK;
}

int gvom_process_batch(GvomHandle *h, const GvomScan *scans, int32_t n_scans, int32_t points_on_device) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    if (n_scans < 0 || (n_scans > 0 && !scans)) return fail(GVOM_ERR_ARG, "bad scan list");
    if (n_scans == 0) return GVOM_OK;
    std::lock_guard<std::mutex> lk(h->mu);
    std::vector<ScanIn> v;
    bool pinned = false;
    int skipped = 0;
    int rc;
    if ((rc = stage_batch(h, scans, n_scans, points_on_device, v, pinned, skipped))) return rc;
    if ((rc = enqueue_scans(h, v, skipped))) return rc;
    if (pinned) CUDA_TRY(cudaStreamSynchronize(h->st));
    for (int a = 0; a < 3; a++) h->ego[a] = scans[n_scans - 1].ego[a];
    return GVOM_OK;
}

// A combine call in three parts, like a process call.
struct CombPlan {
    MergeParams mp;
    ColumnParams cp;
    Maps2DParams m2;
    int nb = 0;
};

int prepare_combine(GvomHandle *h, CombPlan &pl) {
    const int lp = h->phys_of[h->last_buffer_index];
    if (lp < 0 || !h->slots[lp].valid) return fail(GVOM_NO_DATA, "ERROR: No data in buffer");
    const Slot &ls = h->slots[lp];
    const int nb = h->have_comb ? 1 - h->cur : 0;  // buffer receiving the new combined map
    pl.nb = nb;
    MergeParams &mp = pl.mp;
    std::memset(&mp, 0, sizeof(mp));
    mp.g = h->g;
    for (int a = 0; a < 3; a++) mp.co[a] = ls.od[a];
    int ns = 0;
    for (int i = 0; i < h->B; i++) {  // ring order, as the reference merges
        if (h->phys_of[i] < 0) continue;
        const Slot &s = h->slots[h->phys_of[i]];
        if (!s.valid) continue;
        h->slot_epoch[h->phys_of[i]] = h->n_comb;  // read by this combine (see comb_done)
        MergeSrc &m = mp.src[ns++];
        m.idx = s.idx;
        m.rec = s.rec;
        m.dx = (int)(mp.co[0] - s.od[0]);
        m.dy = (int)(mp.co[1] - s.od[1]);
        m.dz = (int)(mp.co[2] - s.od[2]);
        m.is_last = 0;
    }
    if (h->have_comb) {
        MergeSrc &m = mp.src[ns++];
        m.idx = h->cidx[h->cur];
        m.rec = h->crec[h->cur];
        m.dx = (int)(mp.co[0] - h->cod[h->cur][0]);
        m.dy = (int)(mp.co[1] - h->cod[h->cur][1]);
        m.dz = (int)(mp.co[2] - h->cod[h->cur][2]);
        m.is_last = 1;
    }
    mp.nsrc = ns;
    mp.out_idx = h->cidx[nb];
    mp.out_rec = h->crec[nb];
    mp.out_count = h->d_combC + nb;
    mp.list = h->occ_list[nb];
    mp.num_sms = h->num_sms;
    mp.planes = h->tun.merge_planes;
    mp.stats_bpsm = h->tun.stats_bpsm;
    mp.colinfo = h->colinfo[nb];
    ColumnParams &cp = pl.cp;
    std::memset(&cp, 0, sizeof(cp));
    cp.X = h->g.X;
    cp.Z = h->g.Z;
    cp.planes = h->tun.merge_planes;
    cp.idx = mp.out_idx;
    cp.rec = mp.out_rec;
    cp.colinfo = h->colinfo[nb];
    for (int a = 0; a < 3; a++) {
        cp.co[a] = mp.co[a];
        cp.ego[a] = h->ego[a];
    }
    cp.xy_res = h->p.xy_resolution;
    cp.z_res = h->p.z_resolution;
    cp.robot_r2 = h->p.robot_radius * h->p.robot_radius;
    cp.disc_h = h->ego[2] - h->p.ground_to_lidar_height;
    cp.pos_thr = h->p.positive_obstacle_threshold;
    cp.robot_h = h->p.robot_height;
    cp.pthr_v = (float)(h->p.positive_obstacle_threshold / h->p.z_resolution);
    cp.robh_v = (float)(h->p.robot_height / h->p.z_resolution);
    cp.base_xf = (float)(mp.co[0] * h->p.xy_resolution - h->ego[0]);
    cp.base_yf = (float)(mp.co[1] * h->p.xy_resolution - h->ego[1]);
    cp.res_f = (float)h->p.xy_resolution;
    cp.r2_f = (float)cp.robot_r2;
    cp.height = h->height;
    cp.inferred = h->inferred;
    cp.pos_density = h->pos_density;
    cp.zlow = h->zlow;
    cp.mlow = h->mlow;
    Maps2DParams &m2 = pl.m2;
    std::memset(&m2, 0, sizeof(m2));
    m2.X = h->g.X;
    m2.xy_res = h->p.xy_resolution;
    m2.z_res = h->p.z_resolution;
    m2.slope_thr = h->p.slope_obstacle_threshold;
    m2.slope_thr_f = (float)h->p.slope_obstacle_threshold;
    m2.neg_thr = h->p.negative_obstacle_threshold;
    m2.height = h->height;
    m2.inferred = h->inferred;
    m2.pos_density = h->pos_density;
    m2.zlow = h->zlow;
    m2.mlow = h->mlow;
    m2.slope_x = h->slope_x;
    m2.slope_y = h->slope_y;
    m2.rough = h->rough;
    m2.guess = h->guess;
    m2.pos = h->pos;
    m2.neg = h->neg;
    m2.vis = h->vis;
    m2.tile_cells = h->tun.maps_tile;
    return GVOM_OK;
}

// stream-ordered work of a prepared combine on h->st.
// `part`: 0 the whole combine (below); 1 the index and count merges on `st`;
// 2 columns and maps on h->st, with ev_cols[buffer] recorded between them.
// part 0: with `timing`, every kernel in sequence on h->st.  Without events,
// the index and count merges on `st`, then the statistics merge forked onto
// `side` beside the columns and maps, joined at the end.  With `idx_ready`
// (recorded once the ring's index maps are complete) the index merge runs on
// `side` after that event, overlapping the rest of the process kernels.  With
// `mom_ready` too (recorded once the slots' records hold hit, total and min
// height, after the cell moments), `side` goes on with the count merge, the
// columns and the maps after that event, while h->st, after the process
// tail (neighbourhood statistics, clean-up), runs the statistics merge; h->st
// joins `side` at the end.
int launch_comb(GvomHandle *h, const CombPlan &pl, cudaEvent_t idx_ready, bool timing, int part = 0,
                cudaStream_t st = nullptr, cudaEvent_t mom_ready = nullptr) {
    if (!st) st = h->st;
    if (part == 2) {
        CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->st, nullptr, 2));
        CUDA_TRY(rec_event_external(h->ev_cols[pl.nb], h->st));
        CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->st, nullptr, 3));
        return GVOM_OK;
    }
    if (timing) {
        CUDA_TRY(rec_memset(pl.mp.out_count, 0, sizeof(int), h->st));
        CUDA_TRY(launch_combine(pl.mp, pl.cp, pl.m2, h->st, h->timer.begin(kProcessKernels, kCombineKernels)));
        return GVOM_OK;
    }
    if (idx_ready && mom_ready && part == 0) {
        CUDA_TRY(rec_wait_internal(h->side, idx_ready));
        CUDA_TRY(rec_memset(pl.mp.out_count, 0, sizeof(int), h->side));
        CUDA_TRY(launch_merge_index(pl.mp, h->side));
        CUDA_TRY(rec_event_internal(h->ev_join, h->side));
        CUDA_TRY(rec_wait_internal(h->side, mom_ready));
        CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->side, nullptr, 1));
        CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->side, nullptr, 2));
        CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->side, nullptr, 3));
        CUDA_TRY(rec_event_internal(h->ev_msj, h->side));
        CUDA_TRY(rec_wait_internal(h->st, h->ev_join));
        CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->st, nullptr, 4));
        CUDA_TRY(rec_wait_internal(h->st, h->ev_msj));
        return GVOM_OK;
    }
    if (idx_ready) {
        CUDA_TRY(rec_wait_internal(h->side, idx_ready));
        CUDA_TRY(rec_memset(pl.mp.out_count, 0, sizeof(int), h->side));
        CUDA_TRY(launch_merge_index(pl.mp, h->side));
        CUDA_TRY(rec_event_internal(h->ev_join, h->side));
        CUDA_TRY(rec_wait_internal(st, h->ev_join));
    } else {
        CUDA_TRY(rec_memset(pl.mp.out_count, 0, sizeof(int), st));
        CUDA_TRY(launch_merge_index(pl.mp, st));
    }
    CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, st, nullptr, 1));
    if (part == 1) return GVOM_OK;
    CUDA_TRY(rec_event_internal(h->ev_ms, h->st));
    CUDA_TRY(rec_wait_internal(h->side, h->ev_ms));
    CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->side, nullptr, 4));
    CUDA_TRY(rec_event_internal(h->ev_msj, h->side));
    CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->st, nullptr, 2));
    CUDA_TRY(launch_combine_rest(pl.mp, pl.cp, pl.m2, h->st, nullptr, 3));
    CUDA_TRY(rec_wait_internal(h->st, h->ev_msj));
    return GVOM_OK;
}

void commit_combine(GvomHandle *h, const CombPlan &pl) {
    const int nb = pl.nb;
    const MergeParams &mp = pl.mp;
    for (int a = 0; a < 3; a++) h->cod[nb][a] = mp.co[a];
    h->cur = nb;
    h->have_comb = true;
    h->have_maps = true;
}

// the caller's four buffers laid out as the device block: roughness, then
// positive, negative and visibility, back to back
static bool outputs_in_block(size_t X2, const int32_t *pos, const int32_t *neg, const double *rough,
                             const int32_t *vis) {
    if (!pos || !neg || !rough || !vis) return false;
    const char *r = reinterpret_cast<const char *>(rough);
    return reinterpret_cast<const char *>(pos) == r + X2 * 8 && neg == pos + X2 && vis == neg + X2;
}

// origin (scripts/gvom.py:385-388) and the four maps to host or device buffers
int copy_outputs(GvomHandle *h, const CombPlan &pl, double origin[3], int32_t *pos, int32_t *neg, double *rough,
                 int32_t *vis, bool to_host) {
    if (origin) {
        origin[0] = pl.mp.co[0] * h->p.xy_resolution;
        origin[1] = pl.mp.co[1] * h->p.xy_resolution;
        origin[2] = pl.mp.co[2] * h->p.z_resolution;
    }
    const size_t X2 = (size_t)h->g.X * h->g.X;
    const cudaMemcpyKind kind = to_host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (outputs_in_block(X2, pos, neg, rough, vis)) {
        CUDA_TRY(cudaMemcpyAsync(rough, h->rough, X2 * kOutBytesPerCell, kind, h->st));
        if (to_host) CUDA_TRY(cudaStreamSynchronize(h->st));
        return GVOM_OK;
    }
    if (pos) CUDA_TRY(cudaMemcpyAsync(pos, h->pos, X2 * 4, kind, h->st));
    if (neg) CUDA_TRY(cudaMemcpyAsync(neg, h->neg, X2 * 4, kind, h->st));
    if (rough) CUDA_TRY(cudaMemcpyAsync(rough, h->rough, X2 * 8, kind, h->st));
    if (vis) CUDA_TRY(cudaMemcpyAsync(vis, h->vis, X2 * 4, kind, h->st));
    if (to_host) CUDA_TRY(cudaStreamSynchronize(h->st));
    return GVOM_OK;
}

// the four maps into the caller's device buffers, on the instance stream, as
// part of the sequence (graph) that computes them
static int enqueue_device_outputs(GvomHandle *h, int32_t *pos, int32_t *neg, double *rough, int32_t *vis) {
    const size_t X2 = (size_t)h->g.X * h->g.X;
    if (outputs_in_block(X2, pos, neg, rough, vis)) {
        CUDA_TRY(rec_memcpy(rough, h->rough, X2 * kOutBytesPerCell, cudaMemcpyDeviceToDevice, h->st));
        return GVOM_OK;
    }
    if (pos) CUDA_TRY(rec_memcpy(pos, h->pos, X2 * 4, cudaMemcpyDeviceToDevice, h->st));
    if (neg) CUDA_TRY(rec_memcpy(neg, h->neg, X2 * 4, cudaMemcpyDeviceToDevice, h->st));
    if (rough) CUDA_TRY(rec_memcpy(rough, h->rough, X2 * 8, cudaMemcpyDeviceToDevice, h->st));
    if (vis) CUDA_TRY(rec_memcpy(vis, h->vis, X2 * 4, cudaMemcpyDeviceToDevice, h->st));
    return GVOM_OK;
}

static int combine_impl(GvomHandle *h, double origin[3], int32_t *pos, int32_t *neg, double *rough, int32_t *vis,
                        bool to_host) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    h->st_dirty = true;  // work on the instance stream: see the step pipeline
    CombPlan pl;
    int rc = prepare_combine(h, pl);
    if (rc) return rc;
    // right after a process call: its index merge starts once the index maps
    // are complete and its count merge, columns and maps once the cell moments
    // are, beside the process tail (direct launches: the waits name the
    // process call's events)
    const bool overlap = h->proc_events && h->tun.step_overlap && !h->timer.on;
    h->proc_events = false;
    if (overlap) rc = launch_comb(h, pl, h->ev_idx, false, 0, nullptr, h->ev_mom);
    else rc = run_graphed(h, 1, [&]() -> int { return launch_comb(h, pl, nullptr, !h->graphs); });
    if (rc) return rc;
    if ((rc = comb_done(h, h->st))) return rc;
    commit_combine(h, pl);
    return copy_outputs(h, pl, origin, pos, neg, rough, vis, to_host);
}

int gvom_combine(GvomHandle *h, double origin[3], int32_t *pos, int32_t *neg, double *roughness, int32_t *visibility) {
    return combine_impl(h, origin, pos, neg, roughness, visibility, true);
}

int gvom_combine_device(GvomHandle *h, double origin[3], int32_t *d_pos, int32_t *d_neg, double *d_roughness,
                        int32_t *d_visibility) {
    return combine_impl(h, origin, d_pos, d_neg, d_roughness, d_visibility, false);
}

int gvom_step(GvomHandle *h, const GvomScan *scans, int32_t n_scans, int32_t points_on_device, double origin[3],
              int32_t *pos, int32_t *neg, double *roughness, int32_t *visibility, int32_t outputs_on_device) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    if (n_scans < 1 || !scans) return fail(GVOM_ERR_ARG, "a step needs at least one scan");
    std::lock_guard<std::mutex> lk(h->mu);
    const bool timing = !h->graphs && h->timer.on;
    const bool dev_out = outputs_on_device != 0;
    // with stage timing the kernels run in sequence so that each interval is one
    // kernel; a step whose maps go to host memory ends with a host wait, so the
    // next call cannot overlap it, and one graph (level 0, with the same
    // overlap inside the step) is cheaper to submit than the pipeline's six
    const int pipe = (timing || !dev_out) ? 0 : h->tun.step_pipeline;
    if (pipe >= 2 && h->st_dirty) {  // order the pipeline streams after other calls' work
        CUDA_TRY(cudaEventRecord(h->ev_host, h->st));
        CUDA_TRY(cudaStreamWaitEvent(h->tr, h->ev_host, 0));
        CUDA_TRY(cudaStreamWaitEvent(h->bs, h->ev_host, 0));
        CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_host, 0));
        h->st_dirty = false;
    }
    // a pipelined step stages its points and traces on `tr`, once the previous
    // process is done with the per-scan scratch and the staging buffer
    if (pipe) CUDA_TRY(cudaStreamWaitEvent(h->tr, h->ev_scratch[h->sset], 0));
    std::vector<ScanIn> v;
    bool pinned = false;
    int skipped = 0;
    int rc;
    if ((rc = stage_batch(h, scans, n_scans, points_on_device, v, pinned, skipped, pipe ? h->tr : h->st))) return rc;
    ProcPlan pp;
    // pipelined: spare slots for two steps, so the trace never waits for a combine in flight
    if ((rc = prepare_scans(h, v, pp, pipe ? 2 * (int)v.size() : 0, skipped))) return rc;
    // the trace stream waits until no combine in flight reads the slots it fills
    if ((rc = wait_slots_free(h, pp.slot_of, pp.k, pipe ? h->tr : h->st))) {
        release_slots(h, pp);
        return rc;
    }
    commit_scans(h, pp);  // host ring bookkeeping; the combine plan reads the ring after this batch
    for (int a = 0; a < 3; a++) h->ego[a] = scans[n_scans - 1].ego[a];
    CombPlan cp;
    if ((rc = prepare_combine(h, cp))) return rc;
    cudaEvent_t idx = (timing || !h->tun.step_overlap) ? nullptr : h->ev_idx;
    cudaEvent_t mom = idx ? h->ev_mom : nullptr;
    h->proc_events = false;
    if (pipe == 2) {
        // tr: the trace
        rc = run_graphed(h, 3, [&]() -> int {
            if ((rc = launch_scans(h, pp, nullptr, false, 1, h->tr))) return rc;
            CUDA_TRY(rec_event_external(h->ev_traced, h->tr));
            return GVOM_OK;
        }, h->tr);
        if (rc) return rc;
        // bs: the rest of the process, after the trace; ev_idx marks the slots'
        // index maps complete, ev_mom their records' hit, total and min height,
        // ev_scratch[set] the whole process
        CUDA_TRY(cudaStreamWaitEvent(h->bs, h->ev_traced, 0));
        rc = run_graphed(h, 4, [&]() -> int {
            if ((rc = launch_scans(h, pp, h->ev_idx, false, 2, h->bs, true, h->ev_mom))) return rc;
            CUDA_TRY(rec_event_external(h->ev_scratch[pp.set], h->bs));
            return GVOM_OK;
        }, h->bs);
        if (rc) return rc;
        // side: the combine's merges, in stream order after the previous step's
        // statistics merge (which reads the combined buffer this merge writes)
        // and after the columns pass that last read that buffer; the index merge
        // once the index maps are complete, beside the statistics kernels
        CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_cols[cp.nb], 0));
        CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_idx, 0));
        rc = run_graphed(h, 7, [&]() -> int {
            CUDA_TRY(rec_memset(cp.mp.out_count, 0, sizeof(int), h->side));
            CUDA_TRY(launch_merge_index(cp.mp, h->side));
            return GVOM_OK;
        }, h->side);
        if (rc) return rc;
        // the count merge once the slots' records hold hit, total and min
        // height; the statistics merge once they are complete
        CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_mom, 0));
        rc = run_graphed(h, 6, [&]() -> int {
            CUDA_TRY(launch_combine_rest(cp.mp, cp.cp, cp.m2, h->side, nullptr, 1));
            CUDA_TRY(rec_event_external(h->ev_merged, h->side));
            return GVOM_OK;
        }, h->side);
        if (rc) return rc;
        CUDA_TRY(cudaStreamWaitEvent(h->side, h->ev_scratch[pp.set], 0));
        rc = run_graphed(h, 8, [&]() -> int {
            CUDA_TRY(launch_combine_rest(cp.mp, cp.cp, cp.m2, h->side, nullptr, 4));
            CUDA_TRY(rec_event_external(h->ev_stats[cp.nb], h->side));
            return GVOM_OK;
        }, h->side);
        if (rc) return rc;
        if ((rc = comb_done(h, h->side))) return rc;
        // st: columns and maps after the count merge, beside the statistics
        // merge and the next step's process
        CUDA_TRY(cudaStreamWaitEvent(h->st, h->ev_merged, 0));
        rc = run_graphed(h, 5, [&]() -> int {
            if ((rc = launch_comb(h, cp, nullptr, false, 2))) return rc;
            return dev_out ? enqueue_device_outputs(h, pos, neg, roughness, visibility) : GVOM_OK;
        });
        if (!rc) CUDA_TRY(cudaStreamWaitEvent(h->st, h->ev_stats[cp.nb], 0));  // later calls see whole records
    } else if (pipe == 1) {
        h->st_dirty = true;
        // the trace waits only for the previous process to release the scratch
        // (and for its slots), so it runs beside the previous step's combine
        rc = run_graphed(h, 3, [&]() -> int {
            if ((rc = launch_scans(h, pp, nullptr, false, 1, h->tr))) return rc;
            CUDA_TRY(rec_event_external(h->ev_traced, h->tr));
            return GVOM_OK;
        }, h->tr);
        if (rc) return rc;
        CUDA_TRY(cudaStreamWaitEvent(h->st, h->ev_traced, 0));
        rc = run_graphed(h, 4, [&]() -> int {
            if ((rc = launch_scans(h, pp, idx, false, 2, nullptr, false, mom))) return rc;
            // in graph mode an event-record node of the graph
            CUDA_TRY(rec_event_external(h->ev_scratch[pp.set], h->st));
            if ((rc = launch_comb(h, cp, idx, false, 0, nullptr, mom))) return rc;
            return dev_out ? enqueue_device_outputs(h, pos, neg, roughness, visibility) : GVOM_OK;
        });
        if (!rc) rc = comb_done(h, h->st);
    } else {
        h->st_dirty = true;
        rc = run_graphed(h, 2, [&]() -> int {
            if ((rc = launch_scans(h, pp, idx, timing, 0, nullptr, false, mom))) return rc;
            if ((rc = launch_comb(h, cp, idx, timing, 0, nullptr, mom))) return rc;
            return dev_out ? enqueue_device_outputs(h, pos, neg, roughness, visibility) : GVOM_OK;
        });
        if (!rc) CUDA_TRY(cudaEventRecord(h->ev_scratch[pp.set], h->st));
        if (!rc) rc = comb_done(h, h->st);
    }
    if (rc) return rc;
    commit_combine(h, cp);
    // device outputs were written by the step's own sequence; host outputs are copied here
    if (dev_out) rc = copy_outputs(h, cp, origin, nullptr, nullptr, nullptr, nullptr, false);
    else rc = copy_outputs(h, cp, origin, pos, neg, roughness, visibility, true);
    if (rc) return rc;
    if (pinned) CUDA_TRY(cudaStreamSynchronize(pipe ? h->tr : h->st));  // the caller may reuse its buffers
    return GVOM_OK;
}

int gvom_debug_voxel_map(GvomHandle *h, float *out, int64_t capacity_rows, int64_t *rows) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    h->st_dirty = true;  // work on the instance stream: see the step pipeline
    if (!h->have_comb) return fail(GVOM_NO_DATA, "No data");
    const long long V = h->g.V;
    const int chunk = debug_chunk();
    const int nblocks = (int)((V + chunk - 1) / chunk);
    if (!h->d_dbg) {
        int rc = dalloc_t(h, &h->d_dbg, (size_t)nblocks + 1);
        if (rc) return rc;
    }
    CUDA_TRY(launch_debug_count(h->cidx[h->cur], V, h->d_dbg, nblocks, h->st));
    std::vector<int> counts(nblocks);
    CUDA_TRY(cudaMemcpyAsync(counts.data(), h->d_dbg, sizeof(int) * nblocks, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    long long tot = 0;
    for (int b = 0; b < nblocks; b++) {
        const int c = counts[b];
        counts[b] = (int)tot;
        tot += c;
    }
    if (rows) *rows = tot;
    if (!out || tot == 0) return GVOM_OK;
    CUDA_TRY(cudaMemcpyAsync(h->d_dbg, counts.data(), sizeof(int) * nblocks, cudaMemcpyHostToDevice, h->st));
    float *dout = nullptr;
    const long long nrow = std::min<long long>(tot, capacity_rows);
    int rc = dalloc_t(h, &dout, (size_t)std::max<long long>(nrow, 1) * 8);
    if (rc) return rc;
    DebugVoxParams p;
    p.idx = h->cidx[h->cur];
    p.rec = h->crec[h->cur];
    p.block_off = h->d_dbg;
    p.V = V;
    p.X = h->g.X;
    for (int a = 0; a < 3; a++) p.co[a] = h->cod[h->cur][a];
    p.xy_res = h->p.xy_resolution;
    p.z_res = h->p.z_resolution;
    p.out = dout;
    p.cap = nrow;
    cudaError_t e = launch_debug_voxels(p, nblocks, h->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, (size_t)nrow * 8 * sizeof(float), cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    dfree(h, dout, (size_t)std::max<long long>(nrow, 1) * 8 * sizeof(float));
    if (e != cudaSuccess) return fail(GVOM_ERR_CUDA, std::string("debug voxel export: ") + cudaGetErrorString(e));
    return GVOM_OK;
}

static int debug_maps(GvomHandle *h, float *out_h, float *out_i) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    h->st_dirty = true;  // work on the instance stream: see the step pipeline
    if (!h->have_maps) return fail(GVOM_NO_DATA, "No data");
    if (!out_h && !out_i) return fail(GVOM_ERR_ARG, "output is NULL");
    const size_t X2 = (size_t)h->g.X * h->g.X;
    const size_t cols = out_h ? 7 : 3;
    float *dout = nullptr;
    int rc = dalloc_t(h, &dout, X2 * cols);
    if (rc) return rc;
    DebugMapParams p;
    p.X = h->g.X;
    for (int a = 0; a < 3; a++) p.co[a] = h->cod[h->cur][a];
    p.xy_res = h->p.xy_resolution;
    p.z_res = h->p.z_resolution;
    p.height = h->height;
    p.rough = h->rough;
    p.slope_x = h->slope_x;
    p.slope_y = h->slope_y;
    p.guess = h->guess;
    p.out_h = out_h ? dout : nullptr;
    p.out_i = out_h ? nullptr : dout;
    cudaError_t e = launch_debug_maps(p, h->st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out_h ? (void *)out_h : (void *)out_i, dout, X2 * cols * sizeof(float),
                            cudaMemcpyDeviceToHost, h->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->st);
    dfree(h, dout, X2 * cols * sizeof(float));
    if (e != cudaSuccess) return fail(GVOM_ERR_CUDA, std::string("debug map export: ") + cudaGetErrorString(e));
    return GVOM_OK;
}

namespace {

// Address of the allocation-free export's scratch array, looked up once per
// device (with that device current) and cached; the lock also serialises the
// calls that share the array.
constexpr int kMaxDevices = 64;
std::mutex g_static_mu[kMaxDevices];
int *g_static_ptr[kMaxDevices] = {};

}  // namespace

int gvom_debug_voxel_map_noalloc(GvomHandle *h, float *d_out, int64_t capacity_rows, int64_t *rows) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    if (capacity_rows < 0) return fail(GVOM_ERR_ARG, "capacity_rows is negative");
    std::lock_guard<std::mutex> lk(h->mu);
    h->st_dirty = true;  // work on the instance stream: see the step pipeline
    const long long V = h->g.V;
    const int chunk = debug_chunk();
    const long long nblocks = (V + chunk - 1) / chunk;
    if (nblocks > kStaticDebugBlocks)
        return fail(GVOM_ERR_ARG, "grid of " + std::to_string(V) + " voxels is above the " +
                                      std::to_string((long long)kStaticDebugBlocks * chunk) +
                                      " voxels the allocation-free export supports; use gvom_debug_voxel_map");
    if (!h->have_comb) return fail(GVOM_NO_DATA, "No data");
    // the scratch array and its lock belong to the instance's device (current
    // here through the DeviceScope)
    const int dev = h->dev;
    if (dev < 0 || dev >= kMaxDevices) return fail(GVOM_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> dl(g_static_mu[dev]);
    if (!g_static_ptr[dev]) {
        int *p = nullptr;
        const cudaError_t e = debug_static_scratch(&p);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return fail(GVOM_ERR_CUDA, std::string("scratch address lookup: ") + cudaGetErrorString(e));
        }
        g_static_ptr[dev] = p;
    }
    int *scratch = g_static_ptr[dev];
    // once a kernel is queued, every exit waits for the stream, so that the
    // lock covers all device work on the shared scratch array
    int total = 0;
    cudaError_t e = launch_debug_count(h->cidx[h->cur], V, scratch, (int)nblocks, h->st);
    if (e == cudaSuccess) e = launch_debug_offsets(scratch, (int)nblocks, h->st);
    if (e == cudaSuccess && d_out && capacity_rows > 0) {
        DebugVoxParams p;
        p.idx = h->cidx[h->cur];
        p.rec = h->crec[h->cur];
        p.block_off = scratch;
        p.V = V;
        p.X = h->g.X;
        for (int a = 0; a < 3; a++) p.co[a] = h->cod[h->cur][a];
        p.xy_res = h->p.xy_resolution;
        p.z_res = h->p.z_resolution;
        p.out = d_out;
        p.cap = capacity_rows;
        e = launch_debug_voxels(p, (int)nblocks, h->st);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, scratch + nblocks, sizeof(int), cudaMemcpyDeviceToHost, h->st);
    const cudaError_t es = cudaStreamSynchronize(h->st);
    if (e == cudaSuccess) e = es;
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(GVOM_ERR_CUDA, std::string("allocation-free debug voxel export: ") + cudaGetErrorString(e));
    }
    if (rows) *rows = total;
    return GVOM_OK;
}

int gvom_ros_grids(GvomHandle *h, const GvomRosParams *rp, int8_t *hard, int8_t *soft, int8_t *certainty,
                   int8_t *negative, int8_t *roughness, int32_t outputs_on_device) {
    if (!h || !rp) return fail(GVOM_ERR_ARG, "handle or params is NULL");
    DeviceScope ds(h->dev);
    if (!(rp->max_roughness != rp->min_roughness)) return fail(GVOM_ERR_ARG, "max_roughness must differ from min_roughness");
    std::lock_guard<std::mutex> lk(h->mu);
    h->st_dirty = true;  // work on the instance stream: see the step pipeline
    if (!h->have_maps) return fail(GVOM_NO_DATA, "No data");
    const size_t X2 = (size_t)h->g.X * h->g.X;
    int8_t *outs[5] = {hard, soft, certainty, negative, roughness};
    RosGridParams p;
    p.X = h->g.X;
    p.pos = h->pos;
    p.neg = h->neg;
    p.vis = h->vis;
    p.rough = h->rough;
    p.density_thr = rp->density_threshold;
    p.min_r = rp->min_roughness;
    p.max_r = rp->max_roughness;
    signed char *dst[5];
    if (outputs_on_device) {
        for (int k = 0; k < 5; k++) dst[k] = reinterpret_cast<signed char *>(outs[k]);
    } else {
        if (!h->d_ros) {
            int rc = dalloc(h, reinterpret_cast<void **>(&h->d_ros), X2 * 5);
            if (rc) return rc;
        }
        for (int k = 0; k < 5; k++) dst[k] = outs[k] ? reinterpret_cast<signed char *>(h->d_ros) + k * X2 : nullptr;
    }
    p.hard = dst[0];
    p.soft = dst[1];
    p.certainty = dst[2];
    p.negative = dst[3];
    p.roughness = dst[4];
    CUDA_TRY(launch_ros_grids(p, h->st));
    if (!outputs_on_device) {
        for (int k = 0; k < 5; k++)
            if (outs[k]) CUDA_TRY(cudaMemcpyAsync(outs[k], dst[k], X2, cudaMemcpyDeviceToHost, h->st));
        CUDA_TRY(cudaStreamSynchronize(h->st));
    }
    return GVOM_OK;
}

int gvom_debug_height_map(GvomHandle *h, float *out) { return debug_maps(h, out, nullptr); }

int gvom_debug_inferred_height_map(GvomHandle *h, float *out) { return debug_maps(h, nullptr, out); }

int gvom_ring_state(GvomHandle *h, int64_t *buffer_index, int64_t *last_buffer_index) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    if (buffer_index) *buffer_index = h->buffer_index;
    if (last_buffer_index) *last_buffer_index = h->last_buffer_index;
    return GVOM_OK;
}

static int read_int(GvomHandle *h, const int *d, int *v) {
    CUDA_TRY(cudaMemcpyAsync(v, d, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return GVOM_OK;
}

int gvom_slot_count(GvomHandle *h, int32_t slot, int64_t *count) {
    if (!h || !count) return fail(GVOM_ERR_ARG, "NULL argument");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    if (slot < 0 || slot >= h->B) return fail(GVOM_ERR_ARG, "slot out of range");
    const int p = h->phys_of[slot];
    if (p < 0 || !h->slots[p].valid) {
        *count = -1;
        return GVOM_OK;
    }
    int c = 0;
    int rc = read_int(h, h->d_slotC + p, &c);
    if (rc) return rc;
    *count = c;
    return GVOM_OK;
}

// unpack records into the reference's per-array layout
static int copy_records(GvomHandle *h, const VoxelRec *d_rec, long long C, int32_t *hit, int32_t *total, float *min_h,
                        float *metrics, float *eigen) {
    if (C <= 0) return GVOM_OK;
    if (!hit && !total && !min_h && !metrics && !eigen) return GVOM_OK;
    std::vector<VoxelRec> r((size_t)C);
    CUDA_TRY(cudaMemcpyAsync(r.data(), d_rec, sizeof(VoxelRec) * C, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    for (long long c = 0; c < C; c++) {
        const VoxelRec &v = r[c];
        if (hit) hit[c] = v.hit;
        if (total) total[c] = v.total;
        if (min_h) min_h[c] = v.min_h;
        if (metrics) {
            float *m = metrics + c * 10;
            m[0] = v.mean[0];
            m[1] = v.mean[1];
            m[2] = v.mean[2];
            for (int t = 0; t < 6; t++) m[3 + t] = v.cov[t];
            m[9] = v.count;
        }
        if (eigen) {
            eigen[c * 3 + 0] = v.aux[0];
            eigen[c * 3 + 1] = v.aux[1];
            eigen[c * 3 + 2] = v.aux[2];
        }
    }
    return GVOM_OK;
}

int gvom_get_slot(GvomHandle *h, int32_t slot, int32_t *index, int32_t *hit, int32_t *total, float *min_height,
                  float *metrics, double origin[3]) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    if (slot < 0 || slot >= h->B) return fail(GVOM_ERR_ARG, "slot out of range");
    const int p = h->phys_of[slot];
    if (p < 0 || !h->slots[p].valid) return fail(GVOM_NO_DATA, "slot is empty");
    const Slot &s = h->slots[p];
    int C = 0;
    int rc = read_int(h, h->d_slotC + p, &C);
    if (rc) return rc;
    if (index) {
        CUDA_TRY(cudaMemcpyAsync(index, s.idx, sizeof(int) * h->g.V, cudaMemcpyDeviceToHost, h->st));
        CUDA_TRY(cudaStreamSynchronize(h->st));
    }
    if ((rc = copy_records(h, s.rec, C, hit, total, min_height, metrics, nullptr))) return rc;
    if (origin)
        for (int a = 0; a < 3; a++) origin[a] = s.od[a];
    return GVOM_OK;
}

int gvom_combined_count(GvomHandle *h, int64_t *count) {
    if (!h || !count) return fail(GVOM_ERR_ARG, "NULL argument");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->have_comb) {
        *count = -1;
        return GVOM_OK;
    }
    int c = 0;
    int rc = read_int(h, h->d_combC + h->cur, &c);
    if (rc) return rc;
    *count = c;
    return GVOM_OK;
}

int gvom_get_combined(GvomHandle *h, int32_t *index, int32_t *hit, int32_t *total, float *min_height, float *metrics,
                      float *eigen, double origin[3]) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->have_comb) return fail(GVOM_NO_DATA, "No data");
    // the device map addresses records by voxel id; export them compacted in
    // ascending voxel-id order, with the index map renumbered to match
    std::vector<int32_t> idx((size_t)h->g.V);
    CUDA_TRY(cudaMemcpyAsync(idx.data(), h->cidx[h->cur], sizeof(int) * h->g.V, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    std::vector<int32_t> vids;
    for (long long v = 0; v < h->g.V; v++)
        if (idx[v] >= 0) {
            idx[v] = (int32_t)vids.size();
            vids.push_back((int32_t)v);
        }
    if (index) std::memcpy(index, idx.data(), sizeof(int) * h->g.V);
    const int C = (int)vids.size();
    if (C > 0 && (hit || total || min_height || metrics || eigen)) {
        int *d_vids = nullptr;
        VoxelRec *d_out = nullptr;
        int rc = dalloc_t(h, &d_vids, (size_t)C);
        if (rc) return rc;
        rc = dalloc_t(h, &d_out, (size_t)C);
        if (rc) {
            dfree(h, d_vids, sizeof(int) * C);
            return rc;
        }
        cudaError_t e = cudaMemcpyAsync(d_vids, vids.data(), sizeof(int) * C, cudaMemcpyHostToDevice, h->st);
        if (e == cudaSuccess) e = launch_gather_records(h->crec[h->cur], d_vids, C, d_out, h->st);
        int rc2 = GVOM_OK;
        if (e == cudaSuccess) rc2 = copy_records(h, d_out, C, hit, total, min_height, metrics, eigen);
        else rc2 = fail(GVOM_ERR_CUDA, std::string("gather: ") + cudaGetErrorString(e));
        dfree(h, d_vids, sizeof(int) * C);
        dfree(h, d_out, sizeof(VoxelRec) * C);
        if (rc2) return rc2;
    }
    if (origin)
        for (int a = 0; a < 3; a++) origin[a] = h->cod[h->cur][a];
    return GVOM_OK;
}

int gvom_get_maps(GvomHandle *h, double *height, double *inferred, double *slope_x, double *slope_y, double *roughness,
                  double *guess) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    if (!h->have_maps) return fail(GVOM_NO_DATA, "No data");
    const size_t b = (size_t)h->g.X * h->g.X * 8;
    double *dst[6] = {height, inferred, slope_x, slope_y, roughness, guess};
    const double *src[6] = {h->height, h->inferred, h->slope_x, h->slope_y, h->rough, h->guess};
    for (int i = 0; i < 6; i++)
        if (dst[i]) CUDA_TRY(cudaMemcpyAsync(dst[i], src[i], b, cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return GVOM_OK;
}

int gvom_set_stream(GvomHandle *h, void *stream) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    h->st_dirty = true;  // work on the instance stream: see the step pipeline
    cudaStream_t ns = stream ? static_cast<cudaStream_t>(stream) : h->own;
    if (ns != h->st) {
        // order the new stream after everything queued so far
        cudaEvent_t ev;
        CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        cudaError_t e = cudaEventRecord(ev, h->st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ns, ev, 0);
        cudaEventDestroy(ev);
        if (e != cudaSuccess) return fail(GVOM_ERR_CUDA, std::string("set_stream: ") + cudaGetErrorString(e));
        h->st = ns;
    }
    return GVOM_OK;
}

int gvom_synchronize(GvomHandle *h) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    CUDA_TRY(cudaStreamSynchronize(h->st));
    CUDA_TRY(cudaGetLastError());
    return GVOM_OK;
}

int gvom_last_process_stats(GvomHandle *h, int64_t *valid_points, int64_t *hits, int64_t *ray_steps) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    if (h->last_ctr < 0) return fail(GVOM_NO_DATA, "no scan processed yet");
    ScanCounters c;
    CUDA_TRY(cudaMemcpyAsync(&c, h->d_ctr + h->last_ctr, sizeof(c), cudaMemcpyDeviceToHost, h->st));
    CUDA_TRY(cudaStreamSynchronize(h->st));
    if (c.overflow) return fail(GVOM_ERR_STATE, "record capacity overflow in the last scan");
    if (valid_points) *valid_points = (int64_t)c.valid;
    if (hits) *hits = (int64_t)c.hits;
    if (ray_steps) *ray_steps = (int64_t)c.steps;
    return GVOM_OK;
}

int gvom_set_tuning(GvomHandle *h, const GvomTuning *t) {
    if (!h || !t) return fail(GVOM_ERR_ARG, "handle or tuning is NULL");
    if (!(t->points_per_block == 128 || t->points_per_block == 256))
        return fail(GVOM_ERR_ARG, "points_per_block must be 128 or 256");
    if (!(t->merge_planes_per_thread == 4 || t->merge_planes_per_thread == 8 || t->merge_planes_per_thread == 16))
        return fail(GVOM_ERR_ARG, "merge_planes_per_thread must be 4, 8 or 16");
    if (!(t->stats_blocks_per_sm == 2 || t->stats_blocks_per_sm == 4 || t->stats_blocks_per_sm == 8))
        return fail(GVOM_ERR_ARG, "stats_blocks_per_sm must be 2, 4 or 8");
    if (!(t->step_overlap == 0 || t->step_overlap == 1)) return fail(GVOM_ERR_ARG, "step_overlap must be 0 or 1");
    if (!(t->maps_tile_cells == 64 || t->maps_tile_cells == 128 || t->maps_tile_cells == 224 ||
          t->maps_tile_cells == 256))
        return fail(GVOM_ERR_ARG, "maps_tile_cells must be 64, 128, 224 or 256");
    if (!(t->step_pipeline >= 0 && t->step_pipeline <= 2)) return fail(GVOM_ERR_ARG, "step_pipeline must be 0, 1 or 2");
    std::lock_guard<std::mutex> lk(h->mu);
    h->tun.pts_block = t->points_per_block;
    h->tun.merge_planes = t->merge_planes_per_thread;
    h->tun.stats_bpsm = t->stats_blocks_per_sm;
    h->tun.step_overlap = t->step_overlap;
    h->tun.maps_tile = t->maps_tile_cells;
    h->tun.step_pipeline = t->step_pipeline;
    return GVOM_OK;
}

int gvom_get_tuning(GvomHandle *h, GvomTuning *t) {
    if (!h || !t) return fail(GVOM_ERR_ARG, "handle or tuning is NULL");
    std::lock_guard<std::mutex> lk(h->mu);
    t->points_per_block = h->tun.pts_block;
    t->merge_planes_per_thread = h->tun.merge_planes;
    t->stats_blocks_per_sm = h->tun.stats_bpsm;
    t->step_overlap = h->tun.step_overlap;
    t->maps_tile_cells = h->tun.maps_tile;
    t->step_pipeline = h->tun.step_pipeline;
    return GVOM_OK;
}

int gvom_set_graphs(GvomHandle *h, int32_t on) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    h->graphs = on != 0;
    return GVOM_OK;
}

int gvom_set_stage_timing(GvomHandle *h, int32_t on) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    h->timer.reset();
    h->timer.on = on != 0;
    return GVOM_OK;
}

int gvom_stage_times(GvomHandle *h, double *total_ms, int64_t *launches, int32_t n_stages) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    std::lock_guard<std::mutex> lk(h->mu);
    h->timer.harvest();
    for (int i = 0; i < n_stages && i < kStages; i++) {
        if (total_ms) total_ms[i] = h->timer.ms[i];
        if (launches) launches[i] = h->timer.n[i];
    }
    return GVOM_OK;
}

const char *gvom_stage_name(int32_t stage) {
    return (stage >= 0 && stage < kStages) ? kStageNames[stage] : "";
}

int gvom_device_bytes(GvomHandle *h, int64_t *bytes) {
    if (!h || !bytes) return fail(GVOM_ERR_ARG, "NULL argument");
    *bytes = h->bytes;
    return GVOM_OK;
}

int gvom_expand_binary(const int32_t *d_in, int32_t *d_out, int32_t xy_size, double r, void *stream) {
    if (!d_in || !d_out || xy_size <= 0) return fail(GVOM_ERR_ARG, "expand_binary: NULL image or size <= 0");
    if (!(r < 4096.0)) return fail(GVOM_ERR_ARG, "expand_binary: radius must be below 4096");
    CUDA_TRY(launch_expand_binary(d_in, d_out, xy_size, r, static_cast<cudaStream_t>(stream)));
    return GVOM_OK;
}

int gvom_lowpass_binary(const int32_t *d_in, int32_t *d_out, int32_t xy_size, int32_t filter_size,
                        double filter_fraction, void *stream) {
    if (!d_in || !d_out || xy_size <= 0) return fail(GVOM_ERR_ARG, "lowpass_binary: NULL image or size <= 0");
    if (filter_size < 0 || filter_size > 1023) return fail(GVOM_ERR_ARG, "lowpass_binary: filter_size must be in [0, 1023]");
    CUDA_TRY(launch_lowpass_binary(d_in, d_out, xy_size, filter_size, filter_fraction,
                                   static_cast<cudaStream_t>(stream)));
    return GVOM_OK;
}

int gvom_convolve(const double *d_in, double *d_out, const double *d_kernel, int32_t xy_size, int32_t kernel_size,
                  void *stream) {
    if (!d_in || !d_out || !d_kernel || xy_size <= 0) return fail(GVOM_ERR_ARG, "convolve: NULL buffer or size <= 0");
    if (kernel_size < 1 || kernel_size > 255) return fail(GVOM_ERR_ARG, "convolve: kernel_size must be in [1, 255]");
    CUDA_TRY(launch_convolve(d_in, d_out, d_kernel, xy_size, kernel_size, static_cast<cudaStream_t>(stream)));
    return GVOM_OK;
}

int gvom_reserve(GvomHandle *h, int32_t max_scans, int64_t max_points, int64_t max_row_bytes) {
    if (!h) return fail(GVOM_ERR_ARG, "handle is NULL");
    DeviceScope ds(h->dev);
    if (max_scans < 1 || max_scans > kMaxBatch) return fail(GVOM_ERR_ARG, "max_scans must be in [1, 16]");
    if (max_points < 0 || max_row_bytes < 0) return fail(GVOM_ERR_ARG, "negative size");
    std::lock_guard<std::mutex> lk(h->mu);
    CUDA_TRY(cudaStreamSynchronize(h->st));
    int rc;
    for (int set = 0; set < 2; set++)
        if ((rc = ensure_cnt(h, max_scans, set))) return rc;
    if ((rc = ensure_points(h, std::max<long long>(max_points, 1)))) return rc;
    const size_t stage = (size_t)max_points * (size_t)max_row_bytes + 256 * (size_t)max_scans;
    if ((rc = ensure_dpts(h, stage))) return rc;
    const int want = std::min(kMaxPhysSlots, h->B + 2 * max_scans);
    while ((int)h->slots.size() < want)
        if ((rc = add_slot(h))) return rc;
    for (int s = 0; s < (int)h->slots.size(); s++)
        if ((rc = ensure_slot(h, s, max_points))) return rc;
    CUDA_TRY(cudaStreamSynchronize(h->st));
    return GVOM_OK;
}

}  // extern "C"
