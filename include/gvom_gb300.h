/*
 * gvom_gb300.h - C ABI of the GB300-native G-VOM scan->map hot path.
 *
 * One handle = one map instance (the reference's `Gvom` object): a ring of
 * `buffer_size` per-scan voxel maps plus the previous combined map, all held
 * in device memory.  Every entry point returns a status code (GVOM_OK = 0);
 * gvom_last_error() gives the message of the calling thread's last failure.
 * Calls on one handle are serialised by the library, so process and combine
 * may be issued from different threads as the reference allows
 * (README.md:49, scripts/gvom.py:198-208, 243-292, 333-336).
 *
 * Arrays:
 *   points     (n, row_stride) row-major, dtype GVOM_F32 or GVOM_F64; columns 0-2 are x, y, z
 *   transform  4x4 row-major, GVOM_F32 or GVOM_F64, or NULL (no transform)
 *   2-D maps   (xy_size, xy_size) row-major [x][y] (y fastest), like the reference's outputs
 *   voxel id   x + y*xy_size + z*xy_size*xy_size (scripts/gvom.py:1167)
 */
#ifndef GVOM_GB300_H
#define GVOM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GVOM_OK 0
#define GVOM_NO_DATA 1     /* combine/debug on an empty ring (scripts/gvom.py:225-227, 396-431) */
#define GVOM_ERR_ARG 2     /* bad argument (shape, dtype, null pointer, size limit) */
#define GVOM_ERR_OOM 3     /* device allocation failed or refused by the free-memory admission check */
#define GVOM_ERR_CUDA 4    /* CUDA runtime error (message in gvom_last_error) */
#define GVOM_ERR_TIMEOUT 5 /* a bounded wait ran out */
#define GVOM_ERR_STATE 6   /* call not valid in the handle's current state */

#define GVOM_NONE (-1)
#define GVOM_F32 0
#define GVOM_F64 1

/* Constructor parameters, in the order of Gvom.__init__ (scripts/gvom.py:21-22). */
typedef struct GvomParams {
    double xy_resolution;
    double z_resolution;
    int32_t xy_size;
    int32_t z_size;
    int32_t buffer_size;
    double min_distance;
    double positive_obstacle_threshold;
    double negative_obstacle_threshold;
    double slope_obstacle_threshold;
    double robot_height;
    double robot_radius;
    double ground_to_lidar_height;
    int32_t xy_eigen_dist;
    int32_t z_eigen_dist;
} GvomParams;

typedef struct GvomHandle GvomHandle;

/* One scan of a batch (see gvom_process_batch). */
typedef struct GvomScan {
    const void *points;      /* host or device pointer, per `points_on_device` of the call */
    int32_t dtype;           /* GVOM_F32 / GVOM_F64 */
    int32_t transform_dtype; /* GVOM_NONE / GVOM_F32 / GVOM_F64 */
    int64_t n;
    int64_t row_stride;      /* elements per row, >= 3 */
    double ego[3];
    const void *transform;   /* host pointer, 16 elements, or NULL */
} GvomScan;

/* Replaces Gvom.__init__ (scripts/gvom.py:21-101).  Allocates the instance's
 * device state; refuses (GVOM_ERR_OOM) when free device memory is short. */
int gvom_create(const GvomParams *params, GvomHandle **out);

/* Releases every device buffer of the instance. */
int gvom_destroy(GvomHandle *h);

/* Replaces Gvom.Process_pointcloud (scripts/gvom.py:105-217): voxelises one
 * scan (optional 4x4 transform, hit counts, ray-traced pass-through counts,
 * per-voxel statistics) into ring slot `buffer_index` and advances the ring.
 * `points` is a host pointer; it may be reused when the call returns. */
int gvom_process(GvomHandle *h, const void *points, int32_t dtype, int64_t n, int64_t row_stride,
                 const double ego[3], const void *transform, int32_t transform_dtype);

/* Same as gvom_process with `points` already in device memory (stream-ordered
 * on the instance stream; the buffer must stay valid until the work is done). */
int gvom_process_device(GvomHandle *h, const void *d_points, int32_t dtype, int64_t n,
                        int64_t row_stride, const double ego[3], const void *transform,
                        int32_t transform_dtype);

/* A PointCloud2 scan as the reference's ROS node maps it (scripts/gvom_ros.py:
 * 85-109): the cloud's little-endian x / y / z fields (field_dtype GVOM_F32 or
 * GVOM_F64, byte offsets in xyz_offsets, point_step bytes per point) widened
 * to float64 as ros_numpy's pointcloud2_to_xyz_array does, points with a
 * non-finite coordinate dropped, and the sensor pose given as the tf lookup's
 * translation and quaternion (x, y, z, w) turned into the float64 4x4
 * transform of tf's fromTranslationRotation; then Process_pointcloud.
 * `data` is host memory (copied) or, with data_on_device, device memory. */
int gvom_process_pointcloud2(GvomHandle *h, const void *data, int64_t n_points, int32_t point_step,
                             const int32_t xyz_offsets[3], int32_t field_dtype, int32_t data_on_device,
                             const double ego[3], const double translation[3], const double rotation_xyzw[4]);

/* The float64 4x4 transform of tf's fromTranslationRotation (row major). */
int gvom_pose_to_transform(const double translation[3], const double rotation_xyzw[4], double out[16]);

/* Several scans, equivalent to calling gvom_process on each in order, run as
 * one set of launches over all scans.  No reference counterpart; it serves
 * multi-sensor callers of Process_pointcloud (README.md:49). */
int gvom_process_batch(GvomHandle *h, const GvomScan *scans, int32_t n_scans, int32_t points_on_device);

/* Replaces Gvom.combine_maps (scripts/gvom.py:222-393).  Writes the world
 * origin of the map (3 doubles) and the positive-obstacle, negative-obstacle,
 * roughness and visibility maps into host buffers.  GVOM_NO_DATA when the
 * last written slot is empty.  Buffers laid out back to back as roughness
 * (X*X doubles), pos, neg, visibility (X*X int32 each) -- the library's own
 * device layout -- come down in one copy; any other layout takes four. */
int gvom_combine(GvomHandle *h, double origin[3], int32_t *pos, int32_t *neg, double *roughness,
                 int32_t *visibility);

/* Same as gvom_combine with the four maps written to device memory,
 * stream-ordered on the instance stream (no host synchronisation). */
int gvom_combine_device(GvomHandle *h, double origin[3], int32_t *d_pos, int32_t *d_neg,
                        double *d_roughness, int32_t *d_visibility);

/* One scan-to-map step: gvom_process_batch followed by gvom_combine (host
 * outputs) or gvom_combine_device (outputs_on_device != 0), with the same
 * results; no counterpart in the reference.  Submitted together, the index
 * merge of the combine runs beside the process call's statistics kernels
 * (it needs only the ring's index maps).  With step_pipeline (GvomTuning),
 * steps submitted back to back overlap: at 1 a step's ray tracing runs on a
 * second stream beside the previous step's combine; at 2 the rest of its
 * process and its merge also run, on a third stream, beside the previous
 * step's columns and 2-D maps.  A step with host outputs ends with a host
 * wait, so it runs as at 0.  The maps are complete in stream order of the
 * instance stream either way; in graph mode each stream's part of a step is
 * one executable graph. */
int gvom_step(GvomHandle *h, const GvomScan *scans, int32_t n_scans, int32_t points_on_device, double origin[3],
              int32_t *pos, int32_t *neg, double *roughness, int32_t *visibility, int32_t outputs_on_device);

/* Replaces Gvom.make_debug_voxel_map (scripts/gvom.py:395-410, 481-503):
 * rows [x, y, z, hit/total, hit, l0-l1, l1-l2, l2] of every occupied voxel of
 * the combined map, in ascending voxel-id order.  *rows = number of rows; at
 * most `capacity_rows` are written (call with out = NULL to size). */
int gvom_debug_voxel_map(GvomHandle *h, float *out, int64_t capacity_rows, int64_t *rows);

/* Allocation-free form of gvom_debug_voxel_map; no counterpart in the
 * reference.  For callers that must not allocate or free device memory: a
 * debug publisher sharing the GPU with a latency-bound mapping loop (cudaFree
 * synchronises the device and stalls every other instance's work), or a
 * process whose device footprint must stay fixed after start-up.  The same
 * rows, in the same order, go to `d_out`, a DEVICE buffer of capacity_rows x 8
 * floats owned by the caller (NULL or capacity 0: only size).  The only
 * scratch is a fixed 128 KB device array; grids above 32M voxels
 * (xy_size^2 * z_size > 33,554,432) are refused with GVOM_ERR_ARG.  The first
 * call on a device looks up that array's address; make it before any stream
 * capture.  The array is shared by all instances on a device: calls are
 * serialised by a process-wide lock held until their device work is done.
 * Returns after the rows are written (host waits on the instance stream). */
int gvom_debug_voxel_map_noalloc(GvomHandle *h, float *d_out, int64_t capacity_rows, int64_t *rows);

/* The OccupancyGrid payloads the reference's ROS node builds from
 * combine_maps' result (scripts/gvom_ros.py:141-164), computed on the device
 * from the last combine: hard obstacles max(100 (pos > density_threshold),
 * neg); soft obstacles 100 (0 < pos <= density_threshold); ground certainty
 * 100 vis; negative obstacles; roughness ((clip(r, min, max) + min) /
 * (max - min)) 100.  Each is xy_size^2 int8 in the node's column-major order
 * (x fastest), cast as numpy does on an x86 host (truncation, low 8 bits).
 * Any output may be NULL.  Node defaults: density_threshold 50,
 * min_roughness -10, max_roughness 0 (launch/gvom_node.launch:17-20). */
typedef struct GvomRosParams {
    double density_threshold;
    double min_roughness;
    double max_roughness;
} GvomRosParams;
int gvom_ros_grids(GvomHandle *h, const GvomRosParams *params, int8_t *hard, int8_t *soft, int8_t *certainty,
                   int8_t *negative, int8_t *roughness, int32_t outputs_on_device);

/* Replace make_debug_height_map / make_debug_inferred_height_map
 * (scripts/gvom.py:412-442, 455-479): (xy_size^2, 7) and (xy_size^2, 3) float32. */
int gvom_debug_height_map(GvomHandle *h, float *out);
int gvom_debug_inferred_height_map(GvomHandle *h, float *out);

/* ---- 2-D image kernels that no reference caller launches -----------------
 * Images are xy_size x xy_size, [x][y] row major (y fastest, the layout of
 * the maps), in DEVICE memory; the kernels run on `stream` (a cudaStream_t,
 * NULL for the default stream) without host synchronisation. */

/* Replaces Gvom.__expand_binary (scripts/gvom.py:807-831): out = 1 where a
 * cell equal to 1 lies within the disc of radius r (float64 row extents
 * floor(sqrt(r^2 - i^2)), as the reference), else 0.  r < 4096. */
int gvom_expand_binary(const int32_t *d_in, int32_t *d_out, int32_t xy_size, double r, void *stream);

/* Replaces Gvom.__lowpass_binary (scripts/gvom.py:833-861): out = 0 where in
 * is 0, else 1 where the mean over the (2 filter_size + 1)^2 window, clipped
 * to the image, is >= filter_fraction. */
int gvom_lowpass_binary(const int32_t *d_in, int32_t *d_out, int32_t xy_size, int32_t filter_size,
                        double filter_fraction, void *stream);

/* Replaces Gvom.__convolve (scripts/gvom.py:863-885) with its indexing as
 * written: out[x, y] = sum over the kernel's entries [0, 2r] x [0, 2r], in
 * row order, of in[x + r, y + r] times the entry, 0 where (x + r, y + r) is
 * outside; r = (kernel_size - 1) / 2 in integers (the reference's float
 * radius cannot be passed to range(), so its kernel never runs); the
 * kernel is kernel_size x kernel_size, row major.  kernel_size <= 255. */
int gvom_convolve(const double *d_in, double *d_out, const double *d_kernel, int32_t xy_size, int32_t kernel_size,
                  void *stream);

/* ---- state access for parity checks (host copies) ---------------------- */

/* Ring position: next slot to write and last slot written
 * (Gvom.buffer_index / last_buffer_index, scripts/gvom.py:72-73, 211-216). */
int gvom_ring_state(GvomHandle *h, int64_t *buffer_index, int64_t *last_buffer_index);

/* Occupied-voxel count of ring slot `slot` (-1 if the slot is empty). */
int gvom_slot_count(GvomHandle *h, int32_t slot, int64_t *count);

/* Copies slot `slot`: index map (V int32), per occupied voxel hit, total,
 * min height and 10 statistics (mean xyz, cov xx xy xz yy yz zz, count),
 * and its voxel origin.  Any pointer may be NULL. */
int gvom_get_slot(GvomHandle *h, int32_t slot, int32_t *index, int32_t *hit, int32_t *total,
                  float *min_height, float *metrics, double origin[3]);

/* Occupied-voxel count of the current combined map (-1 before the first combine). */
int gvom_combined_count(GvomHandle *h, int64_t *count);

/* Copies the current combined map (scripts/gvom.py:259-318 state): index map,
 * hit, total, min height, 10 statistics and 3 eigenvalues per occupied voxel,
 * and its voxel origin.  Any pointer may be NULL. */
int gvom_get_combined(GvomHandle *h, int32_t *index, int32_t *hit, int32_t *total, float *min_height,
                      float *metrics, float *eigen, double origin[3]);

/* Copies the 2-D intermediate maps of the last combine (height, inferred
 * height, x/y slope, roughness, guessed height delta), each xy_size^2 float64. */
int gvom_get_maps(GvomHandle *h, double *height, double *inferred, double *slope_x, double *slope_y,
                  double *roughness, double *guess);

/* ---- streams and timing -------------------------------------------------- */

/* Use `stream` (a cudaStream_t) for all further work of this handle; NULL
 * restores the handle's own stream. */
int gvom_set_stream(GvomHandle *h, void *stream);

/* Blocks until all queued work of the handle is complete. */
int gvom_synchronize(GvomHandle *h);

/* Per-kernel device time: when enabled, CUDA events are recorded around each
 * kernel launch of process / combine; gvom_stage_times waits for the queued
 * work and returns, for stages 0..n-1, the summed milliseconds and launch
 * counts since timing was (re-)enabled.  Stage names: gvom_stage_name. */
/* Launch shapes chosen by the autotuner (gvom_gb300/autotune.py); no
 * counterpart in the reference.  They change speed only, never results.
 * Defaults: 256, 8, 4, 1, 256, 2. */
typedef struct GvomTuning {
    int32_t points_per_block;         /* point-parallel kernels: 128 or 256 */
    int32_t merge_planes_per_thread;  /* index merge: 4, 8 or 16 z planes */
    int32_t stats_blocks_per_sm;      /* statistics merge: 2, 4 or 8 */
    int32_t step_overlap;             /* gvom_step: index merge beside the statistics kernels, 0 or 1 */
    int32_t maps_tile_cells;          /* 2-D maps tile: 256 (8 x 32), 224 (14 x 16: 304 blocks at 256^2,
                                         two per SM), 128 (8 x 16) or 64 (4 x 16) */
    int32_t step_pipeline;            /* gvom_step streams: 0 one; 1 the trace beside the previous step's combine;
                                         2 also the process and merge beside the previous step's columns and maps */
} GvomTuning;
int gvom_set_tuning(GvomHandle *h, const GvomTuning *t);
int gvom_get_tuning(GvomHandle *h, GvomTuning *t);

/* CUDA-graph mode (off by default); no counterpart in the reference.  When on,
 * each process / combine call captures its launch sequence and replays it
 * through an executable graph that is updated in place while the sequence
 * keeps its shape (the same batch-size class and source count), which removes
 * per-kernel launch gaps.  Stage timing records nothing while it is on. */
int gvom_set_graphs(GvomHandle *h, int32_t on);

#define GVOM_STAGES 11
int gvom_set_stage_timing(GvomHandle *h, int32_t on);
int gvom_stage_times(GvomHandle *h, double *total_ms, int64_t *launches, int32_t n_stages);
const char *gvom_stage_name(int32_t stage);

/* Device-side counts of the last processed scan: valid points, in-grid hits,
 * ray steps (pass-through increments). */
int gvom_last_process_stats(GvomHandle *h, int64_t *valid_points, int64_t *hits, int64_t *ray_steps);

/* Bytes of device memory held by the handle. */
int gvom_device_bytes(GvomHandle *h, int64_t *bytes);

/* Allocates now what later process / step calls of up to `max_scans` scans
 * (<= 16) and `max_points` points in all would otherwise allocate on first
 * use: both sets of per-scan scratch, the staging buffer for host points of
 * up to `max_row_bytes` bytes per point, record capacity for `max_points`
 * voxels in every ring slot, and the step pipeline's spare slots.  No
 * counterpart in the reference; for request loops whose latency must not
 * include an allocation (cudaFree waits for the whole device).  Waits for the
 * instance's queued work; GVOM_ERR_OOM when device memory is short. */
int gvom_reserve(GvomHandle *h, int32_t max_scans, int64_t max_points, int64_t max_row_bytes);

/* Message of the calling thread's last failed call ("" if none). */
const char *gvom_last_error(void);

/* Library version string. */
const char *gvom_version(void);

#ifdef __cplusplus
}
#endif

#endif /* GVOM_GB300_H */
