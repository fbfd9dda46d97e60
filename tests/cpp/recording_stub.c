/* A stand-in for libgvom_gb300.so that records the arguments of the calls the
 * Python binding makes (tests/test_binding_cpu.py).  Compiled against the real
 * header, so every signature is the library's.  No computation: process and
 * combine calls only store their arguments; combine writes a marker origin. */
#include <stdint.h>
#include <string.h>

#include "gvom_gb300.h"

static int handle_storage;
/* process / process_device */
const void *rec_points;
int32_t rec_dtype, rec_tdtype, rec_device;
int64_t rec_n, rec_stride;
double rec_ego[3];
const void *rec_transform;
/* process_batch / step */
GvomScan rec_scans[16];
int32_t rec_nscans, rec_points_on_device, rec_outputs_on_device;
/* combine / step outputs */
void *rec_out[5];
int32_t rec_calls;

int gvom_create(const GvomParams *params, GvomHandle **out) {
    (void)params;
    *out = (GvomHandle *)&handle_storage;
    return GVOM_OK;
}
int gvom_destroy(GvomHandle *h) { (void)h; return GVOM_OK; }

static int rec_process(const void *points, int32_t dtype, int64_t n, int64_t row_stride, const double ego[3],
                       const void *transform, int32_t transform_dtype, int32_t device) {
    rec_points = points;
    rec_dtype = dtype;
    rec_n = n;
    rec_stride = row_stride;
    memcpy(rec_ego, ego, sizeof rec_ego);
    rec_transform = transform;
    rec_tdtype = transform_dtype;
    rec_device = device;
    rec_calls++;
    return GVOM_OK;
}
int gvom_process(GvomHandle *h, const void *points, int32_t dtype, int64_t n, int64_t row_stride,
                 const double ego_position[3], const void *transform, int32_t transform_dtype) {
    (void)h;
    return rec_process(points, dtype, n, row_stride, ego_position, transform, transform_dtype, 0);
}
int gvom_process_device(GvomHandle *h, const void *d_points, int32_t dtype, int64_t n, int64_t row_stride,
                        const double ego_position[3], const void *transform, int32_t transform_dtype) {
    (void)h;
    return rec_process(d_points, dtype, n, row_stride, ego_position, transform, transform_dtype, 1);
}
static void rec_batch(const GvomScan *scans, int32_t n_scans, int32_t on_device) {
    rec_nscans = n_scans;
    rec_points_on_device = on_device;
    for (int i = 0; i < n_scans && i < 16; i++) rec_scans[i] = scans[i];
    rec_calls++;
}
int gvom_process_batch(GvomHandle *h, const GvomScan *scans, int32_t n_scans, int32_t points_on_device) {
    (void)h;
    rec_batch(scans, n_scans, points_on_device);
    return GVOM_OK;
}
static void rec_outputs(double origin[3], void *a, void *b, void *c, void *d) {
    rec_out[0] = origin;
    rec_out[1] = a;
    rec_out[2] = b;
    rec_out[3] = c;
    rec_out[4] = d;
    origin[0] = 1.5;
    origin[1] = -2.5;
    origin[2] = 0.25;
}
int gvom_combine(GvomHandle *h, double origin[3], int32_t *pos, int32_t *neg, double *roughness, int32_t *vis) {
    (void)h;
    rec_outputs(origin, pos, neg, roughness, vis);
    rec_calls++;
    return GVOM_OK;
}
int gvom_step(GvomHandle *h, const GvomScan *scans, int32_t n_scans, int32_t points_on_device, double origin[3],
              int32_t *pos, int32_t *neg, double *roughness, int32_t *visibility, int32_t outputs_on_device) {
    (void)h;
    rec_batch(scans, n_scans, points_on_device);
    rec_outputs(origin, pos, neg, roughness, visibility);
    rec_outputs_on_device = outputs_on_device;
    return GVOM_OK;
}
const char *gvom_last_error(void) { return "recording stub"; }
const char *gvom_version(void) { return "recording stub"; }
const char *gvom_stage_name(int32_t stage) { (void)stage; return "stub"; }

/* the rest of the ABI: present so the binding loads; never called by the test */
#define STUB(name, ...) int name(__VA_ARGS__) { return GVOM_ERR_STATE; }
STUB(gvom_combine_device, GvomHandle *h, double o[3], int32_t *a, int32_t *b, double *c, int32_t *d)
STUB(gvom_debug_voxel_map, GvomHandle *h, float *o, int64_t c, int64_t *r)
STUB(gvom_debug_voxel_map_noalloc, GvomHandle *h, float *o, int64_t c, int64_t *r)
STUB(gvom_set_graphs, GvomHandle *h, int32_t on)
STUB(gvom_ros_grids, GvomHandle *h, const GvomRosParams *p, int8_t *a, int8_t *b, int8_t *c, int8_t *d, int8_t *e,
     int32_t od)
STUB(gvom_process_pointcloud2, GvomHandle *h, const void *d, int64_t n, int32_t s, const int32_t o[3], int32_t f,
     int32_t dev, const double e[3], const double t[3], const double q[4])
STUB(gvom_pose_to_transform, const double t[3], const double q[4], double o[16])
STUB(gvom_set_tuning, GvomHandle *h, const GvomTuning *t)
STUB(gvom_get_tuning, GvomHandle *h, GvomTuning *t)
STUB(gvom_debug_height_map, GvomHandle *h, float *o)
STUB(gvom_debug_inferred_height_map, GvomHandle *h, float *o)
STUB(gvom_ring_state, GvomHandle *h, int64_t *a, int64_t *b)
STUB(gvom_slot_count, GvomHandle *h, int32_t s, int64_t *c)
STUB(gvom_get_slot, GvomHandle *h, int32_t s, int32_t *a, int32_t *b, int32_t *c, float *d, float *e, double f[3])
STUB(gvom_combined_count, GvomHandle *h, int64_t *c)
STUB(gvom_get_combined, GvomHandle *h, int32_t *a, int32_t *b, int32_t *c, float *d, float *e, float *f,
     double g[3])
STUB(gvom_get_maps, GvomHandle *h, double *a, double *b, double *c, double *d, double *e, double *f)
STUB(gvom_set_stream, GvomHandle *h, void *s)
STUB(gvom_synchronize, GvomHandle *h)
STUB(gvom_set_stage_timing, GvomHandle *h, int32_t on)
STUB(gvom_stage_times, GvomHandle *h, double *a, int64_t *b, int32_t n)
STUB(gvom_last_process_stats, GvomHandle *h, int64_t *a, int64_t *b, int64_t *c)
STUB(gvom_device_bytes, GvomHandle *h, int64_t *b)
STUB(gvom_reserve, GvomHandle *h, int32_t s, int64_t p, int64_t b)
STUB(gvom_expand_binary, const int32_t *a, int32_t *b, int32_t n, double r, void *s)
STUB(gvom_lowpass_binary, const int32_t *a, int32_t *b, int32_t n, int32_t f, double q, void *s)
STUB(gvom_convolve, const double *a, double *b, const double *k, int32_t n, int32_t ks, void *s)
