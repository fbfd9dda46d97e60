/*
 * TEST INFRASTRUCTURE - the CPU oracle for the G-VOM scan->map hot path.
 *
 * A plain-C restatement of the reference mapper (scripts/gvom.py) used only
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the
 * checker; no product code links or calls it.
 *
 * Every stage follows the reference kernel named beside it, op by op, with the
 * scalar types compiled Numba gives those expressions (float32 where both
 * operands are float32, float64 as soon as a Python float / float64 array /
 * int64 enters, math.floor -> int64, math.sqrt(float32) -> float32).  Build
 * with -ffp-contract=off so no multiply-add is fused (the reference's CPU path,
 * the Numba CUDA simulator, evaluates every operation separately too).
 *
 * Pinned: tests/test_oracle_golden.py checks it, floats included, bit for bit
 * against the reference's own outputs (tests/golden/*.npz, made by running
 * scripts/gvom.py unchanged through tests/golden/make_golden.py).
 *
 * Modes: threads == 1 runs every kernel sequentially in thread-index order
 * (a valid schedule of the reference's launches: its atomics make all integer
 * results order-free, and compact indices are order-dependent but not
 * observable).  threads > 1 runs the same loops under OpenMP with atomics, for
 * the timed CPU baseline only.
 *
 * Divergences from the reference, shared with the GPU path and documented:
 *  - a scan with no points, or with no occupied voxel, is a valid slot (the
 *    reference raises on its zero-block launches, gvom.py:147,173,262);
 *  - a point with a non-finite coordinate is dropped (the reference's
 *    float->int conversion of NaN is undefined);
 *  - combine_maps' visibility map is fully written (gvom.py:378-380 never
 *    initialises it, but its kernel writes every cell, so the result is equal).
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define GVO_OK 0
#define GVO_NO_DATA 1
#define GVO_BAD_ARG 2
#define GVO_OOM 3

typedef struct {
    double xy_resolution, z_resolution;
    int32_t xy_size, z_size, buffer_size;
    double min_distance, positive_obstacle_threshold, negative_obstacle_threshold,
        slope_obstacle_threshold, robot_height, robot_radius, ground_to_lidar_height;
    int32_t xy_eigen_dist, z_eigen_dist;
} gvo_params;

typedef struct {
    int valid;
    int64_t C;
    int32_t *index;   /* V */
    int32_t *hit;     /* C */
    int32_t *total;   /* C */
    double *metrics;  /* C*10: mean xyz, cov xx xy xz yy yz zz, count */
    float *min_h;     /* C */
    double origin[3];
} gvo_slot;

typedef struct {
    int valid;
    int64_t C;
    int32_t *index;
    int32_t *hit, *total;
    float *metrics; /* C*10 */
    float *min_h;
    double origin[3];
} gvo_comb;

typedef struct {
    gvo_params p;
    int64_t X, Z, V;
    int threads;
    gvo_slot *slots;
    int64_t buffer_index, last_buffer_index;
    double ego[3];
    gvo_comb cur, last;
    int have_last;
    float *eigen; /* Cc*3 */
    double *height, *inferred, *rough, *slope_x, *slope_y, *guess; /* X*X, [x][y] */
    int32_t *pos, *neg, *vis;
    int have_maps;
    int32_t *tmp_hit, *tmp_total; /* V scratch */
    int64_t last_ray_steps, last_hits, last_valid_points;
} gvo_map;

static void *xcalloc(size_t n, size_t sz) {
    if (n == 0) n = 1;
    return calloc(n, sz);
}

gvo_map *gvo_create(const gvo_params *p, int threads) {
    if (!p || p->xy_size <= 0 || p->z_size <= 0 || p->buffer_size <= 0) return NULL;
    gvo_map *m = (gvo_map *)calloc(1, sizeof(gvo_map));
    if (!m) return NULL;
    m->p = *p;
    m->X = p->xy_size;
    m->Z = p->z_size;
    m->V = m->X * m->X * m->Z;
    m->threads = threads < 1 ? 1 : threads;
    m->slots = (gvo_slot *)calloc((size_t)p->buffer_size, sizeof(gvo_slot));
    m->tmp_hit = (int32_t *)xcalloc((size_t)m->V, 4);
    m->tmp_total = (int32_t *)xcalloc((size_t)m->V, 4);
    size_t X2 = (size_t)(m->X * m->X);
    m->height = (double *)xcalloc(X2, 8);
    m->inferred = (double *)xcalloc(X2, 8);
    m->rough = (double *)xcalloc(X2, 8);
    m->slope_x = (double *)xcalloc(X2, 8);
    m->slope_y = (double *)xcalloc(X2, 8);
    m->guess = (double *)xcalloc(X2, 8);
    m->pos = (int32_t *)xcalloc(X2, 4);
    m->neg = (int32_t *)xcalloc(X2, 4);
    m->vis = (int32_t *)xcalloc(X2, 4);
    return m;
}

static void slot_free(gvo_slot *s) {
    free(s->index); free(s->hit); free(s->total); free(s->metrics); free(s->min_h);
    memset(s, 0, sizeof(*s));
}
static void comb_free(gvo_comb *c) {
    free(c->index); free(c->hit); free(c->total); free(c->metrics); free(c->min_h);
    memset(c, 0, sizeof(*c));
}

void gvo_destroy(gvo_map *m) {
    if (!m) return;
    for (int i = 0; i < m->p.buffer_size; i++) slot_free(&m->slots[i]);
    free(m->slots);
    comb_free(&m->last); /* `cur` aliases `last` */
    free(m->eigen);
    free(m->tmp_hit); free(m->tmp_total);
    free(m->height); free(m->inferred); free(m->rough); free(m->slope_x); free(m->slope_y);
    free(m->guess); free(m->pos); free(m->neg); free(m->vis);
    free(m);
}

void gvo_set_threads(gvo_map *m, int threads) { m->threads = threads < 1 ? 1 : threads; }

/* ------------------------------------------------------------------------ */
/* atomics (only used when threads > 1)                                       */
/* ------------------------------------------------------------------------ */
static inline int32_t at_add_i32(int32_t *a, int32_t v, int par) {
    if (!par) { int32_t o = *a; *a = o + v; return o; }
    return __atomic_fetch_add(a, v, __ATOMIC_RELAXED);
}
static inline int64_t at_add_i64(int64_t *a, int64_t v, int par) {
    if (!par) { int64_t o = *a; *a = o + v; return o; }
    return __atomic_fetch_add(a, v, __ATOMIC_RELAXED);
}
static inline void at_add_f64(double *a, double v, int par) {
    if (!par) { *a += v; return; }
    int64_t oi = __atomic_load_n((int64_t *)a, __ATOMIC_RELAXED), ni;
    double old, nw;
    do {
        memcpy(&old, &oi, 8);
        nw = old + v;
        memcpy(&ni, &nw, 8);
    } while (!__atomic_compare_exchange_n((int64_t *)a, &oi, ni, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED));
}
static inline void at_min_f32(float *a, float v, int par) {
    if (!par) { if (v < *a) *a = v; return; }
    int32_t oi, ni;
    float old;
    oi = __atomic_load_n((int32_t *)a, __ATOMIC_RELAXED);
    for (;;) {
        memcpy(&old, &oi, 4);
        if (!(v < old)) return;
        memcpy(&ni, &v, 4);
        if (__atomic_compare_exchange_n((int32_t *)a, &oi, ni, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
    }
}

/* ------------------------------------------------------------------------ */
/* point access                                                               */
/* ------------------------------------------------------------------------ */
typedef struct {
    int is64;
    int64_t n;
    float *f;
    double *d;
} pts_t;

static inline double px(const pts_t *P, int64_t i, int k) {
    return P->is64 ? P->d[i * 3 + k] : (double)P->f[i * 3 + k];
}

/* d2 = x*x + y*y + z*z in the point dtype (gvom.py:1145-1146) */
static inline double point_d2(const pts_t *P, int64_t i) {
    if (P->is64) {
        double x = P->d[i * 3], y = P->d[i * 3 + 1], z = P->d[i * 3 + 2];
        return x * x + y * y + z * z;
    }
    float x = P->f[i * 3], y = P->f[i * 3 + 1], z = P->f[i * 3 + 2];
    float a = x * x;
    float b = y * y;
    float c = z * z;
    float s = a + b;
    s = s + c;
    return (double)s;
}

static inline int point_finite(const pts_t *P, int64_t i) {
    return isfinite(px(P, i, 0)) && isfinite(px(P, i, 1)) && isfinite(px(P, i, 2));
}

/* ------------------------------------------------------------------------ */
/* __transform_pointcloud (gvom.py:1121-1138)                                 */
/* ------------------------------------------------------------------------ */
static void transform_points(pts_t *P, const void *T, int Tdt) {
    for (int64_t i = 0; i < P->n; i++) {
        double out[3];
        if (!P->is64 && Tdt == 0) { /* float32 * float32: all float32 ops */
            const float *t = (const float *)T;
            float p0 = P->f[i * 3], p1 = P->f[i * 3 + 1], p2 = P->f[i * 3 + 2];
            for (int r = 0; r < 3; r++) {
                float a = p0 * t[r * 4 + 0];
                float b = p1 * t[r * 4 + 1];
                float c = p2 * t[r * 4 + 2];
                float s = a + b;
                s = s + c;
                s = s + t[r * 4 + 3];
                out[r] = (double)s;
            }
        } else { /* any float64 operand: float64 ops */
            double p0 = px(P, i, 0), p1 = px(P, i, 1), p2 = px(P, i, 2);
            for (int r = 0; r < 3; r++) {
                double t0, t1, t2, t3;
                if (Tdt == 0) {
                    const float *t = (const float *)T;
                    t0 = t[r * 4]; t1 = t[r * 4 + 1]; t2 = t[r * 4 + 2]; t3 = t[r * 4 + 3];
                } else {
                    const double *t = (const double *)T;
                    t0 = t[r * 4]; t1 = t[r * 4 + 1]; t2 = t[r * 4 + 2]; t3 = t[r * 4 + 3];
                }
                double a = p0 * t0;
                double b = p1 * t1;
                double c = p2 * t2;
                double s = a + b;
                s = s + c;
                s = s + t3;
                out[r] = s;
            }
        }
        for (int r = 0; r < 3; r++) {
            if (P->is64) P->d[i * 3 + r] = out[r];
            else P->f[i * 3 + r] = (float)out[r];
        }
    }
}

/* ------------------------------------------------------------------------ */
/* __point_2_map (gvom.py:1140-1231)                                          */
/* ------------------------------------------------------------------------ */
static void point_2_map(gvo_map *m, const pts_t *P, const double origin[3], const double ego[3],
                        int par, int64_t *steps_out, int64_t *hits_out, int64_t *valid_out) {
    const double xr = m->p.xy_resolution, zr = m->p.z_resolution;
    const int64_t X = m->X, Z = m->Z;
    const double md2 = m->p.min_distance * m->p.min_distance;
    int64_t steps = 0, hits = 0, valid = 0;
    const float pt0 = (float)(ego[0] / xr), pt1 = (float)(ego[1] / xr), pt2 = (float)(ego[2] / zr);
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : steps, hits, valid) if (par)
    for (int64_t i = 0; i < P->n; i++) {
        if (!point_finite(P, i)) continue;
        if (point_d2(P, i) < md2) continue;
        valid++;
        double q0 = px(P, i, 0) / xr, q1 = px(P, i, 1) / xr, q2 = px(P, i, 2) / zr;
        int64_t xi = (int64_t)floor(q0 - origin[0]);
        int64_t yi = (int64_t)floor(q1 - origin[1]);
        int64_t zi = (int64_t)floor(q2 - origin[2]);
        int oob = (xi < 0 || xi >= X) || (yi < 0 || yi >= X) || (zi < 0 || zi >= Z);
        if (!oob) {
            int64_t idx = xi + yi * X + zi * X * X;
            at_add_i32(&m->tmp_hit[idx], 1, par);
            at_add_i32(&m->tmp_total[idx], 1, par);
            hits++;
        }
        float pt[3] = {pt0, pt1, pt2};
        float end[3] = {(float)q0, (float)q1, (float)q2};
        float slope[3];
        slope[0] = end[0] - pt[0];
        slope[1] = end[1] - pt[1];
        slope[2] = end[2] - pt[2];
        float a = slope[0] * slope[0];
        float b = slope[1] * slope[1];
        float c = slope[2] * slope[2];
        float ss = a + b;
        ss = ss + c;
        float ray_length = sqrtf(ss);
        slope[0] = slope[0] / ray_length;
        slope[1] = slope[1] / ray_length;
        slope[2] = slope[2] / ray_length;
        float a0 = fabsf(slope[0]), a1 = fabsf(slope[1]), a2 = fabsf(slope[2]);
        float inner = a2 > a1 ? a2 : a1; /* max(abs(s1), abs(s2)) */
        float smax = inner > a0 ? inner : a0;
        int k = 0;
        if (smax == a1) k = 1;
        if (smax == a2) k = 2;
        int k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        double length = 0.0;
        const float dir = slope[k] / fabsf(slope[k]);
        const double R = (double)ray_length - 1.0;
        while (length < R) {
            pt[k] += dir;
            pt[k1] += slope[k1] / fabsf(slope[k]);
            pt[k2] += slope[k2] / fabsf(slope[k]);
            int64_t x = (int64_t)floor((double)pt[0] - origin[0]);
            if (x < 0 || x >= X) break;
            int64_t y = (int64_t)floor((double)pt[1] - origin[1]);
            if (y < 0 || y >= X) break;
            int64_t z = (int64_t)floor((double)pt[2] - origin[2]);
            if (z < 0 || z >= Z) break;
            at_add_i32(&m->tmp_total[x + y * X + z * X * X], 1, par);
            steps++;
            length += fabs(1.0 / (double)slope[k]);
        }
    }
    *steps_out = steps;
    *hits_out = hits;
    *valid_out = valid;
}

/* ------------------------------------------------------------------------ */
/* __calculate_mean / __calculate_covariance / __calculate_min_height          */
/* (gvom.py:1249-1421) and their normalisations                               */
/* ------------------------------------------------------------------------ */
static void calculate_metrics(gvo_map *m, const pts_t *P, const double origin[3], gvo_slot *s, int par) {
    const double xr = m->p.xy_resolution, zr = m->p.z_resolution;
    const int64_t X = m->X, Z = m->Z;
    const double md2 = m->p.min_distance * m->p.min_distance;
    const int64_t exy = m->p.xy_eigen_dist, ez = m->p.z_eigen_dist;
    double *met = s->metrics;
    const int32_t *index_map = s->index;
    /* mean sums */
#pragma omp parallel for schedule(dynamic, 256) if (par)
    for (int64_t i = 0; i < P->n; i++) {
        if (!point_finite(P, i)) continue;
        if (point_d2(P, i) < md2) continue;
        double q0 = px(P, i, 0) / xr, q1 = px(P, i, 1) / xr, q2 = px(P, i, 2) / zr;
        int64_t xb = (int64_t)floor(q0 - origin[0]);
        int64_t yb = (int64_t)floor(q1 - origin[1]);
        int64_t zb = (int64_t)floor(q2 - origin[2]);
        for (int64_t x = xb - exy; x < xb + 1 + exy; x++) {
            if (x < 0 || x >= X) continue;
            for (int64_t y = yb - exy; y < yb + 1 + exy; y++) {
                if (y < 0 || y >= X) continue;
                for (int64_t z = zb - ez; z < zb + 1 + ez; z++) {
                    if (z < 0 || z >= Z) continue;
                    double l0 = (q0 - origin[0]) - (double)x;
                    double l1 = (q1 - origin[1]) - (double)y;
                    double l2 = (q2 - origin[2]) - (double)z;
                    int32_t idx = index_map[x + y * X + z * X * X];
                    if (idx < 0) continue;
                    at_add_f64(&met[idx * 10 + 0], l0, par);
                    at_add_f64(&met[idx * 10 + 1], l1, par);
                    at_add_f64(&met[idx * 10 + 2], l2, par);
                    at_add_f64(&met[idx * 10 + 9], 1.0, par);
                }
            }
        }
    }
    /* __normalize_mean (gvom.py:1300-1308) */
#pragma omp parallel for if (par)
    for (int64_t c = 0; c < s->C; c++)
        for (int j = 0; j < 3; j++) met[c * 10 + j] = met[c * 10 + j] / met[c * 10 + 9];
    /* covariance sums */
#pragma omp parallel for schedule(dynamic, 256) if (par)
    for (int64_t i = 0; i < P->n; i++) {
        if (!point_finite(P, i)) continue;
        if (point_d2(P, i) < md2) continue;
        double q0 = px(P, i, 0) / xr, q1 = px(P, i, 1) / xr, q2 = px(P, i, 2) / zr;
        int64_t xb = (int64_t)floor(q0 - origin[0]);
        int64_t yb = (int64_t)floor(q1 - origin[1]);
        int64_t zb = (int64_t)floor(q2 - origin[2]);
        for (int64_t x = xb - exy; x < xb + 1 + exy; x++) {
            if (x < 0 || x >= X) continue;
            for (int64_t y = yb - exy; y < yb + 1 + exy; y++) {
                if (y < 0 || y >= X) continue;
                for (int64_t z = zb - ez; z < zb + 1 + ez; z++) {
                    if (z < 0 || z >= Z) continue;
                    double l0 = (q0 - origin[0]) - (double)x;
                    double l1 = (q1 - origin[1]) - (double)y;
                    double l2 = (q2 - origin[2]) - (double)z;
                    int32_t idx = index_map[x + y * X + z * X * X];
                    if (idx < 0) continue;
                    double *r = &met[idx * 10];
                    at_add_f64(&r[3], (l0 - r[0]) * (l0 - r[0]), par);
                    at_add_f64(&r[4], (l0 - r[0]) * (l1 - r[1]), par);
                    at_add_f64(&r[5], (l0 - r[0]) * (l2 - r[2]), par);
                    at_add_f64(&r[6], (l1 - r[1]) * (l1 - r[1]), par);
                    at_add_f64(&r[7], (l1 - r[1]) * (l2 - r[2]), par);
                    at_add_f64(&r[8], (l2 - r[2]) * (l2 - r[2]), par);
                }
            }
        }
    }
    /* __normalize_covariance (gvom.py:1375-1387) */
#pragma omp parallel for if (par)
    for (int64_t c = 0; c < s->C; c++)
        for (int j = 0; j < 6; j++) {
            if (met[c * 10 + 9] <= 0) met[c * 10 + j + 3] = 0;
            else met[c * 10 + j + 3] = met[c * 10 + j + 3] / met[c * 10 + 9];
        }
    /* __calculate_min_height (gvom.py:1389-1421) */
#pragma omp parallel for schedule(dynamic, 256) if (par)
    for (int64_t i = 0; i < P->n; i++) {
        if (!point_finite(P, i)) continue;
        if (point_d2(P, i) < md2) continue;
        double q0 = px(P, i, 0) / xr, q1 = px(P, i, 1) / xr, q2 = px(P, i, 2) / zr;
        int64_t x = (int64_t)floor(q0 - origin[0]);
        if (x < 0 || x >= X) continue;
        int64_t y = (int64_t)floor(q1 - origin[1]);
        if (y < 0 || y >= X) continue;
        int64_t z = (int64_t)floor(q2 - origin[2]);
        if (z < 0 || z >= Z) continue;
        double l2 = (q2 - origin[2]) - (double)z;
        int32_t idx = index_map[x + y * X + z * X * X];
        at_min_f32(&s->min_h[idx], (float)l2, par);
    }
}

/* ------------------------------------------------------------------------ */
/* Process_pointcloud (gvom.py:105-217)                                       */
/* ------------------------------------------------------------------------ */
int gvo_process(gvo_map *m, const void *points, int dtype, int64_t n, int64_t row_stride,
                const double ego[3], const void *T, int Tdt) {
    if (!m || n < 0 || (n > 0 && !points) || (dtype != 0 && dtype != 1) || !ego) return GVO_BAD_ARG;
    if (T && Tdt != 0 && Tdt != 1) return GVO_BAD_ARG;
    if (row_stride < 3) return GVO_BAD_ARG;
    const int par = m->threads > 1;
#ifdef _OPENMP
    if (par) omp_set_num_threads(m->threads);
#endif
    m->ego[0] = ego[0]; m->ego[1] = ego[1]; m->ego[2] = ego[2];
    const int64_t X = m->X, Z = m->Z, V = m->V;
    pts_t P = {dtype == 1, n, NULL, NULL};
    if (P.is64) {
        P.d = (double *)xcalloc((size_t)n * 3, 8);
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) P.d[i * 3 + k] = ((const double *)points)[i * row_stride + k];
    } else {
        P.f = (float *)xcalloc((size_t)n * 3, 4);
        for (int64_t i = 0; i < n; i++)
            for (int k = 0; k < 3; k++) P.f[i * 3 + k] = ((const float *)points)[i * row_stride + k];
    }
    /* gvom.py:119-131: index_map = -1, tmp_hit = tmp_total = 0 */
    memset(m->tmp_hit, 0, (size_t)V * 4);
    memset(m->tmp_total, 0, (size_t)V * 4);
    /* gvom.py:138-141 */
    double origin[3];
    origin[0] = floor((ego[0] / m->p.xy_resolution) - (double)X / 2.0);
    origin[1] = floor((ego[1] / m->p.xy_resolution) - (double)X / 2.0);
    origin[2] = floor((ego[2] / m->p.z_resolution) - (double)Z / 2.0);
    if (T) transform_points(&P, T, Tdt);
    point_2_map(m, &P, origin, ego, par, &m->last_ray_steps, &m->last_hits, &m->last_valid_points);

    gvo_slot ns;
    memset(&ns, 0, sizeof(ns));
    ns.index = (int32_t *)xcalloc((size_t)V, 4);
    /* __assign_indices (gvom.py:1233-1240); sequential mode allocates in voxel order */
    int64_t cell_count = 0;
    if (!par) {
        for (int64_t v = 0; v < V; v++) {
            if (m->tmp_hit[v] > 0) ns.index[v] = (int32_t)(cell_count++);
            else ns.index[v] = -m->tmp_total[v] - 1;
        }
    } else {
#pragma omp parallel for schedule(static, 4096)
        for (int64_t v = 0; v < V; v++) {
            if (m->tmp_hit[v] > 0) ns.index[v] = (int32_t)at_add_i64(&cell_count, 1, 1);
            else ns.index[v] = -m->tmp_total[v] - 1;
        }
    }
    ns.C = cell_count;
    ns.hit = (int32_t *)xcalloc((size_t)ns.C, 4);
    ns.total = (int32_t *)xcalloc((size_t)ns.C, 4);
    /* __move_data x2 (gvom.py:1242-1247) */
#pragma omp parallel for schedule(static, 4096) if (par)
    for (int64_t v = 0; v < V; v++) {
        int32_t c = ns.index[v];
        if (c >= 0) {
            ns.hit[c] = m->tmp_hit[v];
            ns.total[c] = m->tmp_total[v];
        }
    }
    /* __calculate_metrics_master (gvom.py:1069-1119) */
    ns.metrics = (double *)xcalloc((size_t)ns.C * 10, 8);
    ns.min_h = (float *)xcalloc((size_t)ns.C, 4);
    for (int64_t c = 0; c < ns.C; c++) ns.min_h[c] = 1.0f;
    calculate_metrics(m, &P, origin, &ns, par);
    ns.origin[0] = origin[0]; ns.origin[1] = origin[1]; ns.origin[2] = origin[2];
    ns.valid = 1;
    /* slot write + ring advance (gvom.py:198-216) */
    slot_free(&m->slots[m->buffer_index]);
    m->slots[m->buffer_index] = ns;
    m->last_buffer_index = m->buffer_index;
    m->buffer_index += 1;
    if (m->buffer_index >= m->p.buffer_size) m->buffer_index = 0;
    free(P.f);
    free(P.d);
    (void)Z;
    return GVO_OK;
}

/* ------------------------------------------------------------------------ */
/* __combine_indices / __combine_old_indices (gvom.py:1009-1063)              */
/* ------------------------------------------------------------------------ */
static void combine_indices(gvo_map *m, int32_t *cidx, const double co[3], const int32_t *oidx,
                            const double oo[3], int64_t *counter, int old_rule, int par) {
    const int64_t X = m->X, Z = m->Z;
    const double dx = co[0] - oo[0], dy = co[1] - oo[1], dz = co[2] - oo[2];
#pragma omp parallel for collapse(2) schedule(static) if (par)
    for (int64_t z = 0; z < Z; z++)
        for (int64_t y = 0; y < X; y++)
            for (int64_t x = 0; x < X; x++) {
                if (((double)x + dx) >= (double)X || ((double)y + dy) >= (double)X ||
                    ((double)z + dz) >= (double)Z || ((double)x + dx) < 0 || ((double)y + dy) < 0 ||
                    ((double)z + dz) < 0)
                    continue;
                int64_t index = x + y * X + z * X * X;
                int64_t index_old = (int64_t)(((double)x + dx) + ((double)y + dy) * (double)X +
                                              ((double)z + dz) * (double)X * (double)X);
                int32_t o = oidx[index_old];
                int32_t c = cidx[index];
                int alloc = old_rule ? (o >= 0 && c <= -1 && c >= -11) : (o >= 0 && c <= -1);
                if (alloc) cidx[index] = (int32_t)at_add_i64(counter, 1, par);
                else if (o < -1 && c <= -1) cidx[index] = c + (o + 1);
            }
}

/* ------------------------------------------------------------------------ */
/* __combine_metrics (gvom.py:888-980).  `om` is float64 for a ring slot and  */
/* float32 for the previous combined map; the arithmetic types follow that.   */
/* ------------------------------------------------------------------------ */
#define CM(j) (cm[(j)])
static void combine_metrics(gvo_map *m, gvo_comb *cb, const int32_t *oidx, const double oo[3],
                            const double *om64, const float *om32, const int32_t *ohit,
                            const int32_t *ototal, const float *omin, int par) {
    const int64_t X = m->X, Z = m->Z;
    const double *co = cb->origin;
    const double dx = co[0] - oo[0], dy = co[1] - oo[1], dz = co[2] - oo[2];
#pragma omp parallel for collapse(2) schedule(static) if (par)
    for (int64_t z = 0; z < Z; z++)
        for (int64_t y = 0; y < X; y++)
            for (int64_t x = 0; x < X; x++) {
                if (((double)x + dx) >= (double)X || ((double)y + dy) >= (double)X ||
                    ((double)z + dz) >= (double)Z || ((double)x + dx) < 0 || ((double)y + dy) < 0 ||
                    ((double)z + dz) < 0)
                    continue;
                int32_t index = cb->index[x + y * X + z * X * X];
                int32_t io = oidx[(int64_t)(((double)x + dx) + ((double)y + dy) * (double)X +
                                            ((double)z + dz) * (double)X * (double)X)];
                if (index < 0 || io < 0) continue;
                float *cm = &cb->metrics[(int64_t)index * 10];
                if (om64) {
                    const double *o = &om64[(int64_t)io * 10];
                    /* float32*float32 products, promoted to float64 on mixing */
                    double den = (double)CM(9) + o[9];
                    double mx = ((double)(CM(0) * CM(9)) + o[0] * o[9]) / den;
                    double my = ((double)(CM(1) * CM(9)) + o[1] * o[9]) / den;
                    double mz = ((double)(CM(2) * CM(9)) + o[2] * o[9]) / den;
                    double mean[3] = {mx, my, mz};
                    static const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
                    float nc[6];
                    for (int t = 0; t < 6; t++) {
                        int a = pa[t], b = pb[t];
                        double t1 = (double)(CM(9) * CM(3 + t));
                        double t2 = o[9] * o[3 + t];
                        double t3 = ((double)CM(9) * ((double)CM(a) - mean[a])) * ((double)CM(b) - mean[b]);
                        double t4 = (o[9] * (o[a] - mean[a])) * (o[b] - mean[b]);
                        double s = t1 + t2;
                        s = s + t3;
                        s = s + t4;
                        nc[t] = (float)(s / ((double)CM(9) + o[9]));
                    }
                    for (int t = 0; t < 6; t++) CM(3 + t) = nc[t];
                    CM(0) = (float)mx; CM(1) = (float)my; CM(2) = (float)mz;
                    CM(9) = (float)((double)CM(9) + o[9]);
                } else {
                    const float *o = &om32[(int64_t)io * 10];
                    /* all float32 */
                    float den = CM(9) + o[9];
                    float mx = (CM(0) * CM(9) + o[0] * o[9]) / den;
                    float my = (CM(1) * CM(9) + o[1] * o[9]) / den;
                    float mz = (CM(2) * CM(9) + o[2] * o[9]) / den;
                    float mean[3] = {mx, my, mz};
                    static const int pa[6] = {0, 0, 0, 1, 1, 2}, pb[6] = {0, 1, 2, 1, 2, 2};
                    float nc[6];
                    for (int t = 0; t < 6; t++) {
                        int a = pa[t], b = pb[t];
                        float t1 = CM(9) * CM(3 + t);
                        float t2 = o[9] * o[3 + t];
                        float u = CM(9) * (CM(a) - mean[a]);
                        float t3 = u * (CM(b) - mean[b]);
                        float w = o[9] * (o[a] - mean[a]);
                        float t4 = w * (o[b] - mean[b]);
                        float s = t1 + t2;
                        s = s + t3;
                        s = s + t4;
                        nc[t] = s / (CM(9) + o[9]);
                    }
                    for (int t = 0; t < 6; t++) CM(3 + t) = nc[t];
                    CM(0) = mx; CM(1) = my; CM(2) = mz;
                    CM(9) = CM(9) + o[9];
                }
                cb->hit[index] = cb->hit[index] + ohit[io];
                cb->total[index] = cb->total[index] + ototal[io];
                float a = cb->min_h[index], b = omin[io];
                cb->min_h[index] = (b < a) ? b : a;
            }
}
#undef CM

/* ------------------------------------------------------------------------ */
/* __calculate_eigenvalues (gvom.py:1423-1487)                                */
/* ------------------------------------------------------------------------ */
static void calculate_eigenvalues(float *ev, const float *met, int64_t C, int par) {
#pragma omp parallel for schedule(static) if (par)
    for (int64_t i = 0; i < C; i++) {
        const float *r = &met[i * 10];
        float xx = r[3], xy = r[4], xz = r[5], yy = r[6], yz = r[7], zz = r[8];
        float a = xy * xy, b = xz * xz, c = yz * yz;
        float p1 = a + b;
        p1 = p1 + c;
        float tr = xx + yy;
        tr = tr + zz;
        double q = (double)tr / 3.0;
        float *e = &ev[i * 3];
        if (p1 == 0) {
            float m12 = yy > zz ? yy : zz; /* max(yy, zz) */
            e[0] = xx > m12 ? xx : m12;
            float n12 = yy < zz ? yy : zz;
            e[2] = xx < n12 ? xx : n12;
            e[1] = (float)(3.0 * q - (double)e[0] - (double)e[2]);
        } else {
            double dxx = (double)xx - q, dyy = (double)yy - q, dzz = (double)zz - q;
            double p2 = dxx * dxx + dyy * dyy;
            p2 = p2 + dzz * dzz;
            p2 = p2 + 2.0 * (double)p1;
            double p = sqrt(p2 / 6.0);
            double B0 = ((double)xx - q) / p, B1 = (double)xy / p, B2 = (double)xz / p;
            double B3 = ((double)yy - q) / p, B4 = (double)yz / p, B5 = ((double)zz - q) / p;
            double rr = B0 * (B3 * B5 - B4 * B4) - B1 * (B1 * B5 - B4 * B2) + B2 * (B1 * B4 - B3 * B2);
            rr = rr / 2;
            double phi;
            if (rr <= -1) phi = M_PI / 3.0;
            else if (rr >= 1) phi = 0.0;
            else phi = acos(rr) / 3.0;
            e[0] = (float)(q + 2.0 * p * cos(phi));
            e[2] = (float)(q + 2.0 * p * cos(phi + (2.0 * M_PI / 3.0)));
            e[1] = (float)(3.0 * q - (double)e[0] - (double)e[2]);
        }
    }
}

/* ------------------------------------------------------------------------ */
/* 2-D maps (gvom.py:444-805)                                                 */
/* ------------------------------------------------------------------------ */
#define M2(a, x, y) ((a)[(x) * X + (y)])

static void make_height_maps(gvo_map *m, int par) {
    const int64_t X = m->X, Z = m->Z;
    const double *co = m->cur.origin;
    const double xr = m->p.xy_resolution, zr = m->p.z_resolution;
    const double rad = m->p.robot_radius;
#pragma omp parallel for schedule(static) if (par)
    for (int64_t x = 0; x < X; x++)
        for (int64_t y = 0; y < X; y++) {
            /* __make_height_map (gvom.py:560-576) */
            double h = -1000.0;
            double xp = ((co[0] + (double)x) * xr) - m->ego[0];
            double yp = ((co[1] + (double)y) * xr) - m->ego[1];
            double s = xp * xp;
            s = s + yp * yp;
            if (s <= rad * rad) h = m->ego[2] - m->p.ground_to_lidar_height;
            for (int64_t z = 0; z < Z; z++) {
                int32_t idx = m->cur.index[x + y * X + z * X * X];
                if (idx >= 0) {
                    h = (((double)m->cur.min_h[idx] + (double)z) + co[2]) * zr;
                    break;
                }
            }
            M2(m->height, x, y) = h;
            /* __make_inferred_height_map (gvom.py:579-590) */
            double ih = -1000.0;
            for (int64_t z = 0; z < Z; z++) {
                int32_t idx = m->cur.index[x + y * X + z * X * X];
                if (idx < -1) {
                    ih = ((double)z + co[2]) * zr;
                    break;
                }
            }
            M2(m->inferred, x, y) = ih;
        }
}

/* __calculate_slope (gvom.py:717-805) */
static void calculate_slope(gvo_map *m, int par) {
    const int64_t X = m->X;
    const double xr = m->p.xy_resolution;
    const double *hm = m->height;
#pragma omp parallel for schedule(static) if (par)
    for (int64_t x0 = 0; x0 < X; x0++)
        for (int64_t y0 = 0; y0 < X; y0++) {
            M2(m->rough, x0, y0) = -1.0;
            M2(m->slope_x, x0, y0) = 0.0;
            M2(m->slope_y, x0, y0) = 0.0;
            int64_t xl = x0 - 1 > 0 ? x0 - 1 : 0, xh = x0 + 2 < X ? x0 + 2 : X;
            int64_t yl = y0 - 1 > 0 ? y0 - 1 : 0, yh = y0 + 2 < X ? y0 + 2 : X;
            int n_good = 0;
            for (int64_t x = xl; x < xh; x++)
                for (int64_t y = yl; y < yh; y++)
                    if (M2(hm, x, y) > -1000) n_good++;
            if (n_good < 3) continue;
            double pts[3][9];
            int i = 0;
            double mean_x = 0.0, mean_y = 0.0, mean_z = 0.0;
            for (int64_t x = xl; x < xh; x++)
                for (int64_t y = yl; y < yh; y++)
                    if (M2(hm, x, y) > -1000) {
                        pts[0][i] = (double)x * xr;
                        pts[1][i] = (double)y * xr;
                        pts[2][i] = M2(hm, x, y);
                        mean_x += pts[0][i];
                        mean_y += pts[1][i];
                        mean_z += pts[2][i];
                        i++;
                    }
            mean_x /= (double)i;
            mean_y /= (double)i;
            mean_z /= (double)i;
            double xx = 0.0, xy = 0.0, xz = 0.0, yy = 0.0, yz = 0.0;
            for (int j = 0; j < n_good; j++) {
                xx += (pts[0][j] - mean_x) * (pts[0][j] - mean_x);
                xy += (pts[0][j] - mean_x) * (pts[1][j] - mean_y);
                xz += (pts[0][j] - mean_x) * (pts[2][j] - mean_z);
                yy += (pts[1][j] - mean_y) * (pts[1][j] - mean_y);
                yz += (pts[1][j] - mean_y) * (pts[2][j] - mean_z);
            }
            double det = xx * yy - xy * xy;
            if (det == 0.0) continue;
            double a0 = (yy * xz - xy * yz) / det;
            double a1 = (xx * yz - xy * xz) / det;
            double err = 0.0;
            double mm = a0 * a0 + a1 * a1;
            mm = mm + 1;
            mm = sqrt(mm);
            a0 /= mm;
            a1 /= mm;
            for (int j = 0; j < n_good; j++) {
                double e = (pts[2][j] - mean_z) - (a0 * (pts[0][j] - mean_x) + a1 * (pts[1][j] - mean_y));
                err += e * e;
            }
            err /= (double)n_good;
            if (err > 0) err = log(err);
            M2(m->rough, x0, y0) = err;
            M2(m->slope_x, x0, y0) = atan2(a0, 1.0 / mm);
            M2(m->slope_y, x0, y0) = atan2(a1, 1.0 / mm);
        }
}

/* __guess_height (gvom.py:592-714), including its loop-condition and y_nh bugs */
static void guess_height(gvo_map *m, int par) {
    const int64_t X = m->X;
    const double *hm = m->height, *im = m->inferred;
#pragma omp parallel for schedule(static) if (par)
    for (int64_t x0 = 0; x0 < X; x0++)
        for (int64_t y0 = 0; y0 < X; y0++) {
            M2(m->guess, x0, y0) = 0.0;
            if (M2(hm, x0, y0) > -1000) continue;
            if (M2(im, x0, y0) == -1000.0) continue;
            int xpd = 0, xnd = 0, ypd = 0, ynd = 0;
            int64_t xp = x0, xn = x0, yp = y0, yn = y0;
            double xph = -1000, xnh = -1000, yph = -1000, ynh = -1000;
            int64_t i = 0;
            while ((i < 15) && (!(xnd && xnd && ypd && ynd))) {
                xp += 1; xn -= 1; yp += 1; yn -= 1;
                i += 1;
                if (!xpd) {
                    if (xp < X) {
                        for (int64_t dy = -i; dy < i; dy++) {
                            if (y0 + dy >= X || y0 + dy < 0) continue;
                            if (M2(hm, xp, y0 + dy) > -1000) { xph = M2(hm, xp, y0 + dy); xpd = 1; break; }
                        }
                    } else xpd = 1;
                }
                if (!xnd) {
                    if (xn >= 0) {
                        for (int64_t dy = -i + 1; dy < i + 1; dy++) {
                            if (y0 + dy >= X || y0 + dy < 0) continue;
                            if (M2(hm, xn, y0 + dy) > -1000) { xnh = M2(hm, xn, y0 + dy); xnd = 1; break; }
                        }
                    } else xnd = 1;
                }
                if (!ypd) {
                    if (yp < X) {
                        for (int64_t dx = -i + 1; dx < i + 1; dx++) {
                            if (x0 + dx >= X || x0 + dx < 0) continue;
                            if (M2(hm, x0 + dx, yp) > -1000) { yph = M2(hm, x0 + dx, yp); ypd = 1; break; }
                        }
                    } else ypd = 1;
                }
                if (!ynd) {
                    if (yn >= 0) {
                        for (int64_t dx = -i; dx < i; dx++) {
                            if (x0 + dx >= X || x0 + dx < 0) continue;
                            if (M2(hm, x0 + dx, yn) > -1000) { ynh = M2(hm, x0 + dx, yn); ynd = 1; break; }
                        }
                    } else ynd = 1;
                }
            }
            double min_h = 1000.0, max_h = M2(im, x0, y0);
            /* Python min(a, b) returns a unless b < a; max(a, b) returns a unless b > a */
#define PMIN(a, b) ((b) < (a) ? (b) : (a))
#define PMAX(a, b) ((b) > (a) ? (b) : (a))
            if (xph > -1000) { min_h = PMIN(xph, min_h); max_h = PMAX(xph, max_h); }
            if (xnh > -1000) { min_h = PMIN(xnh, min_h); max_h = PMAX(xnh, max_h); }
            if (yph > -1000) { min_h = PMIN(yph, min_h); max_h = PMAX(yph, max_h); }
            if (xnh > -1000) { min_h = PMIN(ynh, min_h); max_h = PMAX(ynh, max_h); }
#undef PMIN
#undef PMAX
            double dh = max_h - min_h;
            if (dh > 0) M2(m->guess, x0, y0) = dh;
        }
}

static void obstacle_maps(gvo_map *m, int par) {
    const int64_t X = m->X, Z = m->Z;
    const double zr = m->p.z_resolution;
    const double *co = m->cur.origin;
#pragma omp parallel for schedule(static) if (par)
    for (int64_t x = 0; x < X; x++)
        for (int64_t y = 0; y < X; y++) {
            /* __make_positive_obstacle_map (gvom.py:515-555) */
            int32_t pv = 0;
            double sx = M2(m->slope_x, x, y), sy = M2(m->slope_y, x, y);
            double s2 = sx * sx;
            s2 = s2 + sy * sy;
            if (sqrt(s2) >= m->p.slope_obstacle_threshold) {
                pv = 100;
            } else {
                double h = M2(m->height, x, y);
                double min_obs = h + m->p.positive_obstacle_threshold;
                double max_obs = h + m->p.robot_height;
                int64_t zmin = (int64_t)floor((min_obs / zr) - co[2]) + 1;
                int64_t zmax = (int64_t)floor((max_obs / zr) - co[2]);
                if ((zmin >= 0 && zmin < Z) && (zmax >= 0 && zmax < Z)) {
                    double density = 0.0, nn = 0.0;
                    for (int64_t z = zmin; z < zmax + 1; z++) {
                        int32_t idx = m->cur.index[x + y * X + z * X * X];
                        if (idx >= 0 && m->cur.hit[idx] > 10) {
                            nn += (double)m->cur.total[idx];
                            density += (double)m->cur.hit[idx];
                        }
                    }
                    if (nn > 0.0) density /= nn;
                    pv = (int32_t)(density * 100);
                }
            }
            M2(m->pos, x, y) = pv;
            /* __make_negative_obstacle_map (gvom.py:505-512) */
            M2(m->neg, x, y) = (M2(m->guess, x, y) > m->p.negative_obstacle_threshold) ? 100 : 0;
            /* __make_visability_map (gvom.py:444-452) */
            M2(m->vis, x, y) = (M2(m->height, x, y) > -1000) ? 1 : 0;
        }
}

/* ------------------------------------------------------------------------ */
/* combine_maps (gvom.py:222-393)                                             */
/* ------------------------------------------------------------------------ */
int gvo_combine(gvo_map *m, double origin_out[3], int32_t *pos, int32_t *neg, double *rough, int32_t *vis) {
    if (!m) return GVO_BAD_ARG;
    if (!m->slots[m->last_buffer_index].valid) return GVO_NO_DATA;
    const int par = m->threads > 1;
#ifdef _OPENMP
    if (par) omp_set_num_threads(m->threads);
#endif
    const int64_t X = m->X, V = m->V;
    gvo_comb nc;
    memset(&nc, 0, sizeof(nc));
    memcpy(nc.origin, m->slots[m->last_buffer_index].origin, sizeof(nc.origin));
    nc.index = (int32_t *)xcalloc((size_t)V, 4);
    for (int64_t v = 0; v < V; v++) nc.index[v] = -1;
    int64_t counter = 0;
    for (int i = 0; i < m->p.buffer_size; i++) {
        gvo_slot *s = &m->slots[i];
        if (!s->valid) continue;
        combine_indices(m, nc.index, nc.origin, s->index, s->origin, &counter, 0, par);
    }
    if (m->have_last) combine_indices(m, nc.index, nc.origin, m->last.index, m->last.origin, &counter, 1, par);
    nc.C = counter;
    nc.hit = (int32_t *)xcalloc((size_t)nc.C, 4);
    nc.total = (int32_t *)xcalloc((size_t)nc.C, 4);
    nc.min_h = (float *)xcalloc((size_t)nc.C, 4);
    for (int64_t c = 0; c < nc.C; c++) nc.min_h[c] = 1.0f;
    nc.metrics = (float *)xcalloc((size_t)nc.C * 10, 4);
    for (int i = 0; i < m->p.buffer_size; i++) {
        gvo_slot *s = &m->slots[i];
        if (!s->valid) continue;
        combine_metrics(m, &nc, s->index, s->origin, s->metrics, NULL, s->hit, s->total, s->min_h, par);
    }
    if (m->have_last)
        combine_metrics(m, &nc, m->last.index, m->last.origin, NULL, m->last.metrics, m->last.hit,
                        m->last.total, m->last.min_h, par);
    nc.valid = 1;
    /* last_combined = combined (gvom.py:302-308); keep `cur` as the live map */
    comb_free(&m->last);
    m->last = nc;
    m->have_last = 1;
    /* cur aliases last (the reference's combined_* and last_combined_* are the same objects) */
    m->cur = m->last;
    free(m->eigen);
    m->eigen = (float *)xcalloc((size_t)nc.C * 3, 4);
    calculate_eigenvalues(m->eigen, nc.metrics, nc.C, par);
    make_height_maps(m, par);
    calculate_slope(m, par);
    guess_height(m, par);
    obstacle_maps(m, par);
    m->have_maps = 1;
    if (origin_out) {
        origin_out[0] = nc.origin[0] * m->p.xy_resolution;
        origin_out[1] = nc.origin[1] * m->p.xy_resolution;
        origin_out[2] = nc.origin[2] * m->p.z_resolution;
    }
    size_t X2 = (size_t)(X * X);
    if (pos) memcpy(pos, m->pos, X2 * 4);
    if (neg) memcpy(neg, m->neg, X2 * 4);
    if (rough) memcpy(rough, m->rough, X2 * 8);
    if (vis) memcpy(vis, m->vis, X2 * 4);
    return GVO_OK;
}

/* ------------------------------------------------------------------------ */
/* debug exporters (gvom.py:395-503)                                          */
/* ------------------------------------------------------------------------ */
int64_t gvo_combined_count(const gvo_map *m) { return m->have_last ? m->cur.C : -1; }

/* __make_voxel_pointcloud (gvom.py:481-503): row = compact index */
int gvo_debug_voxels(const gvo_map *m, float *out) {
    if (!m->have_last) return GVO_NO_DATA;
    const int64_t X = m->X, Z = m->Z;
    const double *co = m->cur.origin;
    for (int64_t z = 0; z < Z; z++)
        for (int64_t y = 0; y < X; y++)
            for (int64_t x = 0; x < X; x++) {
                int32_t idx = m->cur.index[x + y * X + z * X * X];
                if (idx < 0) continue;
                float *r = &out[(int64_t)idx * 8];
                r[0] = (float)(((double)x + co[0]) * m->p.xy_resolution);
                r[1] = (float)(((double)y + co[1]) * m->p.xy_resolution);
                r[2] = (float)(((double)z + co[2]) * m->p.z_resolution);
                r[3] = (float)((double)m->cur.hit[idx] / (double)m->cur.total[idx]);
                r[4] = (float)m->cur.hit[idx];
                const float *e = &m->eigen[(int64_t)idx * 3];
                float d1 = e[0] - e[1];
                float d2 = e[1] - e[2];
                r[5] = d1;
                r[6] = d2;
                r[7] = e[2];
            }
    return GVO_OK;
}

/* __make_height_map_pointcloud (gvom.py:455-468): row = x + y*X */
int gvo_debug_height_map(const gvo_map *m, float *out) {
    if (!m->have_maps) return GVO_NO_DATA;
    const int64_t X = m->X;
    const double *co = m->cur.origin;
    for (int64_t x = 0; x < X; x++)
        for (int64_t y = 0; y < X; y++) {
            float *r = &out[(x + y * X) * 7];
            double sx = M2(m->slope_x, x, y), sy = M2(m->slope_y, x, y);
            r[0] = (float)(((double)x + co[0]) * m->p.xy_resolution);
            r[1] = (float)(((double)y + co[1]) * m->p.xy_resolution);
            r[2] = (float)(M2(m->height, x, y) - m->p.z_resolution);
            r[3] = (float)M2(m->rough, x, y);
            r[4] = (float)sx;
            r[5] = (float)sy;
            double s = sx * sx;
            s = s + sy * sy;
            r[6] = (float)sqrt(s);
        }
    return GVO_OK;
}

/* __make_infered_height_map_pointcloud (gvom.py:470-479); the reference passes
 * the guessed height delta as its "height map" (gvom.py:439-440) */
int gvo_debug_inferred_height_map(const gvo_map *m, float *out) {
    if (!m->have_maps) return GVO_NO_DATA;
    const int64_t X = m->X;
    const double *co = m->cur.origin;
    for (int64_t x = 0; x < X; x++)
        for (int64_t y = 0; y < X; y++) {
            float *r = &out[(x + y * X) * 3];
            r[0] = (float)(((double)x + co[0]) * m->p.xy_resolution);
            r[1] = (float)(((double)y + co[1]) * m->p.xy_resolution);
            r[2] = (float)(M2(m->guess, x, y) - m->p.z_resolution);
        }
    return GVO_OK;
}

/* ------------------------------------------------------------------------ */
/* state accessors for parity checks                                          */
/* ------------------------------------------------------------------------ */
int gvo_get_combined(const gvo_map *m, int32_t *index, int32_t *hit, int32_t *total, float *min_h,
                     float *metrics, float *eigen, double origin[3]) {
    if (!m->have_last) return GVO_NO_DATA;
    const gvo_comb *c = &m->cur;
    if (index) memcpy(index, c->index, (size_t)m->V * 4);
    if (hit) memcpy(hit, c->hit, (size_t)c->C * 4);
    if (total) memcpy(total, c->total, (size_t)c->C * 4);
    if (min_h) memcpy(min_h, c->min_h, (size_t)c->C * 4);
    if (metrics) memcpy(metrics, c->metrics, (size_t)c->C * 40);
    if (eigen) memcpy(eigen, m->eigen, (size_t)c->C * 12);
    if (origin) memcpy(origin, c->origin, 24);
    return GVO_OK;
}

int gvo_get_maps(const gvo_map *m, double *height, double *inferred, double *slope_x, double *slope_y,
                 double *rough, double *guess) {
    if (!m->have_maps) return GVO_NO_DATA;
    size_t X2 = (size_t)(m->X * m->X);
    if (height) memcpy(height, m->height, X2 * 8);
    if (inferred) memcpy(inferred, m->inferred, X2 * 8);
    if (slope_x) memcpy(slope_x, m->slope_x, X2 * 8);
    if (slope_y) memcpy(slope_y, m->slope_y, X2 * 8);
    if (rough) memcpy(rough, m->rough, X2 * 8);
    if (guess) memcpy(guess, m->guess, X2 * 8);
    return GVO_OK;
}

int64_t gvo_slot_count(const gvo_map *m, int slot) {
    if (slot < 0 || slot >= m->p.buffer_size || !m->slots[slot].valid) return -1;
    return m->slots[slot].C;
}

int gvo_get_slot(const gvo_map *m, int slot, int32_t *index, int32_t *hit, int32_t *total, float *min_h,
                 double *metrics, double origin[3]) {
    if (slot < 0 || slot >= m->p.buffer_size || !m->slots[slot].valid) return GVO_NO_DATA;
    const gvo_slot *s = &m->slots[slot];
    if (index) memcpy(index, s->index, (size_t)m->V * 4);
    if (hit) memcpy(hit, s->hit, (size_t)s->C * 4);
    if (total) memcpy(total, s->total, (size_t)s->C * 4);
    if (min_h) memcpy(min_h, s->min_h, (size_t)s->C * 4);
    if (metrics) memcpy(metrics, s->metrics, (size_t)s->C * 80);
    if (origin) memcpy(origin, s->origin, 24);
    return GVO_OK;
}

void gvo_ring_state(const gvo_map *m, int64_t *buffer_index, int64_t *last_buffer_index) {
    *buffer_index = m->buffer_index;
    *last_buffer_index = m->last_buffer_index;
}

void gvo_last_process_stats(const gvo_map *m, int64_t *ray_steps, int64_t *hits, int64_t *valid_points) {
    *ray_steps = m->last_ray_steps;
    *hits = m->last_hits;
    *valid_points = m->last_valid_points;
}

/* ------------------------------------------------------------------------- */
/* 2-D image kernels that no reference caller launches                        */
/* ------------------------------------------------------------------------- */

/* __expand_binary (scripts/gvom.py:807-831), thread (x, y) in turn. */
void gvo_expand_binary(const int32_t *in, int32_t *out, int X, double r) {
    const long long rint_ = (long long)floor(r);
    for (int x = 0; x < X; x++)
        for (int y = 0; y < X; y++) {
            int v = 0;
            for (long long i = -rint_; i < rint_ + 1 && !v; i++) {
                const long long dy = (long long)floor(sqrt(r * r - (double)(i * i)));
                if (x + i < 0 || x + i >= X) continue;
                for (long long j = -dy; j < dy + 1; j++) {
                    if (y + j < 0 || y + j >= X) continue;
                    if (in[(x + i) * (long long)X + (y + j)] == 1) {
                        v = 1;
                        break;
                    }
                }
            }
            out[(long long)x * X + y] = v;
        }
}

/* __lowpass_binary (scripts/gvom.py:833-861). */
void gvo_lowpass_binary(const int32_t *in, int32_t *out, int X, int filter_size, double filter_fraction) {
    for (int x = 0; x < X; x++)
        for (int y = 0; y < X; y++) {
            if (in[(long long)x * X + y] == 0) {
                out[(long long)x * X + y] = 0;
                continue;
            }
            double tmp_val = 0.0, tmp_count = 0.0;
            for (int i = -filter_size; i < filter_size + 1; i++) {
                if (x + i < 0 || x + i >= X) continue;
                for (int j = -filter_size; j < filter_size + 1; j++) {
                    if (y + j < 0 || y + j >= X) continue;
                    tmp_val += (double)in[(long long)(x + i) * X + (y + j)] * 1.0;
                    tmp_count += 1.0;
                }
            }
            out[(long long)x * X + y] = (tmp_val / tmp_count) >= filter_fraction ? 1 : 0;
        }
}

/* __convolve (scripts/gvom.py:863-885) as written, with the radius an
 * integer: every term reads input[x + r, y + r] and the in-range tests are
 * on x + r and y + r.  (The reference's float radius cannot be passed to
 * range(), so its kernel itself never runs.) */
void gvo_convolve(const double *in, double *out, const double *kernel, int X, int kernel_size) {
    const int r = (kernel_size - 1) / 2;
    for (int x = 0; x < X; x++)
        for (int y = 0; y < X; y++) {
            double tmp_val = 0.0;
            for (int i = -r; i < r + 1; i++) {
                const int x2 = i + r;
                if (x + r < 0 || x + r >= X) continue;
                for (int j = -r; j < r + 1; j++) {
                    const int y2 = j + r;
                    if (y + r < 0 || y + r >= X) continue;
                    tmp_val += in[(long long)(x + r) * X + (y + r)] * kernel[x2 * kernel_size + y2];
                }
            }
            out[(long long)x * X + y] = tmp_val;
        }
}
