/*
 * synth.c — seeded procedural maps, trajectories and ray-cast lidar scans.
 *
 * Stands in for the reference's rosbag + PCD map (absent from the reference tree) with the
 * shapes of the benchmark workloads: a ground plane z = 0 with N(0, 0.03 m) noise,
 * axis-aligned box buildings sampled on their walls, vertical poles, anisotropic Gaussian
 * tree blobs; scans from a rotating multi-ring lidar ray-cast against the same analytic
 * scene with N(0, sigma) range noise, then voxel-downsampled with the centroid rule of
 * src/ndt_cuda/src/test_utils.rs:76-110 (floor(p * 1/leaf), FP64 sums, f32 centroid).
 * All randomness is SplitMix64 keyed by (seed, stream, index), so outputs do not depend on
 * the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_D 3.14159265358979323846

static uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

typedef struct {
    uint64_t s;
} rng_t;

static rng_t rng_make(uint64_t seed, uint64_t stream, uint64_t idx) {
    rng_t r;
    r.s = mix64(seed ^ mix64(stream * 0x632BE59BD9B4E019ull ^ mix64(idx)));
    return r;
}
static double rng_u(rng_t* r) { /* [0,1) */
    r->s += 0x9E3779B97F4A7C15ull;
    uint64_t z = r->s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}
static double rng_range(rng_t* r, double a, double b) { return a + (b - a) * rng_u(r); }
static double rng_n(rng_t* r) {
    double u1 = rng_u(r), u2 = rng_u(r);
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * PI_D * u2);
}

typedef struct {
    double x0, y0, x1, y1, h;
} sbox;
typedef struct {
    double x, y, r, h;
} spole;
typedef struct {
    double cx, cy, cz, sx, sy, sz;
} sblob;

typedef struct {
    double extent; /* square [-extent/2, extent/2]^2 */
    int nb, np, nt;
    sbox* boxes;
    spole* poles;
    sblob* blobs;
} scene_t;

/* keep-out test against a list of clear points (trajectory samples or the sensor) */
static int near_clear(const double* clear, int nclear, double x, double y, double r) {
    for (int i = 0; i < nclear; ++i) {
        double dx = clear[2 * i] - x, dy = clear[2 * i + 1] - y;
        if (dx * dx + dy * dy < r * r) return 1;
    }
    return 0;
}
static int box_near_clear(const double* clear, int nclear, const sbox* b, double margin) {
    for (int i = 0; i < nclear; ++i) {
        double x = clear[2 * i], y = clear[2 * i + 1];
        if (x > b->x0 - margin && x < b->x1 + margin && y > b->y0 - margin && y < b->y1 + margin)
            return 1;
    }
    return 0;
}

void* synth_scene_create(uint64_t seed, double extent, int n_boxes, int n_poles, int n_trees,
                         double box_side_min, double box_side_max, double box_h_min,
                         double box_h_max, const double* clear_xy, int n_clear) {
    scene_t* s = (scene_t*)calloc(1, sizeof(scene_t));
    s->extent = extent;
    s->boxes = (sbox*)calloc((size_t)(n_boxes > 0 ? n_boxes : 1), sizeof(sbox));
    s->poles = (spole*)calloc((size_t)(n_poles > 0 ? n_poles : 1), sizeof(spole));
    s->blobs = (sblob*)calloc((size_t)(n_trees > 0 ? n_trees : 1), sizeof(sblob));
    double h = extent * 0.5;
    rng_t r = rng_make(seed, 1, 0);
    for (int i = 0, tries = 0; i < n_boxes && tries < n_boxes * 200; ++tries) {
        double w = rng_range(&r, box_side_min, box_side_max);
        double d = rng_range(&r, box_side_min, box_side_max);
        double cx = rng_range(&r, -h + w * 0.5, h - w * 0.5);
        double cy = rng_range(&r, -h + d * 0.5, h - d * 0.5);
        sbox b = {cx - w * 0.5, cy - d * 0.5, cx + w * 0.5, cy + d * 0.5,
                  rng_range(&r, box_h_min, box_h_max)};
        if (box_near_clear(clear_xy, n_clear, &b, 6.0)) continue;
        s->boxes[i++] = b;
        s->nb = i;
    }
    r = rng_make(seed, 2, 0);
    for (int i = 0, tries = 0; i < n_poles && tries < n_poles * 200; ++tries) {
        double x = rng_range(&r, -h + 1, h - 1), y = rng_range(&r, -h + 1, h - 1);
        if (near_clear(clear_xy, n_clear, x, y, 3.0)) continue;
        int inside = 0;
        for (int b = 0; b < s->nb; ++b)
            if (x > s->boxes[b].x0 - 0.5 && x < s->boxes[b].x1 + 0.5 &&
                y > s->boxes[b].y0 - 0.5 && y < s->boxes[b].y1 + 0.5)
                inside = 1;
        if (inside) continue;
        spole p = {x, y, 0.15, 6.0};
        s->poles[i++] = p;
        s->np = i;
    }
    r = rng_make(seed, 3, 0);
    for (int i = 0, tries = 0; i < n_trees && tries < n_trees * 200; ++tries) {
        double x = rng_range(&r, -h + 3, h - 3), y = rng_range(&r, -h + 3, h - 3);
        if (near_clear(clear_xy, n_clear, x, y, 6.0)) continue;
        sblob t;
        t.cx = x;
        t.cy = y;
        t.sx = rng_range(&r, 1.0, 3.0);
        t.sy = rng_range(&r, 1.0, 3.0);
        t.sz = rng_range(&r, 1.0, 3.0);
        t.cz = 2.0 + 1.5 * t.sz;
        s->blobs[i++] = t;
        s->nt = i;
    }
    return s;
}

void synth_scene_free(void* p) {
    scene_t* s = (scene_t*)p;
    if (!s) return;
    free(s->boxes);
    free(s->poles);
    free(s->blobs);
    free(s);
}

void synth_scene_counts(const void* p, int* out3) {
    const scene_t* s = (const scene_t*)p;
    out3[0] = s->nb;
    out3[1] = s->np;
    out3[2] = s->nt;
}

/* Map points: surfaces sampled with a uniform areal density (ground, box walls, pole
 * mantles, and tree blobs weighted by their 1-sigma ellipsoid area). */
void synth_map_points(const void* p, uint64_t seed, size_t n, float* out) {
    const scene_t* s = (const scene_t*)p;
    int nobj = 1 + s->nb + s->np + s->nt;
    double* area = (double*)malloc(sizeof(double) * (size_t)nobj);
    double* cum = (double*)malloc(sizeof(double) * (size_t)nobj);
    area[0] = s->extent * s->extent;
    for (int b = 0; b < s->nb; ++b) {
        const sbox* x = &s->boxes[b];
        area[1 + b] = 2.0 * ((x->x1 - x->x0) + (x->y1 - x->y0)) * x->h;
    }
    for (int q = 0; q < s->np; ++q) area[1 + s->nb + q] = 2.0 * PI_D * s->poles[q].r * s->poles[q].h;
    for (int t = 0; t < s->nt; ++t) {
        const sblob* b = &s->blobs[t];
        area[1 + s->nb + s->np + t] = 4.0 * PI_D * (b->sx * b->sy + b->sy * b->sz + b->sx * b->sz) / 3.0;
    }
    double tot = 0.0;
    for (int i = 0; i < nobj; ++i) {
        tot += area[i];
        cum[i] = tot;
    }
    double h = s->extent * 0.5;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (long i = 0; i < (long)n; ++i) {
        rng_t r = rng_make(seed, 10, (uint64_t)i);
        double u = rng_u(&r) * tot;
        int lo = 0, hi = nobj - 1;
        while (lo < hi) {
            int mid = (lo + hi) / 2;
            if (cum[mid] > u)
                hi = mid;
            else
                lo = mid + 1;
        }
        double x, y, z;
        if (lo == 0) {
            x = rng_range(&r, -h, h);
            y = rng_range(&r, -h, h);
            z = 0.03 * rng_n(&r);
        } else if (lo <= s->nb) {
            const sbox* b = &s->boxes[lo - 1];
            double w = b->x1 - b->x0, d = b->y1 - b->y0;
            double t = rng_u(&r) * 2.0 * (w + d);
            if (t < w) {
                x = b->x0 + t;
                y = b->y0;
            } else if (t < w + d) {
                x = b->x1;
                y = b->y0 + (t - w);
            } else if (t < 2 * w + d) {
                x = b->x1 - (t - w - d);
                y = b->y1;
            } else {
                x = b->x0;
                y = b->y1 - (t - 2 * w - d);
            }
            z = rng_u(&r) * b->h;
        } else if (lo <= s->nb + s->np) {
            const spole* q = &s->poles[lo - 1 - s->nb];
            double a = rng_u(&r) * 2.0 * PI_D;
            x = q->x + q->r * cos(a);
            y = q->y + q->r * sin(a);
            z = rng_u(&r) * q->h;
        } else {
            const sblob* b = &s->blobs[lo - 1 - s->nb - s->np];
            x = b->cx + b->sx * rng_n(&r);
            y = b->cy + b->sy * rng_n(&r);
            z = b->cz + b->sz * rng_n(&r);
        }
        out[3 * i] = (float)x;
        out[3 * i + 1] = (float)y;
        out[3 * i + 2] = (float)z;
    }
    free(area);
    free(cum);
}

/* ---- ray casting ------------------------------------------------------------------ */
static double hit_box(const sbox* b, const double* o, const double* d) {
    double t0 = -1e300, t1 = 1e300;
    double lo[3] = {b->x0, b->y0, 0.0}, hi[3] = {b->x1, b->y1, b->h};
    for (int a = 0; a < 3; ++a) {
        if (fabs(d[a]) < 1e-12) {
            if (o[a] < lo[a] || o[a] > hi[a]) return -1.0;
        } else {
            double ta = (lo[a] - o[a]) / d[a], tb = (hi[a] - o[a]) / d[a];
            if (ta > tb) {
                double t = ta;
                ta = tb;
                tb = t;
            }
            if (ta > t0) t0 = ta;
            if (tb < t1) t1 = tb;
        }
    }
    if (t0 > t1) return -1.0;
    if (t0 > 1e-6) return t0;
    if (t1 > 1e-6) return t1;
    return -1.0;
}
static double hit_cyl(const spole* q, const double* o, const double* d) {
    double ox = o[0] - q->x, oy = o[1] - q->y;
    double a = d[0] * d[0] + d[1] * d[1];
    if (a < 1e-12) return -1.0;
    double b = 2.0 * (ox * d[0] + oy * d[1]), c = ox * ox + oy * oy - q->r * q->r;
    double disc = b * b - 4 * a * c;
    if (disc < 0) return -1.0;
    double sq = sqrt(disc);
    double t = (-b - sq) / (2 * a);
    if (t <= 1e-6) t = (-b + sq) / (2 * a);
    if (t <= 1e-6) return -1.0;
    double z = o[2] + t * d[2];
    return (z >= 0.0 && z <= q->h) ? t : -1.0;
}
static double hit_ell(const sblob* e, const double* o, const double* d) {
    double ox = (o[0] - e->cx) / e->sx, oy = (o[1] - e->cy) / e->sy, oz = (o[2] - e->cz) / e->sz;
    double dx = d[0] / e->sx, dy = d[1] / e->sy, dz = d[2] / e->sz;
    double a = dx * dx + dy * dy + dz * dz, b = 2 * (ox * dx + oy * dy + oz * dz),
           c = ox * ox + oy * oy + oz * oz - 1.0;
    double disc = b * b - 4 * a * c;
    if (disc < 0) return -1.0;
    double sq = sqrt(disc), t = (-b - sq) / (2 * a);
    if (t <= 1e-6) t = (-b + sq) / (2 * a);
    return t > 1e-6 ? t : -1.0;
}

/* azimuth interval [a0, a1] (radians, a0 may exceed a1 after wrapping to [-pi, pi]) */
static void az_interval(double sx, double sy, double cx, double cy, double rad, double* a0,
                        double* a1, int* all) {
    double dx = cx - sx, dy = cy - sy, dist = sqrt(dx * dx + dy * dy);
    *all = 0;
    if (dist <= rad * 1.01) {
        *all = 1;
        return;
    }
    double c = atan2(dy, dx), w = asin(rad / dist) + 1e-3;
    *a0 = c - w;
    *a1 = c + w;
}
static int az_in(double a, double a0, double a1) {
    /* a, a0, a1 unwrapped; test a modulo 2pi in [a0, a1] */
    double t = a - a0;
    t -= floor(t / (2 * PI_D)) * 2 * PI_D;
    return t <= (a1 - a0);
}

typedef struct {
    int64_t key;
    double sx, sy, sz;
    int cnt;
} vacc_t;
static int cmp_key(const void* a, const void* b) {
    int64_t ka = ((const vacc_t*)a)->key, kb = ((const vacc_t*)b)->key;
    return ka < kb ? -1 : (ka > kb);
}

/* pose = [x, y, z, yaw] of the sensor in the map frame. Returns the number of scan points
 * (sensor frame, downsampled with `leaf` if > 0) written to out (capacity `cap`). */
/* Ring elevations: `dense` rings spread uniformly over [band_lo, band_hi] (degrees) and the
 * remaining rings uniformly over the rest of [vfov_lo, vfov_hi], the layout of 128-ring
 * units whose rings crowd around the horizon. dense = 0 gives uniform spacing. */
static double ring_elev(int ir, int rings, double lo, double hi, int dense, double blo,
                        double bhi) {
    if (rings <= 1) return lo;
    if (dense <= 0 || dense >= rings) return lo + (hi - lo) * ir / (rings - 1);
    int sparse = rings - dense;
    double below = blo - lo, above = hi - bhi;
    int nb = (int)floor(sparse * below / (below + above) + 0.5);
    int na = sparse - nb;
    if (ir < nb) return lo + below * ir / (nb > 0 ? nb : 1);
    ir -= nb;
    if (ir < dense) return blo + (bhi - blo) * ir / (dense > 1 ? dense - 1 : 1);
    ir -= dense;
    return bhi + above * (ir + 1) / (na > 0 ? na : 1);
}

size_t synth_scan(const void* p, const double* pose, int rings, double vfov_lo_deg,
                  double vfov_hi_deg, int dense, double band_lo_deg, double band_hi_deg,
                  double az_step_deg, double max_range, double range_sigma,
                  double leaf, uint64_t seed, float* out, size_t cap) {
    const scene_t* s = (const scene_t*)p;
    int naz = (int)floor(360.0 / az_step_deg + 0.5);
    double sx = pose[0], sy = pose[1], sz = pose[2], yaw = pose[3];
    double cyw = cos(yaw), syw = sin(yaw);
    int nobj = s->nb + s->np + s->nt;
    /* candidate objects within range */
    int* cand = (int*)malloc(sizeof(int) * (size_t)(nobj > 0 ? nobj : 1));
    double* ia0 = (double*)malloc(sizeof(double) * (size_t)(nobj > 0 ? nobj : 1));
    double* ia1 = (double*)malloc(sizeof(double) * (size_t)(nobj > 0 ? nobj : 1));
    int* iall = (int*)malloc(sizeof(int) * (size_t)(nobj > 0 ? nobj : 1));
    int nc = 0;
    for (int i = 0; i < nobj; ++i) {
        double cx, cy, rad;
        if (i < s->nb) {
            const sbox* b = &s->boxes[i];
            cx = 0.5 * (b->x0 + b->x1);
            cy = 0.5 * (b->y0 + b->y1);
            rad = 0.5 * sqrt((b->x1 - b->x0) * (b->x1 - b->x0) + (b->y1 - b->y0) * (b->y1 - b->y0));
        } else if (i < s->nb + s->np) {
            const spole* q = &s->poles[i - s->nb];
            cx = q->x;
            cy = q->y;
            rad = q->r;
        } else {
            const sblob* e = &s->blobs[i - s->nb - s->np];
            cx = e->cx;
            cy = e->cy;
            rad = e->sx > e->sy ? e->sx : e->sy;
        }
        double dx = cx - sx, dy = cy - sy;
        if (sqrt(dx * dx + dy * dy) - rad > max_range) continue;
        /* intervals are in the sensor frame: subtract yaw */
        double a0 = 0, a1 = 0;
        int all = 0;
        az_interval(sx, sy, cx, cy, rad, &a0, &a1, &all);
        cand[nc] = i;
        ia0[nc] = a0 - yaw;
        ia1[nc] = a1 - yaw;
        iall[nc] = all;
        nc++;
    }
    size_t nray = (size_t)naz * (size_t)rings;
    float* raw = (float*)malloc(sizeof(float) * 3 * nray);
    unsigned char* ok = (unsigned char*)calloc(nray, 1);
    double h = s->extent * 0.5;
#ifdef _OPENMP
#pragma omp parallel
#endif
    {
        int* col = (int*)malloc(sizeof(int) * (size_t)(nc > 0 ? nc : 1));
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int ia = 0; ia < naz; ++ia) {
            double az = -PI_D + (ia + 0.5) * (2.0 * PI_D / naz);
            int ncol = 0;
            for (int k = 0; k < nc; ++k)
                if (iall[k] || az_in(az, ia0[k], ia1[k])) col[ncol++] = cand[k];
            double caz = cos(az), saz = sin(az);
            for (int ir = 0; ir < rings; ++ir) {
                double el = ring_elev(ir, rings, vfov_lo_deg, vfov_hi_deg, dense, band_lo_deg,
                                      band_hi_deg) * (PI_D / 180.0);
                double ds[3] = {cos(el) * caz, cos(el) * saz, sin(el)};
                double dw[3] = {cyw * ds[0] - syw * ds[1], syw * ds[0] + cyw * ds[1], ds[2]};
                double o[3] = {sx, sy, sz};
                double best = max_range;
                int hit = 0;
                if (dw[2] < -1e-9) {
                    double t = -o[2] / dw[2];
                    if (t < best) {
                        double gx = o[0] + t * dw[0], gy = o[1] + t * dw[1];
                        if (gx >= -h && gx <= h && gy >= -h && gy <= h) {
                            best = t;
                            hit = 1;
                        }
                    }
                }
                for (int k = 0; k < ncol; ++k) {
                    int i = col[k];
                    double t;
                    if (i < s->nb)
                        t = hit_box(&s->boxes[i], o, dw);
                    else if (i < s->nb + s->np)
                        t = hit_cyl(&s->poles[i - s->nb], o, dw);
                    else
                        t = hit_ell(&s->blobs[i - s->nb - s->np], o, dw);
                    if (t > 0 && t < best) {
                        best = t;
                        hit = 1;
                    }
                }
                size_t ri = (size_t)ia * rings + ir;
                if (hit) {
                    rng_t r = rng_make(seed, 20, ri);
                    double t = best + range_sigma * rng_n(&r);
                    raw[3 * ri] = (float)(t * ds[0]);
                    raw[3 * ri + 1] = (float)(t * ds[1]);
                    raw[3 * ri + 2] = (float)(t * ds[2]);
                    ok[ri] = 1;
                }
            }
        }
        free(col);
    }
    size_t m = 0;
    if (leaf <= 0.0) {
        for (size_t ri = 0; ri < nray && m < cap; ++ri)
            if (ok[ri]) {
                memcpy(out + 3 * m, raw + 3 * ri, 3 * sizeof(float));
                m++;
            }
    } else {
        size_t nh = 0;
        for (size_t ri = 0; ri < nray; ++ri) nh += ok[ri];
        vacc_t* acc = (vacc_t*)malloc(sizeof(vacc_t) * (nh ? nh : 1));
        float inv = (float)(1.0 / leaf);
        size_t k = 0;
        for (size_t ri = 0; ri < nray; ++ri) {
            if (!ok[ri]) continue;
            const float* q = raw + 3 * ri;
            int32_t vx = (int32_t)floorf(q[0] * inv), vy = (int32_t)floorf(q[1] * inv),
                    vz = (int32_t)floorf(q[2] * inv);
            acc[k].key = ((int64_t)(vx + (1 << 20)) << 42) | ((int64_t)(vy + (1 << 20)) << 21) |
                         (int64_t)(vz + (1 << 20));
            acc[k].sx = q[0];
            acc[k].sy = q[1];
            acc[k].sz = q[2];
            acc[k].cnt = 1;
            k++;
        }
        qsort(acc, k, sizeof(vacc_t), cmp_key);
        size_t i = 0;
        while (i < k && m < cap) {
            size_t j = i + 1;
            double ax = acc[i].sx, ay = acc[i].sy, az2 = acc[i].sz;
            while (j < k && acc[j].key == acc[i].key) {
                ax += acc[j].sx;
                ay += acc[j].sy;
                az2 += acc[j].sz;
                j++;
            }
            double nn = (double)(j - i);
            out[3 * m] = (float)(ax / nn);
            out[3 * m + 1] = (float)(ay / nn);
            out[3 * m + 2] = (float)(az2 / nn);
            m++;
            i = j;
        }
        free(acc);
    }
    free(raw);
    free(ok);
    free(cand);
    free(ia0);
    free(ia1);
    free(iall);
    return m;
}

/* Seeded closed-loop Catmull-Rom (cubic) spline trajectory sampled at constant speed.
 * out: n poses [x, y, z, yaw]; waypoints stay inside `extent - margin`. */
void synth_trajectory(uint64_t seed, double extent, double margin, int n, double spacing,
                      double height, double* out) {
    int nw = 12;
    double wx[12], wy[12];
    rng_t r = rng_make(seed, 30, 0);
    double h = extent * 0.5 - margin;
    for (int i = 0; i < nw; ++i) {
        double a = 2.0 * PI_D * i / nw + rng_range(&r, -0.2, 0.2);
        double rad = h * rng_range(&r, 0.45, 0.95);
        wx[i] = rad * cos(a);
        wy[i] = rad * sin(a);
    }
    /* dense sampling of the spline */
    int per = 400, nd = nw * per;
    double* px = (double*)malloc(sizeof(double) * (size_t)(nd + 1));
    double* py = (double*)malloc(sizeof(double) * (size_t)(nd + 1));
    double* sl = (double*)malloc(sizeof(double) * (size_t)(nd + 1));
    for (int k = 0; k <= nd; ++k) {
        int seg = (k / per) % nw;
        double t = (double)(k % per) / per;
        if (k == nd) {
            seg = 0;
            t = 0.0;
        }
        int i0 = (seg + nw - 1) % nw, i1 = seg, i2 = (seg + 1) % nw, i3 = (seg + 2) % nw;
        double t2 = t * t, t3 = t2 * t;
        double b0 = -0.5 * t3 + t2 - 0.5 * t, b1 = 1.5 * t3 - 2.5 * t2 + 1.0,
               b2 = -1.5 * t3 + 2.0 * t2 + 0.5 * t, b3 = 0.5 * t3 - 0.5 * t2;
        px[k] = b0 * wx[i0] + b1 * wx[i1] + b2 * wx[i2] + b3 * wx[i3];
        py[k] = b0 * wy[i0] + b1 * wy[i1] + b2 * wy[i2] + b3 * wy[i3];
        sl[k] = k ? sl[k - 1] + hypot(px[k] - px[k - 1], py[k] - py[k - 1]) : 0.0;
    }
    double total = sl[nd];
    int k = 0;
    for (int i = 0; i < n; ++i) {
        double target = fmod(i * spacing, total);
        while (k < nd && sl[k + 1] < target) k++;
        if (sl[k] > target) k = 0;
        while (k < nd && sl[k + 1] < target) k++;
        double f = (sl[k + 1] > sl[k]) ? (target - sl[k]) / (sl[k + 1] - sl[k]) : 0.0;
        double x = px[k] + f * (px[k + 1] - px[k]), y = py[k] + f * (py[k + 1] - py[k]);
        out[4 * i] = x;
        out[4 * i + 1] = y;
        out[4 * i + 2] = height;
        out[4 * i + 3] = atan2(py[k + 1] - py[k], px[k + 1] - px[k]);
    }
    free(px);
    free(py);
    free(sl);
}
