/*
 * ndt_oracle.c — CPU restatement of cuda_ndt_matcher's NDT hot path (test infrastructure).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load this file's
 * library. It is the oracle and the timed CPU baseline, never part of the GPU product.
 * Each function cites the reference file:line it restates (paths are relative to the
 * reference project root). Compiled with -ffp-contract=off so every FP operation is one
 * IEEE rounding, on x86-64 and aarch64 alike.
 */
#include "ndt_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------ */
/* Gaussian fit parameters: src/ndt_cuda/src/derivatives/types.rs:61-75                 */
/* ------------------------------------------------------------------------------------ */
void or_gauss_params(double resolution, double outlier_ratio, double* d1, double* d2) {
    double c1 = 10.0 * (1.0 - outlier_ratio);
    double c2 = outlier_ratio / (resolution * resolution * resolution);
    double d3 = -log(c2);
    double g1 = -log(c1 + c2) - d3;
    double nom = -log(c1 * exp(-0.5) + c2) - d3;
    double g2 = -2.0 * log(nom / g1);
    *d1 = g1;
    *d2 = g2;
}

/* ------------------------------------------------------------------------------------ */
/* Voxel coordinate: src/ndt_cuda/src/voxel_grid/types.rs:206-212                      */
/* floor(p / res) in f32, then Rust's saturating `as i32` (NaN -> 0).                  */
/* ------------------------------------------------------------------------------------ */
static int32_t sat_i32(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v < -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}

void or_voxel_coord(const float* p, float res, int32_t* c) {
    for (int i = 0; i < 3; ++i) c[i] = sat_i32(floorf(p[i] / res));
}

/* ------------------------------------------------------------------------------------ */
/* Morton codes: src/ndt_cuda/src/voxel_grid/gpu/morton.rs:197-326                      */
/* x bits at 2,5,8..; y at 1,4,7..; z at 0,3,6..; 21 bits per axis.                     */
/* ------------------------------------------------------------------------------------ */
static uint64_t spread21(uint64_t v) {
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

static uint32_t gather21(uint64_t v) {
    v &= 0x1249249249249249ull;
    v = (v | (v >> 2)) & 0x10C30C30C30C30C3ull;
    v = (v | (v >> 4)) & 0x100F00F00F00F00Full;
    v = (v | (v >> 8)) & 0x1F0000FF0000FFull;
    v = (v | (v >> 16)) & 0x1F00000000FFFFull;
    v = (v | (v >> 32)) & 0x1FFFFFull;
    return (uint32_t)v;
}

uint64_t or_morton_encode(uint32_t x, uint32_t y, uint32_t z) {
    return (spread21(x) << 2) | (spread21(y) << 1) | spread21(z);
}

void or_morton_decode(uint64_t code, uint32_t* x, uint32_t* y, uint32_t* z) {
    *x = gather21(code >> 2);
    *y = gather21(code >> 1);
    *z = gather21(code);
}

static uint32_t grid_q21(float g) {
    /* `if g >= 0 { min(g as u32, 0x1FFFFF) } else { 0 }` with Rust's saturating cast */
    if (!(g >= 0.0f)) return 0;
    if (g >= 2097151.0f) return 0x1FFFFFu;
    return (uint32_t)g;
}

void or_morton_codes_ref(const float* pts, size_t n, float res, uint64_t* codes,
                         float* grid_min3) {
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) mn[a] = fminf(mn[a], pts[3 * i + a]);
    float am[3];
    for (int a = 0; a < 3; ++a) am[a] = floorf(mn[a] / res) * res;
    float inv = 1.0f / res;
    for (size_t i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) q[a] = grid_q21((pts[3 * i + a] - am[a]) * inv);
        codes[i] = or_morton_encode(q[0], q[1], q[2]);
    }
    if (grid_min3)
        for (int a = 0; a < 3; ++a) grid_min3[a] = am[a];
}

static int finite3(const float* p) { return isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]); }

int or_morton_codes_coord(const float* pts, size_t n, float res, uint64_t* codes,
                          int32_t* min_coord3) {
    int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX};
    int32_t mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (size_t i = 0; i < n; ++i) {
        if (!finite3(pts + 3 * i)) continue;
        int32_t c[3];
        or_voxel_coord(pts + 3 * i, res, c);
        for (int a = 0; a < 3; ++a) {
            if (c[a] < mn[a]) mn[a] = c[a];
            if (c[a] > mx[a]) mx[a] = c[a];
        }
    }
    int ok = 1;
    for (int a = 0; a < 3; ++a)
        if (mn[a] <= mx[a] && (int64_t)mx[a] - (int64_t)mn[a] > 0x1FFFFF) ok = 0;
    for (size_t i = 0; i < n; ++i) {
        if (!finite3(pts + 3 * i)) {
            codes[i] = UINT64_MAX;
            continue;
        }
        int32_t c[3];
        or_voxel_coord(pts + 3 * i, res, c);
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            int64_t d = (int64_t)c[a] - (int64_t)mn[a];
            q[a] = d > 0x1FFFFF ? 0x1FFFFFu : (uint32_t)d;
        }
        codes[i] = or_morton_encode(q[0], q[1], q[2]);
    }
    if (min_coord3)
        for (int a = 0; a < 3; ++a) min_coord3[a] = mn[a];
    return ok;
}

/* ------------------------------------------------------------------------------------ */
/* Stable LSD radix sort: src/ndt_cuda/src/voxel_grid/gpu/radix_sort.rs:97-160          */
/* ------------------------------------------------------------------------------------ */
void or_radix_sort_pairs(uint64_t* keys, uint32_t* vals, size_t n) {
    if (n == 0) return;
    uint64_t* kb = (uint64_t*)malloc(n * sizeof(uint64_t));
    uint32_t* vb = (uint32_t*)malloc(n * sizeof(uint32_t));
    uint64_t* ka = keys;
    uint32_t* va = vals;
    for (int pass = 0; pass < 16; ++pass) {
        int shift = pass * 4;
        size_t hist[16] = {0};
        for (size_t i = 0; i < n; ++i) hist[(ka[i] >> shift) & 15u]++;
        size_t off[16], s = 0;
        for (int d = 0; d < 16; ++d) {
            off[d] = s;
            s += hist[d];
        }
        for (size_t i = 0; i < n; ++i) {
            unsigned d = (unsigned)((ka[i] >> shift) & 15u);
            kb[off[d]] = ka[i];
            vb[off[d]] = va[i];
            off[d]++;
        }
        uint64_t* tk = ka;
        ka = kb;
        kb = tk;
        uint32_t* tv = va;
        va = vb;
        vb = tv;
    }
    /* 16 passes: the data is back in the caller's arrays */
    free(kb);
    free(vb);
}

/* ------------------------------------------------------------------------------------ */
/* Segment detection: src/ndt_cuda/src/voxel_grid/gpu/segments.rs:45-89                 */
/* ------------------------------------------------------------------------------------ */
size_t or_detect_segments(const uint64_t* sorted, size_t n, uint32_t* seg_ids,
                          uint32_t* seg_starts) {
    if (n == 0) return 0;
    uint32_t cur = 0;
    seg_starts[0] = 0;
    seg_ids[0] = 0;
    for (size_t i = 1; i < n; ++i) {
        if (sorted[i] != sorted[i - 1]) {
            cur++;
            seg_starts[cur] = (uint32_t)i;
        }
        seg_ids[i] = cur;
    }
    return (size_t)cur + 1;
}

/* ------------------------------------------------------------------------------------ */
/* Symmetric eigen-decomposition (cyclic Jacobi, FP64). Stands in for nalgebra 0.33.2  */
/* `symmetric_eigen` at src/ndt_cuda/src/voxel_grid/types.rs:120 and                     */
/* src/ndt_cuda/src/optimization/newton.rs:102,123. A converged Jacobi decomposition    */
/* agrees with nalgebra's implicit QR to FP64 rounding; eigenvalue order may differ,    */
/* which none of the callers depend on except through summation order.                 */
/* ------------------------------------------------------------------------------------ */
static void jacobi_sym(double* a, double* v, int n, int max_sweeps) {
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) v[i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        double off = 0.0, dg = 0.0;
        for (int i = 0; i < n; ++i) {
            dg += a[i * n + i] * a[i * n + i];
            for (int j = i + 1; j < n; ++j) off += a[i * n + j] * a[i * n + j];
        }
        if (off <= 1e-40 * dg) break;
        for (int p = 0; p < n - 1; ++p) {
            for (int q = p + 1; q < n; ++q) {
                double apq = a[p * n + q];
                if (apq == 0.0) continue;
                double theta = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
                double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
                if (theta < 0.0) t = -t;
                double c = 1.0 / sqrt(t * t + 1.0);
                double s = t * c;
                a[p * n + p] = a[p * n + p] - t * apq;
                a[q * n + q] = a[q * n + q] + t * apq;
                a[p * n + q] = 0.0;
                a[q * n + p] = 0.0;
                for (int r = 0; r < n; ++r) {
                    if (r == p || r == q) continue;
                    double arp = a[r * n + p], arq = a[r * n + q];
                    double np = c * arp - s * arq;
                    double nq = s * arp + c * arq;
                    a[r * n + p] = np;
                    a[p * n + r] = np;
                    a[r * n + q] = nq;
                    a[q * n + r] = nq;
                }
                for (int r = 0; r < n; ++r) {
                    double vrp = v[r * n + p], vrq = v[r * n + q];
                    v[r * n + p] = c * vrp - s * vrq;
                    v[r * n + q] = s * vrp + c * vrq;
                }
            }
        }
    }
}

void or_eigen_sym3(const double* a9, double* ev, double* vecs) {
    double a[9];
    memcpy(a, a9, sizeof a);
    jacobi_sym(a, vecs, 3, 32);
    for (int i = 0; i < 3; ++i) ev[i] = a[i * 3 + i];
}

void or_eigen_sym6(const double* a36, double* ev, double* vecs) {
    double a[36];
    memcpy(a, a36, sizeof a);
    jacobi_sym(a, vecs, 6, 64);
    for (int i = 0; i < 6; ++i) ev[i] = a[i * 6 + i];
}

/* ------------------------------------------------------------------------------------ */
/* Reference hash semantics: src/cuda_ffi/csrc/voxel_hash.cu:33-58 (pack, fmix64 % cap) */
/* and :218-228 (capacity = next power of two >= 2V).                                    */
/* ------------------------------------------------------------------------------------ */
int64_t or_pack_key(int32_t gx, int32_t gy, int32_t gz) {
    int64_t ux = (int64_t)(gx + (1 << 20));
    int64_t uy = (int64_t)(gy + (1 << 20));
    int64_t uz = (int64_t)(gz + (1 << 20));
    return (ux << 42) | (uy << 21) | uz;
}

uint32_t or_hash_slot(int64_t key, uint32_t capacity) {
    uint64_t k = (uint64_t)key;
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return (uint32_t)(k % capacity);
}

struct or_grid {
    size_t nv;
    float res;
    int32_t* coords;
    float* means;
    float* covs;
    float* icovs;
    float* paxes;
    uint32_t* counts;
    uint32_t cap;
    int64_t* hkeys;
    int32_t* hvals;
};

static void hash_insert(or_grid* g, int64_t key, int32_t val) {
    uint32_t slot = or_hash_slot(key, g->cap);
    for (uint32_t i = 0; i < g->cap; ++i) {
        uint32_t s = (slot + i) % g->cap;
        if (g->hkeys[s] == -1 || g->hkeys[s] == key) {
            g->hkeys[s] = key;
            g->hvals[s] = val;
            return;
        }
    }
}

int32_t or_grid_lookup(const or_grid* g, int32_t gx, int32_t gy, int32_t gz) {
    if (!g || g->cap == 0) return -1;
    int64_t key = or_pack_key(gx, gy, gz);
    uint32_t slot = or_hash_slot(key, g->cap);
    for (uint32_t i = 0; i < g->cap; ++i) {
        uint32_t s = (slot + i) % g->cap;
        int64_t k = g->hkeys[s];
        if (k == -1) return -1;
        if (k == key) return g->hvals[s];
    }
    return -1;
}

/* ------------------------------------------------------------------------------------ */
/* Voxel statistics: src/ndt_cuda/src/voxel_grid/types.rs:54-190 (from_statistics,      */
/* regularize_covariance); accumulation order follows build_voxel_grid_cpu              */
/* (src/ndt_cuda/src/voxel_grid/cpu.rs:51-75): points of a voxel in input order.        */
/* ------------------------------------------------------------------------------------ */
static int finalize_voxel(const double* mean, const double* cov, float ratio, float* mean_out,
                          float* cov_out, float* icov_out, float* pax_out) {
    double ev[3], V[9], a9[9];
    memcpy(a9, cov, sizeof a9);
    or_eigen_sym3(a9, ev, V);
    double mx = 0.0;
    for (int i = 0; i < 3; ++i) mx = fmax(mx, ev[i]);
    if (!(mx > 0.0)) return 0;
    int mi = 0;
    for (int i = 1; i < 3; ++i)
        if (ev[i] < ev[mi]) mi = i;
    double thr = mx * (double)ratio;
    int needs = 0;
    double cl[3];
    for (int i = 0; i < 3; ++i) {
        cl[i] = ev[i] < thr ? thr : ev[i];
        if (ev[i] < thr) needs = 1;
    }
    double rc[9], ic[9];
    for (int r = 0; r < 3; ++r) {
        for (int c = r; c < 3; ++c) {
            double sr = 0.0, si = 0.0;
            for (int k = 0; k < 3; ++k) {
                sr += V[r * 3 + k] * cl[k] * V[c * 3 + k];
                si += V[r * 3 + k] * (1.0 / cl[k]) * V[c * 3 + k];
            }
            rc[r * 3 + c] = rc[c * 3 + r] = sr;
            ic[r * 3 + c] = ic[c * 3 + r] = si;
        }
    }
    for (int i = 0; i < 9; ++i) {
        cov_out[i] = (float)(needs ? rc[i] : cov[i]);
        icov_out[i] = (float)ic[i];
    }
    for (int a = 0; a < 3; ++a) {
        mean_out[a] = (float)mean[a];
        pax_out[a] = (float)V[a * 3 + mi];
    }
    return 1;
}

or_grid* or_grid_build(const float* pts, size_t n, float res, int min_points, float ratio,
                       int centered) {
    uint64_t* keys = (uint64_t*)malloc((n ? n : 1) * sizeof(uint64_t));
    uint32_t* idx = (uint32_t*)malloc((n ? n : 1) * sizeof(uint32_t));
    int32_t mn[3];
    if (!or_morton_codes_coord(pts, n, res, keys, mn)) {
        free(keys);
        free(idx);
        return NULL;
    }
    for (size_t i = 0; i < n; ++i) idx[i] = (uint32_t)i;
    or_radix_sort_pairs(keys, idx, n);
    size_t nf = n;
    while (nf > 0 && keys[nf - 1] == UINT64_MAX) nf--; /* non-finite points sort last */

    or_grid* g = (or_grid*)calloc(1, sizeof(or_grid));
    g->res = res;
    size_t cap0 = nf ? nf : 1;
    g->coords = (int32_t*)malloc(cap0 * 3 * sizeof(int32_t));
    g->means = (float*)malloc(cap0 * 3 * sizeof(float));
    g->covs = (float*)malloc(cap0 * 9 * sizeof(float));
    g->icovs = (float*)malloc(cap0 * 9 * sizeof(float));
    g->paxes = (float*)malloc(cap0 * 3 * sizeof(float));
    g->counts = (uint32_t*)malloc(cap0 * sizeof(uint32_t));

    size_t i = 0;
    while (i < nf) {
        size_t j = i + 1;
        while (j < nf && keys[j] == keys[i]) j++;
        size_t cnt = j - i;
        if ((int)cnt >= min_points) {
            double sum[3] = {0, 0, 0}, sq[9] = {0};
            for (size_t k = i; k < j; ++k) {
                const float* p = pts + 3 * (size_t)idx[k];
                double v[3] = {(double)p[0], (double)p[1], (double)p[2]};
                for (int a = 0; a < 3; ++a) sum[a] += v[a];
                if (!centered)
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) sq[r * 3 + c] += v[r] * v[c];
            }
            double nn = (double)cnt, mean[3], cov[9];
            for (int a = 0; a < 3; ++a) mean[a] = sum[a] / nn;
            if (centered) {
                for (size_t k = i; k < j; ++k) {
                    const float* p = pts + 3 * (size_t)idx[k];
                    double d[3] = {(double)p[0] - mean[0], (double)p[1] - mean[1],
                                   (double)p[2] - mean[2]};
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) sq[r * 3 + c] += d[r] * d[c];
                }
                for (int e = 0; e < 9; ++e) cov[e] = sq[e] / (nn - 1.0);
            } else {
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c)
                        cov[r * 3 + c] = (sq[r * 3 + c] - (mean[r] * mean[c]) * nn) / (nn - 1.0);
            }
            size_t v = g->nv;
            if (finalize_voxel(mean, cov, ratio, g->means + 3 * v, g->covs + 9 * v,
                               g->icovs + 9 * v, g->paxes + 3 * v)) {
                or_voxel_coord(pts + 3 * (size_t)idx[i], res, g->coords + 3 * v);
                g->counts[v] = (uint32_t)cnt;
                g->nv++;
            }
        }
        i = j;
    }
    free(keys);
    free(idx);

    uint32_t cap = 1;
    while ((uint64_t)cap < (uint64_t)g->nv * 2) cap *= 2;
    g->cap = cap;
    g->hkeys = (int64_t*)malloc((size_t)cap * sizeof(int64_t));
    g->hvals = (int32_t*)malloc((size_t)cap * sizeof(int32_t));
    for (uint32_t s = 0; s < cap; ++s) {
        g->hkeys[s] = -1;
        g->hvals[s] = -1;
    }
    for (size_t v = 0; v < g->nv; ++v) {
        const int32_t* c = g->coords + 3 * v;
        hash_insert(g, or_pack_key(c[0], c[1], c[2]), (int32_t)v);
    }
    return g;
}

void or_grid_free(or_grid* g) {
    if (!g) return;
    free(g->coords);
    free(g->means);
    free(g->covs);
    free(g->icovs);
    free(g->paxes);
    free(g->counts);
    free(g->hkeys);
    free(g->hvals);
    free(g);
}

size_t or_grid_size(const or_grid* g) { return g ? g->nv : 0; }
uint32_t or_grid_hash_capacity(const or_grid* g) { return g ? g->cap : 0; }

void or_grid_copy(const or_grid* g, int32_t* coords, float* means, float* covs, float* icovs,
                  uint32_t* counts, float* paxes) {
    size_t v = g->nv;
    if (coords) memcpy(coords, g->coords, v * 3 * sizeof(int32_t));
    if (means) memcpy(means, g->means, v * 3 * sizeof(float));
    if (covs) memcpy(covs, g->covs, v * 9 * sizeof(float));
    if (icovs) memcpy(icovs, g->icovs, v * 9 * sizeof(float));
    if (counts) memcpy(counts, g->counts, v * sizeof(uint32_t));
    if (paxes) memcpy(paxes, g->paxes, v * 3 * sizeof(float));
}

/* ------------------------------------------------------------------------------------ */
/* Neighbour queries                                                                    */
/* ------------------------------------------------------------------------------------ */
/* Offsets in the fixed order of src/cuda_ffi/csrc/ndt_graph_kernels.cu:29-39:
 * dx outermost, then dy, then dz, each from -1 to +1. */
static void offset27(int n, int* dx, int* dy, int* dz) {
    *dx = n / 9 - 1;
    *dy = (n / 3) % 3 - 1;
    *dz = n % 3 - 1;
}

/* graph_hash_query_inline (src/cuda_ffi/csrc/ndt_graph_kernels.cu:47-104), f32 arithmetic */
void or_query_gpu_sem(const or_grid* g, const float* q, size_t n, int max_nb, int32_t* idx,
                      int32_t* cnt) {
    float inv = 1.0f / g->res;
    float r2 = g->res * g->res;
    for (size_t i = 0; i < n; ++i) {
        const float* p = q + 3 * i;
        int32_t gx = (int32_t)floorf(p[0] * inv);
        int32_t gy = (int32_t)floorf(p[1] * inv);
        int32_t gz = (int32_t)floorf(p[2] * inv);
        int c = 0;
        for (int k = 0; k < 27 && c < max_nb; ++k) {
            int dx, dy, dz;
            offset27(k, &dx, &dy, &dz);
            int32_t v = or_grid_lookup(g, gx + dx, gy + dy, gz + dz);
            if (v < 0) continue;
            const float* m = g->means + 3 * v;
            float ex = p[0] - m[0], ey = p[1] - m[1], ez = p[2] - m[2];
            float d2 = ex * ex;
            d2 = d2 + ey * ey;
            d2 = d2 + ez * ez;
            if (d2 <= r2) idx[i * (size_t)max_nb + c++] = v;
        }
        for (int k = c; k < max_nb; ++k) idx[i * (size_t)max_nb + k] = -1;
        cnt[i] = c;
    }
}

/* kiddo 4.2.1 ImmutableKdTree::within with SquaredEuclidean (voxel_grid/search.rs:90-99):
 * every centroid with squared f32 distance <= radius^2, nearest first. Candidates come from
 * the 27 cells around the query: a centroid lies inside its own cell, so any centroid within
 * one cell-width of the query is in one of them. */
int or_radius_search(const or_grid* g, const float* q, float radius, int32_t* idx, int cap) {
    float inv = 1.0f / g->res;
    float r2 = radius * radius;
    int32_t gx = (int32_t)floorf(q[0] * inv);
    int32_t gy = (int32_t)floorf(q[1] * inv);
    int32_t gz = (int32_t)floorf(q[2] * inv);
    int32_t cand[27];
    float dist[27];
    int c = 0;
    for (int k = 0; k < 27; ++k) {
        int dx, dy, dz;
        offset27(k, &dx, &dy, &dz);
        int32_t v = or_grid_lookup(g, gx + dx, gy + dy, gz + dz);
        if (v < 0) continue;
        const float* m = g->means + 3 * v;
        float ex = q[0] - m[0], ey = q[1] - m[1], ez = q[2] - m[2];
        float d2 = ex * ex;
        d2 = d2 + ey * ey;
        d2 = d2 + ez * ez;
        if (d2 <= r2) {
            cand[c] = v;
            dist[c] = d2;
            c++;
        }
    }
    /* insertion sort by (distance, index) */
    for (int a = 1; a < c; ++a) {
        int32_t cv = cand[a];
        float cd = dist[a];
        int b = a - 1;
        while (b >= 0 && (dist[b] > cd || (dist[b] == cd && cand[b] > cv))) {
            cand[b + 1] = cand[b];
            dist[b + 1] = dist[b];
            b--;
        }
        cand[b + 1] = cv;
        dist[b + 1] = cd;
    }
    int m = c < cap ? c : cap;
    for (int a = 0; a < m; ++a) idx[a] = cand[a];
    return c;
}

/* ------------------------------------------------------------------------------------ */
/* Pose algebra                                                                         */
/* ------------------------------------------------------------------------------------ */
/* R = Rx(roll) * Ry(pitch) * Rz(yaw): src/ndt_cuda/src/derivatives/cpu.rs:339-378 */
void or_pose_to_T34_xyz(const double* pose, double* T) {
    double sr = sin(pose[3]), cr = cos(pose[3]);
    double sp = sin(pose[4]), cp = cos(pose[4]);
    double sy = sin(pose[5]), cy = cos(pose[5]);
    T[0] = cp * cy;
    T[1] = -cp * sy;
    T[2] = sp;
    T[3] = pose[0];
    T[4] = sr * sp * cy + cr * sy;
    T[5] = cr * cy - sr * sp * sy;
    T[6] = -sr * cp;
    T[7] = pose[1];
    T[8] = sr * sy - cr * sp * cy;
    T[9] = cr * sp * sy + sr * cy;
    T[10] = cr * cp;
    T[11] = pose[2];
}

/* nalgebra UnitQuaternion::from_euler_angles(roll, pitch, yaw) = Rz*Ry*Rx, used by
 * pose_vector_to_isometry (src/ndt_cuda/src/optimization/types.rs:156-161) and hence by
 * the NVTL evaluated on the final isometry. */
void or_pose_to_T34_zyx(const double* pose, double* T) {
    double sr = sin(pose[3]), cr = cos(pose[3]);
    double sp = sin(pose[4]), cp = cos(pose[4]);
    double sy = sin(pose[5]), cy = cos(pose[5]);
    T[0] = cy * cp;
    T[1] = cy * sp * sr - sy * cr;
    T[2] = cy * sp * cr + sy * sr;
    T[3] = pose[0];
    T[4] = sy * cp;
    T[5] = sy * sp * sr + cy * cr;
    T[6] = sy * sp * cr - cy * sr;
    T[7] = pose[1];
    T[8] = -sp;
    T[9] = cp * sr;
    T[10] = cp * cr;
    T[11] = pose[2];
}

/* Angular Jacobian / Hessian terms: src/ndt_cuda/src/derivatives/angular.rs:37-189.
 * The small-angle rule (|angle| < 1e-5 -> sin 0, cos 1) is the CPU path's. */
typedef struct {
    double j[8][3];
    double h[15][3];
} angular_t;

static void angular_init(angular_t* A, double roll, double pitch, double yaw, int small_rule) {
    double sx = sin(roll), cx = cos(roll), sy = sin(pitch), cy = cos(pitch), sz = sin(yaw),
           cz = cos(yaw);
    if (small_rule) {
        if (fabs(roll) < 1e-5) sx = 0.0, cx = 1.0;
        if (fabs(pitch) < 1e-5) sy = 0.0, cy = 1.0;
        if (fabs(yaw) < 1e-5) sz = 0.0, cz = 1.0;
    }
    double j[8][3] = {
        {-sx * sz + cx * sy * cz, -sx * cz - cx * sy * sz, -cx * cy},
        {cx * sz + sx * sy * cz, cx * cz - sx * sy * sz, -sx * cy},
        {-sy * cz, sy * sz, cy},
        {sx * cy * cz, -sx * cy * sz, sx * sy},
        {-cx * cy * cz, cx * cy * sz, -cx * sy},
        {-cy * sz, -cy * cz, 0.0},
        {cx * cz - sx * sy * sz, -cx * sz - sx * sy * cz, 0.0},
        {sx * cz + cx * sy * sz, cx * sy * cz - sx * sz, 0.0},
    };
    double h[15][3] = {
        {-cx * sz - sx * sy * cz, -cx * cz + sx * sy * sz, sx * cy},
        {-sx * sz + cx * sy * cz, -cx * sy * sz - sx * cz, -cx * cy},
        {cx * cy * cz, -cx * cy * sz, cx * sy},
        {sx * cy * cz, -sx * cy * sz, sx * sy},
        {-sx * cz - cx * sy * sz, sx * sz - cx * sy * cz, 0.0},
        {cx * cz - sx * sy * sz, -sx * sy * cz - cx * sz, 0.0},
        {-cy * cz, cy * sz, sy},
        {-sx * sy * cz, sx * sy * sz, sx * cy},
        {cx * sy * cz, -cx * sy * sz, -cx * cy},
        {sy * sz, sy * cz, 0.0},
        {-sx * cy * sz, -sx * cy * cz, 0.0},
        {cx * cy * sz, cx * cy * cz, 0.0},
        {-cy * cz, cy * sz, 0.0},
        {-cx * sz - sx * sy * cz, -cx * cz + sx * sy * sz, 0.0},
        {-sx * sz + cx * sy * cz, -cx * sy * sz - sx * cz, 0.0},
    };
    memcpy(A->j, j, sizeof j);
    memcpy(A->h, h, sizeof h);
}

/* Point Jacobian J (3x6) and point Hessian blocks: src/ndt_cuda/src/derivatives/cpu.rs:27-125.
 * pH[i][j][k] = d^2 T_k / d p_i d p_j for angular i, j (3..5). */
static void point_derivs(const angular_t* A, const double* p, double J[3][6],
                         double pH[3][3][3]) {
    double t[8], s[15];
    for (int r = 0; r < 8; ++r) t[r] = A->j[r][0] * p[0] + A->j[r][1] * p[1] + A->j[r][2] * p[2];
    for (int r = 0; r < 15; ++r)
        s[r] = A->h[r][0] * p[0] + A->h[r][1] * p[1] + A->h[r][2] * p[2];
    memset(J, 0, sizeof(double) * 18);
    J[0][0] = 1.0;
    J[1][1] = 1.0;
    J[2][2] = 1.0;
    J[1][3] = t[0];
    J[2][3] = t[1];
    J[0][4] = t[2];
    J[1][4] = t[3];
    J[2][4] = t[4];
    J[0][5] = t[5];
    J[1][5] = t[6];
    J[2][5] = t[7];
    /* a = [0,a2,a3], b = [0,b2,b3], c = [0,c2,c3], d = [d1,d2,d3], e = [e1,e2,e3], f = [f1,f2,f3] */
    double a[3] = {0.0, s[0], s[1]}, b[3] = {0.0, s[2], s[3]}, c[3] = {0.0, s[4], s[5]};
    double d[3] = {s[6], s[7], s[8]}, e[3] = {s[9], s[10], s[11]}, f[3] = {s[12], s[13], s[14]};
    for (int k = 0; k < 3; ++k) {
        pH[0][0][k] = a[k];
        pH[0][1][k] = b[k];
        pH[1][0][k] = b[k];
        pH[0][2][k] = c[k];
        pH[2][0][k] = c[k];
        pH[1][1][k] = d[k];
        pH[1][2][k] = e[k];
        pH[2][1][k] = e[k];
        pH[2][2][k] = f[k];
    }
}

/* compute_derivative_single: src/ndt_cuda/src/derivatives/cpu.rs:139-240 (Magnusson 6.9-6.13).
 * check_range reproduces the CPU path's `d2*e in [0,1]` guard (the graph kernel has none). */
static void pair_derivs(const double* x, const double* C9, double J[3][6], double pH[3][3][3],
                        double d1, double d2, int check_range, double* score, double* grad,
                        double* hess, int* used) {
    double c[3];
    for (int r = 0; r < 3; ++r) c[r] = C9[r * 3] * x[0] + C9[r * 3 + 1] * x[1] + C9[r * 3 + 2] * x[2];
    double xcx = x[0] * c[0] + x[1] * c[1] + x[2] * c[2];
    double e = exp(-d2 * xcx * 0.5);
    double sc = -d1 * e;
    double w = d2 * e;
    if (check_range && (!(w >= 0.0 && w <= 1.0) || !isfinite(w))) {
        *used = 0;
        return;
    }
    *used = 1;
    w *= d1; /* d1*d2*e */
    double g[6];
    for (int i = 0; i < 6; ++i) g[i] = J[0][i] * c[0] + J[1][i] * c[1] + J[2][i] * c[2];
    *score += sc;
    for (int i = 0; i < 6; ++i) grad[i] += w * g[i];
    double CJ[3][6];
    for (int r = 0; r < 3; ++r)
        for (int i = 0; i < 6; ++i)
            CJ[r][i] = C9[r * 3] * J[0][i] + C9[r * 3 + 1] * J[1][i] + C9[r * 3 + 2] * J[2][i];
    for (int i = 0; i < 6; ++i) {
        for (int j = 0; j < 6; ++j) {
            double jcj = J[0][i] * CJ[0][j] + J[1][i] * CJ[1][j] + J[2][i] * CJ[2][j];
            double ph = 0.0;
            if (i >= 3 && j >= 3) {
                const double* v = pH[i - 3][j - 3];
                ph = c[0] * v[0] + c[1] * v[1] + c[2] * v[2];
            }
            hess[i * 6 + j] += w * (-d2 * g[i] * g[j] + ph + jcj);
        }
    }
}

static void to_d9(const float* f9, double* d9) {
    for (int i = 0; i < 9; ++i) d9[i] = (double)f9[i];
}

void or_derivatives_cpu(const or_grid* g, const float* src, size_t n, const double* pose,
                        double d1, double d2, double* score, double* grad, double* hess,
                        int32_t* ncorr) {
    angular_t A;
    angular_init(&A, pose[3], pose[4], pose[5], 1);
    double T[12];
    or_pose_to_T34_xyz(pose, T);
    *score = 0.0;
    memset(grad, 0, 6 * sizeof(double));
    memset(hess, 0, 36 * sizeof(double));
    int32_t nc = 0;
    int32_t nb[32];
    for (size_t i = 0; i < n; ++i) {
        double p[3] = {(double)src[3 * i], (double)src[3 * i + 1], (double)src[3 * i + 2]};
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = T[r * 4] * p[0] + T[r * 4 + 1] * p[1] + T[r * 4 + 2] * p[2] + T[r * 4 + 3];
        float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
        int k = or_radius_search(g, qf, g->res, nb, 32);
        if (k == 0) continue;
        if (k > 32) k = 32;
        double J[3][6], pH[3][3][3];
        point_derivs(&A, p, J, pH);
        for (int a = 0; a < k; ++a) {
            const float* m = g->means + 3 * nb[a];
            double x[3] = {q[0] - (double)m[0], q[1] - (double)m[1], q[2] - (double)m[2]};
            double C[9];
            to_d9(g->icovs + 9 * nb[a], C);
            int used;
            pair_derivs(x, C, J, pH, d1, d2, 1, score, grad, hess, &used);
            nc++; /* AggregatedDerivatives::add counts zeroed pairs too */
        }
    }
    *ncorr = nc;
}

/* ndt_graph_compute_kernel (src/cuda_ffi/csrc/ndt_graph_kernels.cu:163-302) in FP64:
 * 27 cells in offset order, one voxel per cell, dist^2 <= res^2, at most max_nb. */
void or_derivatives_gpu_sem(const or_grid* g, const float* src, size_t n, const double* pose,
                            double d1, double d2, int max_nb, double* score, double* grad,
                            double* hess, int32_t* ncorr) {
    angular_t A;
    angular_init(&A, pose[3], pose[4], pose[5], 0);
    double T[12];
    or_pose_to_T34_xyz(pose, T);
    double inv = 1.0 / (double)g->res;
    double r2 = (double)g->res * (double)g->res;
    *score = 0.0;
    memset(grad, 0, 6 * sizeof(double));
    memset(hess, 0, 36 * sizeof(double));
    int32_t nc = 0;
    for (size_t i = 0; i < n; ++i) {
        double p[3] = {(double)src[3 * i], (double)src[3 * i + 1], (double)src[3 * i + 2]};
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = T[r * 4] * p[0] + T[r * 4 + 1] * p[1] + T[r * 4 + 2] * p[2] + T[r * 4 + 3];
        int32_t gx = (int32_t)floor(q[0] * inv), gy = (int32_t)floor(q[1] * inv),
                gz = (int32_t)floor(q[2] * inv);
        int32_t nb[27];
        int c = 0;
        for (int k = 0; k < 27 && c < max_nb; ++k) {
            int dx, dy, dz;
            offset27(k, &dx, &dy, &dz);
            int32_t v = or_grid_lookup(g, gx + dx, gy + dy, gz + dz);
            if (v < 0) continue;
            const float* m = g->means + 3 * v;
            double ex = q[0] - m[0], ey = q[1] - m[1], ez = q[2] - m[2];
            if (ex * ex + ey * ey + ez * ez <= r2) nb[c++] = v;
        }
        if (c == 0) continue;
        double J[3][6], pH[3][3][3];
        point_derivs(&A, p, J, pH);
        for (int a = 0; a < c; ++a) {
            const float* m = g->means + 3 * nb[a];
            double x[3] = {q[0] - (double)m[0], q[1] - (double)m[1], q[2] - (double)m[2]};
            double C[9];
            to_d9(g->icovs + 9 * nb[a], C);
            int used;
            pair_derivs(x, C, J, pH, d1, d2, 0, score, grad, hess, &used);
            nc++;
        }
    }
    *ncorr = nc;
}

/* ------------------------------------------------------------------------------------ */
/* Newton steps                                                                         */
/* ------------------------------------------------------------------------------------ */
/* newton_step_negative_definite (src/ndt_cuda/src/optimization/newton.rs:160-176), with
 * is_negative_definite (:96-99), regularize_hessian_negative_definite (:118-144) and the
 * SVD solve of newton_step (:21-37). For a symmetric matrix the SVD pseudo-inverse with an
 * absolute singular-value cut `tol` equals V diag(1/lambda, |lambda| > tol) V^T. */
int or_newton_step_nd(const double* g, const double* H, double min_eig, double tol, double* x) {
    double ev[6], V[36];
    or_eigen_sym6(H, ev, V);
    int nd = 1;
    for (int i = 0; i < 6; ++i)
        if (!(ev[i] < 0.0)) nd = 0;
    if (!nd)
        for (int i = 0; i < 6; ++i)
            if (ev[i] > min_eig) ev[i] = min_eig;
    double mx = 0.0;
    for (int i = 0; i < 6; ++i) mx = fmax(mx, fabs(ev[i]));
    if (mx < tol) return 0;
    for (int i = 0; i < 6; ++i) x[i] = 0.0;
    for (int k = 0; k < 6; ++k) {
        if (!(fabs(ev[k]) > tol)) continue;
        double y = 0.0;
        for (int j = 0; j < 6; ++j) y += V[j * 6 + k] * (-g[j]);
        y /= ev[k];
        for (int i = 0; i < 6; ++i) x[i] += V[i * 6 + k] * y;
    }
    return 1;
}

/* jacobi_svd_solve_6x6_f64 (src/cuda_ffi/csrc/jacobi_svd_6x6.cuh:135-274): cyclic Jacobi,
 * <= 30 sweeps, stop when 2*sum(offdiag^2) < 1e-28 * sum(diag^2), skip |a_pq| < 1e-15, then
 * x = V diag(1/|lambda|) V^T (-g) keeping |lambda| > max(1e-10 * max|lambda|, 1e-15). */
int or_jacobi_svd_solve(const double* H, const double* g, double* x) {
    double A[36], V[36];
    memcpy(A, H, sizeof A);
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) V[i * 6 + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0, dg = 0.0;
        for (int i = 0; i < 6; ++i) {
            dg += A[i * 6 + i] * A[i * 6 + i];
            for (int j = i + 1; j < 6; ++j) off += A[i * 6 + j] * A[i * 6 + j];
        }
        off *= 2.0;
        if (off < 1e-14 * 1e-14 * dg) break;
        for (int p = 0; p < 5; ++p) {
            for (int q = p + 1; q < 6; ++q) {
                double apq = A[p * 6 + q];
                if (fabs(apq) < 1e-15) continue;
                double app = A[p * 6 + p], aqq = A[q * 6 + q];
                double tau = (aqq - app) / (2.0 * apq);
                double t = tau >= 0.0 ? 1.0 / (tau + sqrt(tau * tau + 1.0))
                                      : -1.0 / (-tau + sqrt(tau * tau + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                double c2 = c * c, s2 = s * s, cs = c * s;
                A[p * 6 + p] = c2 * app + s2 * aqq - 2.0 * cs * apq;
                A[q * 6 + q] = s2 * app + c2 * aqq + 2.0 * cs * apq;
                A[p * 6 + q] = 0.0;
                A[q * 6 + p] = 0.0;
                for (int k = 0; k < 6; ++k) {
                    if (k == p || k == q) continue;
                    double apk = A[p * 6 + k], aqk = A[q * 6 + k];
                    double np = c * apk - s * aqk, nq = s * apk + c * aqk;
                    A[p * 6 + k] = np;
                    A[k * 6 + p] = np;
                    A[q * 6 + k] = nq;
                    A[k * 6 + q] = nq;
                }
                for (int i = 0; i < 6; ++i) {
                    double vip = V[i * 6 + p], viq = V[i * 6 + q];
                    V[i * 6 + p] = c * vip - s * viq;
                    V[i * 6 + q] = s * vip + c * viq;
                }
            }
        }
    }
    double ev[6], mx = 0.0;
    for (int i = 0; i < 6; ++i) {
        ev[i] = A[i * 6 + i];
        if (fabs(ev[i]) > mx) mx = fabs(ev[i]);
    }
    double thr = 1e-10 * mx;
    if (thr < 1e-15) thr = 1e-15;
    double y[6], z[6];
    int nz = 0;
    for (int i = 0; i < 6; ++i) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s += V[j * 6 + i] * (-g[j]);
        y[i] = s;
    }
    for (int i = 0; i < 6; ++i) {
        double a = fabs(ev[i]);
        if (a > thr) {
            z[i] = y[i] / a;
            nz++;
        } else {
            z[i] = 0.0;
        }
    }
    for (int i = 0; i < 6; ++i) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s += V[i * 6 + j] * z[j];
        x[i] = s;
    }
    return nz > 0;
}

/* ------------------------------------------------------------------------------------ */
/* Scoring: compute_nvtl_simple (src/ndt_cuda/src/scoring/nvtl.rs:196-260)              */
/* ------------------------------------------------------------------------------------ */
double or_nvtl(const or_grid* g, const float* src, size_t n, const double* T, double resolution,
               double d1, double d2) {
    if (n == 0) return 0.0;
    double total = 0.0;
    size_t cnt = 0;
    int32_t nb[32];
    for (size_t i = 0; i < n; ++i) {
        double p[3] = {(double)src[3 * i], (double)src[3 * i + 1], (double)src[3 * i + 2]};
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = T[r * 4] * p[0] + T[r * 4 + 1] * p[1] + T[r * 4 + 2] * p[2] + T[r * 4 + 3];
        float qf[3] = {(float)q[0], (float)q[1], (float)q[2]};
        int k = or_radius_search(g, qf, (float)resolution, nb, 32);
        if (k == 0) continue;
        if (k > 32) k = 32;
        double best = -INFINITY;
        for (int a = 0; a < k; ++a) {
            const float* m = g->means + 3 * nb[a];
            double x[3] = {q[0] - (double)m[0], q[1] - (double)m[1], q[2] - (double)m[2]};
            const float* C = g->icovs + 9 * nb[a];
            double cx[3];
            for (int r = 0; r < 3; ++r)
                cx[r] = (double)C[r * 3] * x[0] + (double)C[r * 3 + 1] * x[1] +
                        (double)C[r * 3 + 2] * x[2];
            double md = x[0] * cx[0] + x[1] * cx[1] + x[2] * cx[2];
            double s = -d1 * exp(-d2 * md / 2.0);
            if (s > best) best = s;
        }
        total += best;
        cnt++;
    }
    return cnt ? total / (double)cnt : 0.0;
}

void or_score_gpu_sem(const or_grid* g, const float* src, size_t n, const double* T, double d1,
                      double d2, int max_nb, double* score, int32_t* ncorr) {
    double inv = 1.0 / (double)g->res, r2 = (double)g->res * (double)g->res;
    double s = 0.0;
    int32_t nc = 0;
    for (size_t i = 0; i < n; ++i) {
        double p[3] = {(double)src[3 * i], (double)src[3 * i + 1], (double)src[3 * i + 2]};
        double q[3];
        for (int r = 0; r < 3; ++r)
            q[r] = T[r * 4] * p[0] + T[r * 4 + 1] * p[1] + T[r * 4 + 2] * p[2] + T[r * 4 + 3];
        int32_t gx = (int32_t)floor(q[0] * inv), gy = (int32_t)floor(q[1] * inv),
                gz = (int32_t)floor(q[2] * inv);
        int c = 0;
        for (int k = 0; k < 27 && c < max_nb; ++k) {
            int dx, dy, dz;
            offset27(k, &dx, &dy, &dz);
            int32_t v = or_grid_lookup(g, gx + dx, gy + dy, gz + dz);
            if (v < 0) continue;
            const float* m = g->means + 3 * v;
            double x[3] = {q[0] - m[0], q[1] - m[1], q[2] - m[2]};
            if (x[0] * x[0] + x[1] * x[1] + x[2] * x[2] > r2) continue;
            const float* C = g->icovs + 9 * v;
            double cx[3];
            for (int r = 0; r < 3; ++r)
                cx[r] = (double)C[r * 3] * x[0] + (double)C[r * 3 + 1] * x[1] +
                        (double)C[r * 3 + 2] * x[2];
            double md = x[0] * cx[0] + x[1] * cx[1] + x[2] * cx[2];
            s += -d1 * exp(-d2 * md * 0.5);
            c++;
        }
        nc += c;
    }
    *score = s;
    *ncorr = nc;
}

/* ------------------------------------------------------------------------------------ */
/* Alignment loops                                                                      */
/* ------------------------------------------------------------------------------------ */
/* count_oscillation (src/ndt_cuda/src/optimization/oscillation.rs:46-99) over positions */
/* MoreThuenteConfig::default() (more_thuente.rs:36-46) */
#define MT_STEP_MIN 1e-9
#define MT_STEP_MAX 0.1
#define MT_MAX_ITER 10

/* ---- More-Thuente line search (CPU path with use_line_search) ----
 * more_thuente_search (src/ndt_cuda/src/optimization/more_thuente.rs:236-410) after More &
 * Thuente (1994), with the interpolants of Sun & Yuan (2006, eqs. 2.4.2, 2.4.5, 2.4.52). The
 * score is maximised, so the search minimises phi = -score. Until a trial has psi <= 0 and
 * psi' >= 0 the interval [a_l, a_u] is kept on psi(a) = phi(a) - phi(0) - mu phi'(0) a, then
 * on phi itself. */

/* minimiser of the cubic through (a, fa, ga) and (b, fb, gb); *ok = 0 when it is complex */
static double mt_cubic(double a, double fa, double ga, double b, double fb, double gb, int* ok) {
    const double z = 3.0 * (fb - fa) / (b - a) - gb - ga;
    const double w2 = z * z - gb * ga;
    if (w2 < 0.0) {
        *ok = 0;
        return 0.0;
    }
    *ok = 1;
    const double w = sqrt(w2);
    return a + (b - a) * (w - ga - z) / (gb - ga + 2.0 * w);
}

/* trial_value_selection (more_thuente.rs:83-194): l = best end, u = other end, t = trial */
static double mt_next(double al, double fl, double gl, double au, double fu, double gu,
                      double at, double ft, double gt) {
    int ok;
    if (ft > fl) { /* case 1: bracketed by [al, at] */
        const double ac = mt_cubic(al, fl, gl, at, ft, gt, &ok);
        if (!ok) return al - 0.5 * (al - at) * gl / (gl - (fl - ft) / (al - at));
        const double den = gl - (fl - ft) / (al - at);
        if (fabs(den) < 1e-15) return ac;
        const double aq = al - 0.5 * (al - at) * gl / den;
        return fabs(ac - al) < fabs(aq - al) ? ac : 0.5 * (aq + ac);
    }
    if (gt * gl < 0.0) { /* case 2: slopes of opposite sign */
        const double ac = mt_cubic(al, fl, gl, at, ft, gt, &ok);
        const double as = al - (al - at) / (gl - gt) * gl;
        if (!ok) return as;
        return fabs(ac - at) >= fabs(as - at) ? ac : as;
    }
    if (fabs(gt) <= fabs(gl)) { /* case 3: slope shrinking in magnitude */
        double ac = mt_cubic(al, fl, gl, at, ft, gt, &ok);
        if (!ok) ac = at > al ? at + 0.66 * (au - at) : at - 0.66 * (at - au);
        const double as = fabs(gl - gt) > 1e-15 ? al - (al - at) / (gl - gt) * gl : ac;
        const double an = fabs(ac - at) < fabs(as - at) ? ac : as;
        const double lim = at + 0.66 * (au - at);
        return at > al ? fmin(lim, an) : fmax(lim, an);
    }
    /* case 4: cubic through the trial and the other end */
    const double ac = mt_cubic(au, fu, gu, at, ft, gt, &ok);
    return ok ? ac : 0.5 * (al + au);
}

/* update_interval (more_thuente.rs:196-234); 1 when the interval has shrunk to a point */
static int mt_update(double* al, double* fl, double* gl, double* au, double* fu, double* gu,
                     double at, double ft, double gt) {
    if (ft > *fl) {
        *au = at; *fu = ft; *gu = gt;
        return 0;
    }
    const double side = gt * (*al - at);
    if (side > 0.0) {
        *al = at; *fl = ft; *gl = gt;
        return 0;
    }
    if (side < 0.0) {
        *au = *al; *fu = *fl; *gu = *gl;
        *al = at; *fl = ft; *gl = gt;
        return 0;
    }
    return 1;
}

static double mt_clamp(double a, double lo, double hi) { return a < lo ? lo : (a > hi ? hi : a); }

double or_mt_search(or_mt_fn f, void* ctx, double score0, double deriv0, double initial,
                    double step_min, double step_max, double mu, double nu, int32_t max_iter,
                    int32_t* converged, int32_t* evals) {
    *converged = 0;
    *evals = 0;
    if (deriv0 <= 0.0) return 0.0;
    const double phi0 = -score0, dphi0 = -deriv0;
    double at = mt_clamp(initial, step_min, step_max), sc, dr;
    f(at, ctx, &sc, &dr);
    ++*evals;
    double phi = -sc, dphi = -dr;
    if (step_max - step_min < 0.0) {
        *converged = 1;
        return at;
    }
    double al = 0.0, au = 0.0;  /* both ends at 0, on psi: psi(0) = 0, psi'(0) */
    double fl = phi0 - phi0 - mu * dphi0 * al, fu = phi0 - phi0 - mu * dphi0 * au;
    double gl = dphi0 - mu * dphi0, gu = gl;
    int open = 1;
    double psi = phi - phi0 - mu * dphi0 * at, dpsi = dphi - mu * dphi0;
    for (int it = 0; it < max_iter; ++it) {
        if (psi <= 0.0 && fabs(dphi) <= nu * fabs(dphi0)) {
            *converged = 1;
            return at;
        }
        at = open ? mt_next(al, fl, gl, au, fu, gu, at, psi, dpsi)
                  : mt_next(al, fl, gl, au, fu, gu, at, phi, dphi);
        at = mt_clamp(at, step_min, step_max);
        f(at, ctx, &sc, &dr);
        ++*evals;
        phi = -sc;
        dphi = -dr;
        psi = phi - phi0 - mu * dphi0 * at;
        dpsi = dphi - mu * dphi0;
        if (open && psi <= 0.0 && dpsi >= 0.0) {
            open = 0;
            fl = fl + phi0 - mu * dphi0 * al;
            gl += mu * dphi0;
            fu = fu + phi0 - mu * dphi0 * au;
            gu += mu * dphi0;
        }
        const int done = open ? mt_update(&al, &fl, &gl, &au, &fu, &gu, at, psi, dpsi)
                              : mt_update(&al, &fl, &gl, &au, &fu, &gu, at, phi, dphi);
        if (done) break;
    }
    return at;
}

/* one trial of the CPU path's line search: score and directional derivative at
 * pose + alpha dir (line_search_with_regularization, solver.rs:640-700; regularisation off) */
typedef struct {
    const or_grid* g;
    const float* src;
    size_t n;
    const double* pose;
    const double* dir;
    double d1, d2;
} mt_ctx;

static int mt_eval_cpu(double alpha, void* vctx, double* score, double* deriv) {
    const mt_ctx* c = (const mt_ctx*)vctx;
    double p[6], gr[6], H[36];
    for (int i = 0; i < 6; ++i) p[i] = c->pose[i] + c->dir[i] * alpha;
    int32_t nc;
    or_derivatives_cpu(c->g, c->src, c->n, p, c->d1, c->d2, score, gr, H, &nc);
    double d = 0.0;
    for (int i = 0; i < 6; ++i) d += gr[i] * c->dir[i];
    *deriv = d;
    return 0;
}

static int count_osc(const double* pos, int np) {
    int cnt = 0, best = 0;
    for (int i = 2; i < np; ++i) {
        double cv[3], pv[3];
        for (int a = 0; a < 3; ++a) {
            cv[a] = pos[i * 3 + a] - pos[(i - 1) * 3 + a];
            pv[a] = pos[(i - 1) * 3 + a] - pos[(i - 2) * 3 + a];
        }
        double cn = sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
        double pn = sqrt(pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]);
        if (cn < 1e-10 || pn < 1e-10) {
            cnt = 0;
            continue;
        }
        double cosv = (cv[0] * pv[0] + cv[1] * pv[1] + cv[2] * pv[2]) / (cn * pn);
        if (cosv < -0.9)
            cnt++;
        else
            cnt = 0;
        if (cnt > best) best = cnt;
    }
    return best;
}

static void finish_result(const or_grid* g, const float* src, size_t n, const or_config* cfg,
                          double d1, double d2, or_result* out) {
    double T[12];
    or_pose_to_T34_zyx(out->pose, T);
    out->nvtl = or_nvtl(g, src, n, T, cfg->resolution, d1, d2);
    out->transform_probability = n ? out->score / (double)n : 0.0;
}

/* NdtOptimizer::align, src/ndt_cuda/src/optimization/solver.rs:135-305 (no line search,
 * no GNSS regularisation: the library defaults). */
static void align_cpu_impl(const or_grid* g, const float* src, size_t n,
                           const double* pose_in, const or_config* cfg, or_result* out,
                           double* trace);

void or_align_cpu(const or_grid* g, const float* src, size_t n, const double* pose_in,
                  const or_config* cfg, or_result* out) {
    align_cpu_impl(g, src, n, pose_in, cfg, out, NULL);
}

/* as or_align_cpu, plus a 48-double record per iteration in trace (max_iterations records,
 * the layout of or_align_gpu_sem_trace: it, score, correspondences, pose before the step,
 * gradient, Hessian upper triangle, then the step taken in fields 36-41) */
void or_align_cpu_trace(const or_grid* g, const float* src, size_t n, const double* pose_in,
                        const or_config* cfg, or_result* out, double* trace) {
    align_cpu_impl(g, src, n, pose_in, cfg, out, trace);
}

static void align_cpu_impl(const or_grid* g, const float* src, size_t n,
                           const double* pose_in, const or_config* cfg, or_result* out,
                           double* trace) {
    double d1, d2;
    or_gauss_params(cfg->resolution, cfg->outlier_ratio, &d1, &d2);
    memset(out, 0, sizeof *out);
    double pose[6], best_pose[6], last_H[36];
    memcpy(pose, pose_in, sizeof pose);
    memcpy(best_pose, pose_in, sizeof best_pose);
    memset(last_H, 0, sizeof last_H);
    double best_score = -INFINITY;
    int last_corr = 0;
    int maxit = cfg->max_iterations;
    double* hist = (double*)malloc(sizeof(double) * 3 * (size_t)(maxit + 2));
    int nh = 0;
    memcpy(hist, pose_in, 3 * sizeof(double));
    nh = 1;
    for (int it = 0; it < maxit; ++it) {
        double sc, gr[6], H[36];
        int32_t nc;
        or_derivatives_cpu(g, src, n, pose, d1, d2, &sc, gr, H, &nc);
        double* tr = trace ? trace + 48 * (size_t)it : NULL;
        if (tr) {
            tr[0] = it;
            tr[1] = sc;
            tr[2] = nc;
            for (int i = 0; i < 6; ++i) {
                tr[3 + i] = pose[i];
                tr[9 + i] = gr[i];
            }
            int u = 0;
            for (int i = 0; i < 6; ++i)
                for (int j = i; j < 6; ++j) tr[15 + u++] = H[i * 6 + j];
        }
        if (nc < cfg->min_correspondences) {
            if (it == 0) {
                memcpy(out->pose, pose_in, sizeof out->pose);
                out->status = 2;
                free(hist);
                return;
            }
            break;
        }
        last_corr = nc;
        memcpy(last_H, H, sizeof last_H);
        if (sc > best_score) {
            best_score = sc;
            memcpy(best_pose, pose, sizeof best_pose);
        }
        double dx[6];
        if (!or_newton_step_nd(gr, H, -1e-3, 1e-10, dx)) {
            memcpy(out->pose, best_pose, sizeof out->pose);
            out->status = 3;
            out->score = best_score;
            out->iterations = it;
            memcpy(out->hessian, last_H, sizeof last_H);
            out->num_correspondences = last_corr;
            out->oscillation_count = count_osc(hist, nh);
            finish_result(g, src, n, cfg, d1, d2, out);
            free(hist);
            return;
        }
        double dn = 0.0;
        for (int i = 0; i < 6; ++i) dn += dx[i] * dx[i];
        dn = sqrt(dn);
        if (dn < cfg->trans_epsilon) {
            memcpy(out->pose, pose, sizeof out->pose);
            out->status = 0;
            out->converged = 1;
            out->score = sc;
            out->iterations = it + 1;
            memcpy(out->hessian, H, sizeof out->hessian);
            out->num_correspondences = nc;
            out->oscillation_count = count_osc(hist, nh);
            finish_result(g, src, n, cfg, d1, d2, out);
            free(hist);
            return;
        }
        double dir[6], gd = 0.0;
        for (int i = 0; i < 6; ++i) {
            dir[i] = dx[i] / dn;
            gd += gr[i] * dir[i];
        }
        if (gd <= 0.0)
            for (int i = 0; i < 6; ++i) dir[i] = -dir[i];
        double step = dn < cfg->step_size ? dn : cfg->step_size;
        if (cfg->ls_candidates > 0) {
            /* line_search_with_regularization (solver.rs:640-700): More-Thuente from
             * step_size with MoreThuenteConfig::default(); step_max when it does not
             * converge, step_size when the direction is not an ascent one */
            double d0 = 0.0;
            for (int i = 0; i < 6; ++i) d0 += gr[i] * dir[i];
            if (d0 <= 0.0) {
                step = cfg->step_size;
            } else {
                mt_ctx c = {g, src, n, pose, dir, d1, d2};
                int32_t conv, ev;
                const double a = or_mt_search(mt_eval_cpu, &c, sc, d0, cfg->step_size,
                                              MT_STEP_MIN, MT_STEP_MAX, cfg->ls_mu, cfg->ls_nu,
                                              MT_MAX_ITER, &conv, &ev);
                step = conv ? a : MT_STEP_MAX;
            }
        }
        for (int i = 0; i < 6; ++i) pose[i] += dir[i] * step;
        if (tr)
            for (int i = 0; i < 6; ++i) tr[36 + i] = dir[i] * step;
        memcpy(hist + 3 * nh, pose, 3 * sizeof(double));
        nh++;
    }
    memcpy(out->pose, best_pose, sizeof out->pose);
    out->status = 1;
    out->score = best_score;
    out->iterations = maxit;
    memcpy(out->hessian, last_H, sizeof last_H);
    out->num_correspondences = last_corr;
    out->oscillation_count = count_osc(hist, nh);
    finish_result(g, src, n, cfg, d1, d2, out);
    free(hist);
}

/* Graph-kernel path: K1 init (ndt_graph_kernels.cu:113-154), per iteration K2 compute
 * (:163-302), K3 solve without line search (:311-463), K5 update (:618-847), driven by
 * FullGpuPipelineV2::optimize (full_gpu_pipeline_v2.rs:487-669) and assembled by
 * NdtOptimizer::align_full_gpu (solver.rs:328-441). */
static void align_gpu_sem_impl(const or_grid* g, const float* src, size_t n,
                               const double* pose_in, const or_config* cfg, or_result* out,
                               double* trace);

void or_align_gpu_sem(const or_grid* g, const float* src, size_t n, const double* pose_in,
                      const or_config* cfg, or_result* out) {
    align_gpu_sem_impl(g, src, n, pose_in, cfg, out, NULL);
}

/* same, recording the per-iteration trace (48 doubles per iteration, the layout of the
 * GPU library's ndt_debug_read) */
void or_align_gpu_sem_trace(const or_grid* g, const float* src, size_t n,
                            const double* pose_in, const or_config* cfg, or_result* out,
                            double* trace) {
    align_gpu_sem_impl(g, src, n, pose_in, cfg, out, trace);
}

/* Parallel line search of the graph path (ndt_graph_kernels.cu:388-430 set-up,
 * :473-570 candidate scores and gradients, :626-710 selection): candidates alpha_k =
 * 0.618^k (an f32 product chain) along the reversed-if-needed Newton direction dl, each
 * scored with the graph neighbour rule at pose + alpha_k dl; the first candidate meeting the
 * strong Wolfe conditions (phi_k >= phi0 + mu alpha_k dphi0 and |dphi_k| <= nu |dphi0|) wins,
 * else the highest phi_k above phi0, else alpha = 0. No step clamp applies. Updates pose and
 * returns the step length alpha |dl|. */
static double line_search_gpu_sem(const or_grid* g, const float* src, size_t n, double* pose,
                                  const double* dl, double phi0, double dphi0, double dn,
                                  double d1, double d2, const or_config* cfg) {
    int nc = cfg->ls_candidates < 8 ? cfg->ls_candidates : 8;
    double best_alpha = 0.0, best = phi0;
    float a32 = 1.0f;
    for (int k = 0; k < nc; ++k, a32 *= 0.618f) {
        double a = (double)a32, trial[6], sc, gr[6], H[36];
        int32_t ncorr;
        for (int i = 0; i < 6; ++i) trial[i] = pose[i] + a * dl[i];
        or_derivatives_gpu_sem(g, src, n, trial, d1, d2, cfg->max_neighbors, &sc, gr, H, &ncorr);
        double dphi = 0.0;
        for (int i = 0; i < 6; ++i) dphi += gr[i] * dl[i];
        int armijo = sc >= phi0 + cfg->ls_mu * a * dphi0;
        int curvature = fabs(dphi) <= cfg->ls_nu * fabs(dphi0);
        if (armijo && curvature) {
            best_alpha = a;
            break;
        }
        if (sc > best) {
            best = sc;
            best_alpha = a;
        }
    }
    for (int i = 0; i < 6; ++i) pose[i] += best_alpha * dl[i];
    return best_alpha * dn;
}

static void align_gpu_sem_impl(const or_grid* g, const float* src, size_t n,
                               const double* pose_in, const or_config* cfg, or_result* out,
                               double* trace) {
    double d1, d2;
    or_gauss_params(cfg->resolution, cfg->outlier_ratio, &d1, &d2);
    memset(out, 0, sizeof *out);
    double pose[6];
    memcpy(pose, pose_in, sizeof pose);
    double prev[3] = {pose[0], pose[1], pose[2]}, prev2[3] = {pose[0], pose[1], pose[2]};
    int osc = 0, max_osc = 0;
    double eps = (double)sqrtf((float)cfg->trans_epsilon * (float)cfg->trans_epsilon);
    int maxit = cfg->max_iterations;
    for (int it = 0; it < maxit; ++it) {
        double sc, gr[6], H[36];
        int32_t nc;
        or_derivatives_gpu_sem(g, src, n, pose, d1, d2, cfg->max_neighbors, &sc, gr, H, &nc);
        double dl[6];
        int solved = or_jacobi_svd_solve(H, gr, dl);
        if (trace) {
            double* t = trace + (size_t)it * 48;
            t[0] = it;
            t[1] = sc;
            t[2] = nc;
            int u = 0;
            for (int i = 0; i < 6; ++i) {
                t[3 + i] = pose[i];
                t[9 + i] = gr[i];
                t[36 + i] = dl[i];
                for (int j = i; j < 6; ++j) t[15 + u++] = H[i * 6 + j];
            }
            t[42] = 1.0;
            t[43] = solved;
            t[44] = t[45] = t[46] = t[47] = 0.0;
        }
        if (!solved)
            for (int i = 0; i < 6; ++i) dl[i] = -gr[i] * 1e-4;
        double dphi = 0.0;
        for (int i = 0; i < 6; ++i) dphi += gr[i] * dl[i];
        if (dphi <= 0.0) {
            for (int i = 0; i < 6; ++i) dl[i] = -dl[i];
            dphi = -dphi;
        }
        double dn = 0.0;
        for (int i = 0; i < 6; ++i) dn += dl[i] * dl[i];
        dn = sqrt(dn);
        double step;
        if (cfg->ls_candidates > 0) {
            step = line_search_gpu_sem(g, src, n, pose, dl, sc, dphi, dn, d1, d2, cfg);
        } else {
            step = dn > cfg->step_size ? cfg->step_size : dn;
            double scale = dn > 1e-10 ? step / dn : 0.0;
            for (int i = 0; i < 6; ++i) pose[i] += scale * dl[i];
        }
        if (it >= 1) {
            double cv[3], pv[3];
            for (int a = 0; a < 3; ++a) {
                cv[a] = pose[a] - prev[a];
                pv[a] = prev[a] - prev2[a];
            }
            double cn = sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
            double pn = sqrt(pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]);
            if (cn > 1e-10 && pn > 1e-10) {
                double cosv = (cv[0] * pv[0] + cv[1] * pv[1] + cv[2] * pv[2]) / (cn * pn);
                osc = cosv < -0.9 ? osc + 1 : 0;
                if (osc > max_osc) max_osc = osc;
            } else {
                osc = 0;
            }
        }
        for (int a = 0; a < 3; ++a) {
            prev2[a] = prev[a];
            prev[a] = pose[a];
        }
        int conv = step < eps;
        if (conv || it + 1 >= maxit) {
            memcpy(out->pose, pose, sizeof out->pose);
            out->iterations = it + 1;
            out->converged = conv;
            out->score = sc;
            memcpy(out->hessian, H, sizeof out->hessian);
            out->num_correspondences = nc;
            out->oscillation_count = max_osc;
            break;
        }
    }
    if (out->num_correspondences == 0) {
        out->status = 2;
        out->converged = 0;
    } else {
        out->status = out->converged ? 0 : 1;
    }
    finish_result(g, src, n, cfg, d1, d2, out);
}

void or_align_batch(const or_grid* g, const float* const* srcs, const size_t* ns,
                    const double* poses_in, size_t m, const or_config* cfg, int semantics,
                    int nthreads, or_result* out) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
    for (long i = 0; i < (long)m; ++i) {
        if (semantics == 0)
            or_align_gpu_sem(g, srcs[i], ns[i], poses_in + 6 * i, cfg, out + i);
        else
            or_align_cpu(g, srcs[i], ns[i], poses_in + 6 * i, cfg, out + i);
    }
}
