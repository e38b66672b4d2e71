/* ref_graph.c — runs the reference's own graph-path CUDA kernels on the GPU, as a checker.
 *
 * TEST INFRASTRUCTURE, not product code: only tests load it. The kernels are the reference's
 * K1-K5 (src/cuda_ffi/csrc/ndt_graph_kernels.cu:113-847) and its voxel hash build
 * (src/cuda_ffi/csrc/voxel_hash.cu:69-114), compiled unmodified from the reference's sources
 * into device-only cubins (oracle/_ref/*.cubin, made by oracle/build.py). This file is the host
 * side, written here: it loads the cubins through the CUDA driver API and restates the
 * reference's host code for the path:
 *
 *   - GpuVoxelData upload + hash_table_init / hash_table_build
 *     (src/ndt_cuda/src/optimization/full_gpu_pipeline_v2.rs:295-322; capacity rule of
 *     voxel_hash_get_capacity, voxel_hash.cu:218-228; launch shape of voxel_hash_build,
 *     voxel_hash.cu:258-284);
 *   - FullGpuPipelineV2::optimize (full_gpu_pipeline_v2.rs:487-669): zeroed state, reduce,
 *     line-search and output buffers, K1, then per iteration K2, K3, K4 (line search only), K5
 *     (graph_ndt_run_iteration_raw, src/cuda_ffi/src/graph_ndt.rs:493-554) with a device sync
 *     and the convergence flag read after each; launch shapes of ndt_graph_kernels.cu:879-969;
 *   - GraphNdtConfig::new / with_fixed_step / with_line_search
 *     (src/cuda_ffi/src/graph_ndt.rs:104-165).
 *
 * Every buffer the kernels index is allocated with room to spare (256 floats for each of the
 * state, reduce, line-search and output blocks, whose layouts use at most 102), the hash table
 * keeps at least half its slots empty (so every probe loop ends), and debug output is off.
 */
#include <cuda.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

/* GraphNdtConfig (src/cuda_ffi/csrc/ndt_graph_common.cuh:134-160): passed to the kernels by
 * value, so the field order and types must be the reference's. */
typedef struct {
    float gauss_d1, gauss_d2, resolution, epsilon_sq;
    float reg_ref_x, reg_ref_y, reg_scale;
    int32_t reg_enabled;
    int32_t ls_enabled, ls_num_candidates;
    float ls_mu, ls_nu, fixed_step_size;
    uint32_t num_points, num_voxels, hash_capacity;
    int32_t max_iterations;
    int32_t debug_enabled;
} RgConfig;

enum { BLOCK = 256, REDUCE = 29, SLOT_FLOATS = 256, STATE_CONVERGED = 18 };

static struct {
    int open;
    CUcontext ctx;
    CUmodule mk, mh;
    CUfunction k_init, k_compute, k_solve, k_ls, k_update, k_hash, k_query;
    CUdeviceptr means, icov, valid, table, pts, pose, state, reduce, ls, out;
    uint32_t V, cap;
    size_t pts_bytes;
    float res;
} G;

static char g_err[1200];

const char* rg_error(void) { return g_err; }

static int fail(CUresult r, const char* what) {
    const char* s = NULL;
    cuGetErrorString(r, &s);
    snprintf(g_err, sizeof g_err, "%s: %s (%d)", what, s ? s : "?", (int)r);
    return (int)r;
}

#define CK(call, what)                          \
    do {                                        \
        CUresult r_ = (call);                   \
        if (r_ != CUDA_SUCCESS) return fail(r_, what); \
    } while (0)

static int load(CUmodule* m, const char* dir, const char* name) {
    char path[1024];  /* the message adds at most 100 bytes to it */
    snprintf(path, sizeof path, "%s/%s", dir, name);
    CK(cuModuleLoad(m, path), path);
    return 0;
}

/* Loads the cubins of directory dir on device 0's primary context (the one the CUDA runtime
 * uses) and allocates the fixed-size state blocks. */
int rg_open(const char* dir) {
    if (G.open) return 0;
    CUdevice dev;
    CK(cuInit(0), "cuInit");
    CK(cuDeviceGet(&dev, 0), "cuDeviceGet");
    CK(cuDevicePrimaryCtxRetain(&G.ctx, dev), "cuDevicePrimaryCtxRetain");
    CK(cuCtxSetCurrent(G.ctx), "cuCtxSetCurrent");
    int rc;
    if ((rc = load(&G.mk, dir, "ndt_graph_kernels.cubin"))) return rc;
    if ((rc = load(&G.mh, dir, "voxel_hash.cubin"))) return rc;
    CK(cuModuleGetFunction(&G.k_init, G.mk, "ndt_graph_init_kernel"), "K1");
    CK(cuModuleGetFunction(&G.k_compute, G.mk, "ndt_graph_compute_kernel"), "K2");
    CK(cuModuleGetFunction(&G.k_solve, G.mk, "ndt_graph_solve_kernel"), "K3");
    CK(cuModuleGetFunction(&G.k_ls, G.mk, "ndt_graph_linesearch_kernel"), "K4");
    CK(cuModuleGetFunction(&G.k_update, G.mk, "ndt_graph_update_kernel"), "K5");
    CK(cuModuleGetFunction(&G.k_hash, G.mh, "voxel_hash_build_kernel"), "hash build");
    CK(cuModuleGetFunction(&G.k_query, G.mh, "voxel_hash_query_kernel"), "hash query");
    CK(cuMemAlloc(&G.pose, SLOT_FLOATS * 4), "alloc");
    CK(cuMemAlloc(&G.state, SLOT_FLOATS * 4), "alloc");
    CK(cuMemAlloc(&G.reduce, SLOT_FLOATS * 4), "alloc");
    CK(cuMemAlloc(&G.ls, SLOT_FLOATS * 4), "alloc");
    CK(cuMemAlloc(&G.out, SLOT_FLOATS * 4), "alloc");
    G.open = 1;
    return 0;
}

static void free_map(void) {
    CUdeviceptr* b[] = {&G.means, &G.icov, &G.valid, &G.table};
    for (int i = 0; i < 4; ++i)
        if (*b[i]) {
            cuMemFree(*b[i]);
            *b[i] = 0;
        }
    G.V = G.cap = 0;
}

/* The voxel map: V means (xyz, f32) and inverse covariances (row-major 3x3, f32), all valid;
 * then the reference's hash table built from the means by its own kernel. */
int rg_set_map(const float* means, const float* icov, uint32_t V, float resolution) {
    if (!G.open) {
        snprintf(g_err, sizeof g_err, "rg_open first");
        return -1;
    }
    if (V == 0 || V > (1u << 30)) {
        snprintf(g_err, sizeof g_err, "voxel count %u out of range", V);
        return -1;
    }
    free_map();
    uint32_t cap = 1;
    while (cap < 2 * V) cap *= 2; /* voxel_hash_get_capacity: power of two >= 2V */
    CK(cuMemAlloc(&G.means, (size_t)V * 12), "alloc means");
    CK(cuMemAlloc(&G.icov, (size_t)V * 36), "alloc icov");
    CK(cuMemAlloc(&G.valid, (size_t)V * 4), "alloc valid");
    CK(cuMemAlloc(&G.table, (size_t)cap * 16), "alloc table");
    CK(cuMemcpyHtoD(G.means, means, (size_t)V * 12), "copy means");
    CK(cuMemcpyHtoD(G.icov, icov, (size_t)V * 36), "copy icov");
    CK(cuMemsetD32(G.valid, 1u, V), "valid");
    CK(cuMemsetD8(G.table, 0xFF, (size_t)cap * 16), "hash init");
    float inv_res = 1.0f / resolution;
    void* args[] = {&G.means, &G.valid, &V, &inv_res, &G.table, &cap};
    CK(cuLaunchKernel(G.k_hash, (V + BLOCK - 1) / BLOCK, 1, 1, BLOCK, 1, 1, 0, NULL, args, NULL),
       "hash build launch");
    CK(cuCtxSynchronize(), "hash build");
    G.V = V;
    G.cap = cap;
    G.res = resolution;
    return 0;
}

/* One alignment of n points from pose_in. out48 receives the reference's output block
 * (OutputOffset, ndt_graph_common.cuh:90-101): pose[6], iterations, converged, score,
 * Hessian[36], correspondences, max oscillation count, mean step. With debug non-null, K5's
 * own per-iteration record (DebugOffset, ndt_graph_common.cuh:107-121: 50 floats per
 * iteration, max_iter records) is enabled and copied there. */
int rg_align(const float* pts, uint32_t n, const double pose_in[6], float d1, float d2,
             double trans_epsilon, int32_t max_iter, int32_t line_search, float step_size,
             float ls_mu, float ls_nu, float* out48, float* debug) {
    if (!G.open || G.V == 0) {
        snprintf(g_err, sizeof g_err, "rg_open and rg_set_map first");
        return -1;
    }
    memset(out48, 0, 48 * sizeof(float));
    if (n == 0) { /* optimize(): initial pose, converged, no iterations */
        for (int i = 0; i < 6; ++i) out48[i] = (float)pose_in[i];
        out48[7] = 1.0f;
        return 0;
    }
    if ((size_t)n * 12 > G.pts_bytes) {
        if (G.pts) cuMemFree(G.pts);
        G.pts = 0;
        G.pts_bytes = 0;
        CK(cuMemAlloc(&G.pts, (size_t)n * 12), "alloc points");
        G.pts_bytes = (size_t)n * 12;
    }
    CK(cuMemcpyHtoD(G.pts, pts, (size_t)n * 12), "copy points");
    float pose_f[6];
    for (int i = 0; i < 6; ++i) pose_f[i] = (float)pose_in[i];
    CK(cuMemcpyHtoD(G.pose, pose_f, sizeof pose_f), "copy pose");
    CUdeviceptr blocks[] = {G.state, G.reduce, G.ls, G.out};
    for (int i = 0; i < 4; ++i) CK(cuMemsetD32(blocks[i], 0u, SLOT_FLOATS), "zero state");

    RgConfig cfg;
    memset(&cfg, 0, sizeof cfg);
    const float eps = (float)trans_epsilon;
    cfg.gauss_d1 = d1;
    cfg.gauss_d2 = d2;
    cfg.resolution = G.res;
    cfg.epsilon_sq = eps * eps;
    cfg.ls_enabled = line_search ? 1 : 0;
    cfg.ls_num_candidates = 8;
    cfg.ls_mu = ls_mu;
    cfg.ls_nu = ls_nu;
    cfg.fixed_step_size = line_search ? 0.1f : step_size;
    cfg.num_points = n;
    cfg.num_voxels = G.V;
    cfg.hash_capacity = G.cap;
    cfg.max_iterations = max_iter;
    cfg.debug_enabled = debug ? 1 : 0;

    /* K5 writes record `iteration` (< max_iter) of 50 floats when enabled */
    CUdeviceptr no_debug = 0;
    if (debug && max_iter > 0)
        CK(cuMemAlloc(&no_debug, (size_t)max_iter * 50 * sizeof(float)), "alloc debug");
    const unsigned grid = (n + BLOCK - 1) / BLOCK;
    void* a_init[] = {&G.pose, &G.state, &G.reduce, &G.ls};
    void* a_compute[] = {&G.pts, &G.means, &G.icov, &G.table, &cfg, &G.state, &G.reduce};
    void* a_solve[] = {&cfg, &G.state, &G.reduce, &G.ls, &G.out};
    void* a_ls[] = {&G.pts, &G.means, &G.icov, &G.table, &cfg, &G.state, &G.ls};
    void* a_update[] = {&cfg, &G.state, &G.reduce, &G.ls, &G.out, &no_debug};
    CK(cuLaunchKernel(G.k_init, 1, 1, 1, 1, 1, 1, 0, NULL, a_init, NULL), "K1");
    CK(cuCtxSynchronize(), "K1");
    for (int32_t it = 0; it < max_iter; ++it) {
        CK(cuLaunchKernel(G.k_compute, grid, 1, 1, BLOCK, 1, 1, BLOCK * REDUCE * 4, NULL,
                          a_compute, NULL), "K2");
        CK(cuLaunchKernel(G.k_solve, 1, 1, 1, 1, 1, 1, 0, NULL, a_solve, NULL), "K3");
        if (line_search)
            CK(cuLaunchKernel(G.k_ls, grid, 1, 1, BLOCK, 1, 1, BLOCK * 8 * 4, NULL, a_ls, NULL),
               "K4");
        CK(cuLaunchKernel(G.k_update, 1, 1, 1, 1, 1, 1, 0, NULL, a_update, NULL), "K5");
        CK(cuCtxSynchronize(), "iteration");
        float conv = 0.f;
        CK(cuMemcpyDtoH(&conv, G.state + STATE_CONVERGED * 4, 4), "converged flag");
        if (conv > 0.5f) break;
    }
    CK(cuMemcpyDtoH(out48, G.out, 48 * sizeof(float)), "output");
    if (no_debug) {
        CK(cuMemcpyDtoH(debug, no_debug, (size_t)max_iter * 50 * sizeof(float)), "debug");
        cuMemFree(no_debug);
    }
    return 0;
}

/* The reference's K2 alone at one pose (K1 from pose_in, then one compute launch): red29
 * receives its reduce block (ReduceOffset, ndt_graph_common.cuh:51-59): score, gradient[6],
 * Hessian upper triangle[21], correspondences, all FP32 atomic sums. */
int rg_eval(const float* pts, uint32_t n, const double pose_in[6], float d1, float d2,
            float* red29) {
    if (!G.open || G.V == 0 || n == 0) {
        snprintf(g_err, sizeof g_err, "rg_open, rg_set_map and points first");
        return -1;
    }
    if ((size_t)n * 12 > G.pts_bytes) {
        if (G.pts) cuMemFree(G.pts);
        G.pts = 0;
        G.pts_bytes = 0;
        CK(cuMemAlloc(&G.pts, (size_t)n * 12), "alloc points");
        G.pts_bytes = (size_t)n * 12;
    }
    CK(cuMemcpyHtoD(G.pts, pts, (size_t)n * 12), "copy points");
    float pose_f[6];
    for (int i = 0; i < 6; ++i) pose_f[i] = (float)pose_in[i];
    CK(cuMemcpyHtoD(G.pose, pose_f, sizeof pose_f), "copy pose");
    CUdeviceptr blocks[] = {G.state, G.reduce, G.ls, G.out};
    for (int i = 0; i < 4; ++i) CK(cuMemsetD32(blocks[i], 0u, SLOT_FLOATS), "zero state");
    RgConfig cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gauss_d1 = d1;
    cfg.gauss_d2 = d2;
    cfg.resolution = G.res;
    cfg.ls_num_candidates = 8;
    cfg.fixed_step_size = 0.1f;
    cfg.num_points = n;
    cfg.num_voxels = G.V;
    cfg.hash_capacity = G.cap;
    cfg.max_iterations = 1;
    void* a_init[] = {&G.pose, &G.state, &G.reduce, &G.ls};
    void* a_compute[] = {&G.pts, &G.means, &G.icov, &G.table, &cfg, &G.state, &G.reduce};
    CK(cuLaunchKernel(G.k_init, 1, 1, 1, 1, 1, 1, 0, NULL, a_init, NULL), "K1");
    CK(cuLaunchKernel(G.k_compute, (n + BLOCK - 1) / BLOCK, 1, 1, BLOCK, 1, 1,
                      BLOCK * REDUCE * 4, NULL, a_compute, NULL), "K2");
    CK(cuCtxSynchronize(), "K2");
    CK(cuMemcpyDtoH(red29, G.reduce, REDUCE * sizeof(float)), "reduce block");
    return 0;
}

/* Neighbours of n query points by the reference's voxel_hash_query_kernel
 * (voxel_hash.cu:136-210, launch shape of voxel_hash_query, :299-332; search radius = the
 * resolution): idx receives n x 8 voxel indices (-1 padded), cnt the counts. */
int rg_query(const float* q, uint32_t n, int32_t* idx, uint32_t* cnt) {
    if (!G.open || G.V == 0) {
        snprintf(g_err, sizeof g_err, "rg_open and rg_set_map first");
        return -1;
    }
    if (n == 0) return 0;
    CUdeviceptr dq = 0, di = 0, dc = 0;
    int rc = 0;
    CUresult r = cuMemAlloc(&dq, (size_t)n * 12);
    if (r == CUDA_SUCCESS) r = cuMemAlloc(&di, (size_t)n * 8 * 4);
    if (r == CUDA_SUCCESS) r = cuMemAlloc(&dc, (size_t)n * 4);
    if (r == CUDA_SUCCESS) r = cuMemcpyHtoD(dq, q, (size_t)n * 12);
    if (r == CUDA_SUCCESS) {
        float inv_res = 1.0f / G.res, radius_sq = G.res * G.res;
        void* args[] = {&dq, &G.means, &n, &inv_res, &radius_sq, &G.table, &G.cap, &di, &dc};
        r = cuLaunchKernel(G.k_query, (n + BLOCK - 1) / BLOCK, 1, 1, BLOCK, 1, 1, 0, NULL, args,
                           NULL);
    }
    if (r == CUDA_SUCCESS) r = cuCtxSynchronize();
    if (r == CUDA_SUCCESS) r = cuMemcpyDtoH(idx, di, (size_t)n * 8 * 4);
    if (r == CUDA_SUCCESS) r = cuMemcpyDtoH(cnt, dc, (size_t)n * 4);
    if (r != CUDA_SUCCESS) rc = fail(r, "hash query");
    if (dq) cuMemFree(dq);
    if (di) cuMemFree(di);
    if (dc) cuMemFree(dc);
    return rc;
}

void rg_close(void) {
    if (!G.open) return;
    free_map();
    CUdeviceptr* b[] = {&G.pts, &G.pose, &G.state, &G.reduce, &G.ls, &G.out};
    for (int i = 0; i < 6; ++i)
        if (*b[i]) {
            cuMemFree(*b[i]);
            *b[i] = 0;
        }
    G.pts_bytes = 0;
    cuModuleUnload(G.mk);
    cuModuleUnload(G.mh);
    CUdevice dev;
    if (cuDeviceGet(&dev, 0) == CUDA_SUCCESS) cuDevicePrimaryCtxRelease(dev);
    G.open = 0;
}
