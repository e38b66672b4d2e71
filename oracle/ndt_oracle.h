/*
 * ndt_oracle.h — CPU restatement of cuda_ndt_matcher's NDT scan-matching path.
 *
 * TEST INFRASTRUCTURE ONLY. Nothing in the product links this code; only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference legs load it,
 * and only as the oracle (or as the timed CPU baseline), never as the thing measured
 * on the GPU.
 *
 * Parity status: pinned against the reference's own known-answer tests (voxel
 * coordinates, Morton round trips, radix sort, segment detection, Newton steps on
 * diagonal Hessians, Gaussian parameter signs, covariance regularisation, the
 * More-Thuente unit tests) through tests/golden/, tests/test_oracle_golden.py and
 * tests/test_capi_cpu.py. The graph semantics are also compared end to end with the
 * reference's own CUDA kernels, compiled from its sources (oracle/ref_graph.c,
 * tests/test_gpu_reference_kernels.py): this restatement sits as close to them as the
 * reference's FP32 arithmetic allows. The reference's Rust CPU path cannot be built here
 * (no cargo), so the CPU semantics are pinned by the component vectors plus
 * finite-difference derivative checks.
 *
 * Two Newton semantics are restated (they disagree in the reference itself):
 *   - "cpu"  : NdtOptimizer::align (src/ndt_cuda/src/optimization/solver.rs:135-305)
 *   - "gpu"  : the graph kernels K1-K5 (src/cuda_ffi/csrc/ndt_graph_kernels.cu:113-847)
 *              driven by FullGpuPipelineV2::optimize
 *              (src/ndt_cuda/src/optimization/full_gpu_pipeline_v2.rs:487-669),
 *              restated in FP64.
 */
#ifndef NDT_ORACLE_H
#define NDT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_grid or_grid;

typedef struct {
    double pose[6];               /* x, y, z, roll, pitch, yaw; R = Rx*Ry*Rz */
    double score;
    double transform_probability;
    double nvtl;
    double hessian[36];
    int32_t converged;
    int32_t iterations;
    int32_t num_correspondences;
    int32_t oscillation_count;
    int32_t status;               /* 0 converged, 1 max-iter, 2 no-corr, 3 singular */
    int32_t pad;
} or_result;

typedef struct {
    double resolution;
    int32_t max_iterations;
    int32_t max_neighbors;        /* 8 for the graph-kernel semantics */
    double trans_epsilon;
    double step_size;
    double outlier_ratio;
    int32_t min_correspondences;  /* 10 in OptimizationConfig::default() */
    int32_t ls_candidates;        /* line search: 0 off. Graph path: candidates (<= 8);
                                     CPU path: any value > 0 turns on the More-Thuente
                                     search (MoreThuenteConfig::default: step in
                                     [1e-9, 0.1], at most 10 iterations) */
    double ls_mu;                 /* Armijo constant (PipelineV2Config::armijo_mu, 1e-4) */
    double ls_nu;                 /* curvature constant (PipelineV2Config::wolfe_nu, 0.9) */
} or_config;

/* More-Thuente line search (more_thuente.rs:236-410): maximises score(alpha) along a
 * direction from score0 with slope deriv0 > 0, first trial `initial` clamped to
 * [step_min, step_max]. f(alpha, ctx, &score, &deriv) evaluates a trial and returns 0.
 * Returns the step; *converged: the strong Wolfe conditions held at it; *evals: trials. */
typedef int (*or_mt_fn)(double alpha, void* ctx, double* score, double* deriv);
double or_mt_search(or_mt_fn f, void* ctx, double score0, double deriv0, double initial,
                    double step_min, double step_max, double mu, double nu, int32_t max_iter,
                    int32_t* converged, int32_t* evals);

/* derivatives/types.rs:61-75 */
void or_gauss_params(double resolution, double outlier_ratio, double* d1, double* d2);

/* voxel_grid/types.rs:206-212 */
void or_voxel_coord(const float* p, float resolution, int32_t* out3);

/* voxel_grid/gpu/morton.rs:284-326 */
uint64_t or_morton_encode(uint32_t x, uint32_t y, uint32_t z);
void or_morton_decode(uint64_t code, uint32_t* x, uint32_t* y, uint32_t* z);
/* voxel_grid/gpu/morton.rs:197-281 (reference builder rule: aligned-min origin) */
void or_morton_codes_ref(const float* pts, size_t n, float resolution, uint64_t* codes,
                         float* grid_min3);
/* the library's rule: key = morton(voxel_coord - min voxel_coord) */
int or_morton_codes_coord(const float* pts, size_t n, float resolution, uint64_t* codes,
                          int32_t* min_coord3);

/* voxel_grid/gpu/radix_sort.rs:97-160 (stable LSD, 4-bit digits, 16 passes) */
void or_radix_sort_pairs(uint64_t* keys, uint32_t* vals, size_t n);

/* voxel_grid/gpu/segments.rs:45-89; returns the number of segments */
size_t or_detect_segments(const uint64_t* sorted, size_t n, uint32_t* seg_ids,
                          uint32_t* seg_starts);

/* voxel grid (voxel_grid/cpu.rs:51-75, voxel_grid/types.rs:54-190).
 * centered = 0: the reference's uncentred FP64 sums; 1: two-pass centred FP64 moments.
 * Voxels are returned in ascending order of their coordinate Morton key. */
or_grid* or_grid_build(const float* pts, size_t n, float resolution, int min_points,
                       float ratio, int centered);
void or_grid_free(or_grid* g);
size_t or_grid_size(const or_grid* g);
void or_grid_copy(const or_grid* g, int32_t* coords, float* means, float* covs, float* icovs,
                  uint32_t* counts, float* paxes);
uint32_t or_grid_hash_capacity(const or_grid* g);

/* reference hash semantics (src/cuda_ffi/csrc/voxel_hash.cu:33-58, 218-228) */
int64_t or_pack_key(int32_t gx, int32_t gy, int32_t gz);
uint32_t or_hash_slot(int64_t key, uint32_t capacity);
int32_t or_grid_lookup(const or_grid* g, int32_t gx, int32_t gy, int32_t gz);

/* 27-cell query, graph-kernel semantics in f32 (src/cuda_ffi/csrc/ndt_graph_kernels.cu:47-104) */
void or_query_gpu_sem(const or_grid* g, const float* q, size_t n, int max_nb, int32_t* idx,
                      int32_t* cnt);
/* kiddo-equivalent radius search (voxel_grid/search.rs:90-99): all neighbours, nearest first */
int or_radius_search(const or_grid* g, const float* q, float radius, int32_t* idx, int cap);

/* derivatives: CPU path (derivatives/cpu.rs:417-540) and graph-kernel path in FP64 */
void or_derivatives_cpu(const or_grid* g, const float* src, size_t n, const double* pose,
                        double d1, double d2, double* score, double* grad, double* hess,
                        int32_t* ncorr);
void or_derivatives_gpu_sem(const or_grid* g, const float* src, size_t n, const double* pose,
                            double d1, double d2, int max_nb, double* score, double* grad,
                            double* hess, int32_t* ncorr);

/* Newton steps */
int or_newton_step_nd(const double* g, const double* H, double min_eig, double tol, double* x);
int or_jacobi_svd_solve(const double* H, const double* g, double* x);

/* alignment loops */
void or_align_cpu(const or_grid* g, const float* src, size_t n, const double* pose_in,
                  const or_config* cfg, or_result* out);
void or_align_gpu_sem(const or_grid* g, const float* src, size_t n, const double* pose_in,
                      const or_config* cfg, or_result* out);
void or_align_cpu_trace(const or_grid* g, const float* src, size_t n, const double* pose_in,
                        const or_config* cfg, or_result* out, double* trace);
void or_align_gpu_sem_trace(const or_grid* g, const float* src, size_t n,
                            const double* pose_in, const or_config* cfg, or_result* out,
                            double* trace);
/* many alignments on a thread pool (rayon par_iter in the reference, ndt.rs:921) */
void or_align_batch(const or_grid* g, const float* const* srcs, const size_t* ns,
                    const double* poses_in, size_t m, const or_config* cfg, int semantics,
                    int nthreads, or_result* out);

/* scoring (scoring/nvtl.rs:196-260); T = 3x4 row-major world transform */
double or_nvtl(const or_grid* g, const float* src, size_t n, const double* T34,
               double resolution, double d1, double d2);
/* per-pose score / correspondences with graph-kernel neighbour semantics */
void or_score_gpu_sem(const or_grid* g, const float* src, size_t n, const double* T34,
                      double d1, double d2, int max_nb, double* score, int32_t* ncorr);
void or_pose_to_T34_xyz(const double* pose, double* T34);  /* R = Rx*Ry*Rz */
void or_pose_to_T34_zyx(const double* pose, double* T34);  /* nalgebra from_euler_angles */

/* symmetric eigen solvers used above (cyclic Jacobi, FP64) */
void or_eigen_sym3(const double* a9, double* evals3, double* evecs9);
void or_eigen_sym6(const double* a36, double* evals6, double* evecs36);

#ifdef __cplusplus
}
#endif
#endif
