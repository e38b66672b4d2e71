/*
 * ndt_gb300.h — C ABI of the GB300-native NDT scan-matching library (libndt_gb300.so).
 *
 * Drop-in boundary for the hot path of cuda_ndt_matcher: the `ndt_cuda` crate's
 * NdtScanMatcher (src/ndt_cuda/src/ndt.rs:255-1321) calls these functions in place of its
 * CubeCL pipelines and the `cuda_ffi` kernels (src/cuda_ffi/csrc/). Conventions:
 *   - every function returns int: 0 = NDT_OK, negative = NDT_ERR_*, positive = a
 *     cudaError_t passed through from the CUDA runtime (the reference's `CudaError` codes,
 *     src/cuda_ffi/src/radix_sort.rs:59-95);
 *   - no exceptions cross the ABI; ndt_last_error_string() describes the last failure of
 *     the calling thread;
 *   - the caller owns host arrays; a context owns every device buffer and its CUDA stream,
 *     grows capacities monotonically and allocates nothing on the alignment path once
 *     warmed up;
 *   - a context is single-threaded (the reference serialises a matcher behind a Mutex,
 *     src/cuda_ndt_matcher/src/main.rs:951); several contexts may share one device.
 *
 * Poses are 6-vectors [x, y, z, roll, pitch, yaw] with R = Rx(roll)*Ry(pitch)*Rz(yaw), the
 * convention of the reference's derivative kernels
 * (src/cuda_ffi/csrc/persistent_ndt_device.cuh:38-71). Converting an Isometry3 with
 * nalgebra's euler angles (src/ndt_cuda/src/optimization/types.rs:156-174) is the host
 * binding's job, as in the reference.
 */
#ifndef NDT_GB300_H
#define NDT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NDT_OK 0
#define NDT_ERR_INVALID_ARGUMENT (-1)
#define NDT_ERR_NO_TARGET (-2)      /* "No target set. Call set_target() first." */
#define NDT_ERR_EMPTY_INPUT (-3)    /* "Target/Source point cloud is empty" */
#define NDT_ERR_NO_VOXELS (-4)      /* "No voxels created from target points (too sparse?)" */
#define NDT_ERR_RANGE (-5)          /* map extent exceeds the voxel key range */
#define NDT_ERR_HASH_FULL (-6)      /* device: hash insert found no free slot */
#define NDT_ERR_PROBE_LIMIT (-7)    /* device: a probe sequence exceeded its bound */
#define NDT_ERR_DEVICE (-8)         /* device: other status reported by a kernel */
#define NDT_ERR_NO_DEVICE (-9)      /* no CUDA device with compute capability 10.3 */
#define NDT_ERR_CAPACITY (-10)      /* a size exceeds a fixed limit of the entry point */

#define NDT_SEMANTICS_GPU_GRAPH 0   /* align_gpu: graph kernels K1-K5 */
#define NDT_SEMANTICS_CPU 1         /* align with use_gpu = false: NdtOptimizer::align */

/* Cell lookup of the search kernels. Both give the same voxel for a cell (one voxel per
 * cell); they differ in cost. The hash table (the reference's structure, voxel_hash.cu) is
 * always built. The dense index is an array over the map's cell bounding box, 16 bytes per
 * cell {centroid, slot}, built when it takes at most 4 GiB (the 2 x 2 km map at 1 m takes
 * 2.2 GiB): a lookup is one load. */
#define NDT_CELL_INDEX_AUTO 0       /* dense index when it fits, else the hash */
#define NDT_CELL_INDEX_HASH 1       /* hash probing only */
#define NDT_CELL_INDEX_OCTANT 2     /* dense index with a neighbourhood mask per octant of each
                                       cell whenever grid and masks fit the dense budget: AUTO
                                       keeps one mask per cell beyond 256 MiB of masks; this
                                       trades build time and memory on large maps for faster
                                       searches (same results bit for bit) */

#define NDT_STATUS_CONVERGED 0
#define NDT_STATUS_MAX_ITERATIONS 1
#define NDT_STATUS_NO_CORRESPONDENCES 2
#define NDT_STATUS_SINGULAR_HESSIAN 3

/* NdtScanMatcherConfig (src/ndt_cuda/src/ndt.rs:41-107) plus device tuning knobs. */
typedef struct ndt_config {
    float resolution;              /* 2.0 m */
    int32_t max_iterations;        /* 30 */
    double trans_epsilon;          /* 0.01 */
    double step_size;              /* 0.1, maximum step length */
    double outlier_ratio;          /* 0.55 */
    int32_t min_points_per_voxel;  /* 6 */
    float eigenvalue_ratio;        /* 0.01 (VoxelGridConfig::eigenvalue_ratio_threshold) */
    int32_t max_neighbors;         /* 8: graph-kernel truncation (ndt_graph_common.cuh:21) */
    int32_t semantics;             /* NDT_SEMANTICS_* */
    int32_t min_correspondences;   /* 10 (OptimizationConfig, solver.rs:58); CPU semantics */
    int32_t device;                /* CUDA device ordinal */
    int32_t cluster_size;          /* CTAs per alignment; 0 = autotuned */
    int32_t threads_per_cta;       /* 0 = autotuned */
    int32_t hash_capacity_factor;  /* capacity = next pow2 >= factor * V; 2 = reference */
    int32_t max_registers;         /* Newton-kernel register cap (64, 80 or 128; 48 also at
                                      256 threads; 128 only at 512); 0 = autotuned */
    int32_t cell_index;            /* NDT_CELL_INDEX_*: how kernels find a cell's voxel */
    int32_t cuda_graph;            /* 1: batches run as captured CUDA graphs (replayed while
                                      the batch shape repeats); 0: direct launches */
    int32_t use_line_search;       /* NdtScanMatcherConfig::use_line_search (ndt.rs:69, default
                                      false). Graph semantics: the parallel line search, 8
                                      step candidates 0.618^k under the strong Wolfe
                                      conditions (ndt_graph_kernels.cu:388-430,473-570,
                                      626-710) instead of the clamped step. CPU semantics: the
                                      More-Thuente search of NdtOptimizer::align
                                      (solver.rs:268-280,640-700; more_thuente.rs), one trial
                                      pass per search step. Both run on the cluster kernel */
    int32_t work_queue;            /* Newton-kernel form: n > 0 the work-queue kernel (a
                                      persistent grid claiming chunks of n points per thread
                                      of any alignment's iteration); -1 one thread-block
                                      cluster per alignment; 0 autotuned (cluster kernel
                                      until tuned). Line search always uses the cluster
                                      kernel. */
    int32_t lanes_per_point;       /* work-queue kernel, graph semantics, 256 threads at 64
                                      registers: 2 or 4 lanes share each point's neighbour
                                      search (the occupied cells among its 27); 0 or 1: each
                                      lane searches its own point. The autotuner chooses it. */
    int32_t stage_points;          /* work-queue kernel: 1 stages each chunk's points in shared
                                      memory with one bulk copy (the TMA engine) before the
                                      chunk's work; 0 reads them from global memory. The
                                      autotuner chooses it. */
} ndt_config;

/* AlignResult (src/ndt_cuda/src/ndt.rs:219-248) with the pose as a vector. */
typedef struct ndt_result {
    double pose[6];
    double score;
    double transform_probability;  /* score / num source points (solver.rs:707-713) */
    double nvtl;                   /* compute_nvtl_simple at the final pose (scoring/nvtl.rs:211) */
    double hessian[36];            /* row-major */
    int32_t converged;
    int32_t iterations;
    int32_t num_correspondences;
    int32_t oscillation_count;
    int32_t status;                /* NDT_STATUS_* */
    int32_t reserved;
} ndt_result;

/* One scan of a batch (align_parallel_scans, src/ndt_cuda/src/ndt.rs:1224). */
typedef struct ndt_scan {
    const float* xyz;              /* host, num_points * 3 floats */
    uint64_t num_points;
    double initial_pose[6];
} ndt_scan;

typedef struct ndt_map_info {
    uint64_t num_points;           /* finite input points */
    uint64_t num_segments;         /* occupied cells */
    uint64_t num_voxels;           /* valid voxels (count >= min points, regularisable) */
    uint64_t hash_capacity;
    uint32_t max_probe;            /* longest insert probe sequence (slots) */
    uint32_t key_bits[3];          /* local key bits per axis */
    int32_t min_coord[3];
    int32_t max_coord[3];
    float build_ms;                /* device time of the last set_target build */
    float dense_grid_mib;          /* size of the dense cell index, 0 when the hash serves */
    uint32_t masks_per_cell;       /* neighbourhood masks per cell of the dense index: 1, or 8
                                      (one per octant) while they take at most 256 MiB; 0 when
                                      the hash serves */
    uint32_t reserved;
} ndt_map_info;

/* Counters accumulated by a context since creation or the last ndt_stats_reset. */
typedef struct ndt_stats {
    uint64_t align_launches;       /* Newton kernel launches */
    uint64_t alignments;
    uint64_t iterations;           /* sum of Newton iterations */
    uint64_t point_iterations;     /* sum over iterations of scan points processed */
    uint64_t correspondences;      /* sum over iterations of point-voxel pairs */
    double align_kernel_ms;        /* CUDA-event time of the Newton kernel launches */
    uint64_t score_launches;
    double score_kernel_ms;
    uint64_t build_launches;
    double build_ms;
    uint64_t h2d_bytes;
    uint64_t d2h_bytes;
    /* Newton kernel phase split, SM cycles summed over alignments (rank-0 CTA view) */
    uint64_t cycles_points;        /* point work + CTA reduction */
    uint64_t cycles_cluster_wait;  /* waiting for the other CTAs of the cluster */
    uint64_t cycles_control;       /* FP64 reduction, Hessian assembly, 6x6 solve, step */
    uint64_t cycles_broadcast;     /* pose broadcast barrier */
    uint64_t eigen_solves;         /* iterations whose Hessian took the eigen path */
    /* learned initial-pose search: forward passes of the proposal network and their
     * CUDA-event time (features, GEMMs, decode) on the network's stream */
    uint64_t proposal_launches;
    double proposal_kernel_ms;
} ndt_stats;

typedef struct ndt_ctx ndt_ctx;

/* Defaults of NdtScanMatcherConfig::default() (src/ndt_cuda/src/ndt.rs:90-107). */
int ndt_config_default(ndt_config* cfg);

/* NdtScanMatcher::with_config (src/ndt_cuda/src/ndt.rs:279-331). */
int ndt_ctx_create(const ndt_config* cfg, ndt_ctx** out);
int ndt_ctx_destroy(ndt_ctx* ctx);
/* Replaces the alignment parameters of a live context (iterations, epsilon, step size,
 * outlier ratio, neighbour cap, semantics, launch shape) without touching the map. The
 * map parameters (resolution, min points, eigenvalue ratio, hash factor) take effect at the
 * next ndt_set_target. */
int ndt_ctx_configure(ndt_ctx* ctx, const ndt_config* cfg);
/* the context's CUDA stream (a cudaStream_t), for callers that order their own work on it */
void* ndt_ctx_stream(ndt_ctx* ctx);

/* NdtScanMatcher::set_target (src/ndt_cuda/src/ndt.rs:361-407): builds the voxel map
 * (Morton keys, LSD radix sort, segments, FP64 moments, eigen regularisation, hash insert)
 * on the device. `xyz` is host memory; the _device variant takes a device pointer. */
int ndt_set_target(ndt_ctx* ctx, const float* xyz, uint64_t num_points);
int ndt_set_target_device(ndt_ctx* ctx, const float* d_xyz, uint64_t num_points);
int ndt_map_info_get(ndt_ctx* ctx, ndt_map_info* out);

/* Map tiles streamed in and out (the map module's tile loading and the dual matcher's
 * rebuild-and-swap, src/cuda_ndt_matcher/src/map_module.rs:192-360,
 * src/cuda_ndt_matcher/src/dual_ndt_manager.rs). Tiles (host points, uploaded once) stay in
 * device memory under a caller-chosen id; ndt_tile_put adds or replaces one, ndt_tile_remove
 * drops one. The reference rebuilds its whole map from all points on every change; here the
 * work per point happens once, when its tile is put: ndt_tile_put sorts the tile's points by
 * cell and computes every cell's count and FP64 statistics. ndt_tiles_commit then merges the
 * resident tiles' cells into a standby map (cells held by one tile keep its statistics; a cell
 * shared by tiles is recomputed from all its points), on the context's second stream and a
 * background host thread, while alignment calls keep using the active map. The result equals
 * ndt_set_target of the tiles' points concatenated in put order (a replaced tile keeps its
 * place). The first alignment (or map query) call after the merge has finished switches to
 * the new map. wait = 1 waits for the merge and switches before returning. A failed merge
 * leaves the active map in place; ndt_tiles_status reports it. */
int ndt_tile_put(ndt_ctx* ctx, uint64_t tile_id, const float* xyz, uint64_t num_points);
int ndt_tile_remove(ndt_ctx* ctx, uint64_t tile_id);
int ndt_tiles_commit(ndt_ctx* ctx, int32_t wait);
/* pending: 1 while a merge runs; last_rc: result of the last finished merge; build_ms: its
 * device time; put_ms: device time of the last ndt_tile_put's cell statistics. Any output
 * pointer may be NULL. */
int ndt_tiles_status(ndt_ctx* ctx, uint64_t* num_tiles, uint64_t* num_points, int32_t* pending,
                     int32_t* last_rc, float* build_ms, float* put_ms);
/* VoxelGrid accessors (means_flat / inv_covariances_flat, voxel_grid/mod.rs:428-453):
 * valid voxels in ascending coordinate-Morton order; any output pointer may be NULL. */
int ndt_map_voxels(ndt_ctx* ctx, int32_t* coords, float* means, float* covs, float* icovs,
                   uint32_t* counts, uint64_t capacity);

/* NdtScanMatcher::align / align_gpu (src/ndt_cuda/src/ndt.rs:421-510). */
int ndt_align(ndt_ctx* ctx, const float* xyz, uint64_t num_points, const double pose_in[6],
              ndt_result* out);
/* NdtScanMatcher::align_batch_gpu (src/ndt_cuda/src/ndt.rs:959): one scan, many poses. */
int ndt_align_multi_pose(ndt_ctx* ctx, const float* xyz, uint64_t num_points,
                         const double* poses_in, uint64_t num_poses, ndt_result* out);
/* NdtScanMatcher::align_parallel_scans (src/ndt_cuda/src/ndt.rs:1224-1321): uneven scans
 * aligned in one launch (one thread-block cluster per alignment, or the work-queue kernel). */
int ndt_align_batch(ndt_ctx* ctx, const ndt_scan* scans, uint64_t num_scans, ndt_result* out);

/* Asynchronous batches: AsyncBatchPipeline::submit / poll / wait
 * (src/ndt_cuda/src/optimization/async_pipeline.rs:348-615), the double-buffered feed of
 * the scan queue (src/cuda_ndt_matcher/src/scan_queue.rs). Up to 3 batches in flight per
 * context, each on its own stream with its own staging and device buffers, aligned against
 * the context's map as ndt_align_batch would align them (same results).
 *   - ndt_batch_submit stages the scans (the caller's arrays may be reused on return),
 *     queues the copies and kernels, and returns a ticket; NDT_ERR_CAPACITY when 3 batches
 *     wait to be collected.
 *   - ndt_batch_poll sets *ready to 1 once the batch has finished (non-blocking).
 *   - ndt_batch_wait blocks until the batch has finished, writes its num_scans results and
 *     frees the slot; the context's stats and ndt_batch_timings then include it.
 * Calls that change the map (set_target, tile commits) first wait for the batches in
 * flight; their results stay available to ndt_batch_wait. */
int ndt_batch_submit(ndt_ctx* ctx, const ndt_scan* scans, uint64_t num_scans, uint64_t* ticket);
int ndt_batch_poll(ndt_ctx* ctx, uint64_t ticket, int32_t* ready);
int ndt_batch_wait(ndt_ctx* ctx, uint64_t ticket, ndt_result* out);
/* Same, with the scans already resident on the device, concatenated: scan i is
 * d_xyz[3*offsets[i] .. 3*offsets[i+1]); offsets and poses are host arrays. */
int ndt_align_batch_device(ndt_ctx* ctx, const float* d_xyz, const uint64_t* offsets,
                           const double* poses_in, uint64_t num_scans, ndt_result* out);

/* Autotuner for the Newton kernel's launch shape: times the cluster kernel at every
 * (cluster size 1, 2, 4, 8) x (threads per CTA, register cap) candidate and the work-queue
 * kernel at its (threads, registers, points per thread per chunk, lanes per point's neighbour
 * search) candidates (unless the
 * configuration fixes the form, or line search is on) on the given device-resident batch
 * (as ndt_align_batch_device takes it), `repeats` timed runs each, and records the fastest
 * for batches of this size class (log2 of the scan count and of the largest scan). Later
 * calls in that class use it unless the configuration fixes cluster_size /
 * threads_per_cta. No counterpart in the reference, whose launch shapes are constants. */
typedef struct ndt_tune_result {
    int32_t cluster_size;
    int32_t threads_per_cta;
    double kernel_ms;              /* Newton kernel time of the winner, per batch */
    double aligns_per_s;           /* batch size / kernel_ms */
    int32_t candidates;
    int32_t registers;             /* register cap of the winning kernel instance */
    int32_t work_queue;            /* points per thread per chunk of the winner if it is the
                                      work-queue kernel, else 0 */
    int32_t lanes_per_point;       /* lanes sharing each point's neighbour search in the
                                      winning work-queue kernel (1, 2, 4), else 0 */
    int32_t stage_points;          /* 1 when the winning work-queue kernel stages its chunks'
                                      points in shared memory */
    int32_t reserved;
} ndt_tune_result;
int ndt_autotune(ndt_ctx* ctx, const float* d_xyz, const uint64_t* offsets,
                 const double* poses_in, uint64_t num_scans, int32_t repeats,
                 ndt_tune_result* out);

/* evaluate_nvtl / evaluate_transform_probability / evaluate_nvtl_batch
 * (src/ndt_cuda/src/ndt.rs:681-890): per pose, NVTL (mean over points with a neighbour of
 * the best voxel score) and score / correspondences over all voxels within one resolution.
 * T34 = num_poses row-major 3x4 world transforms (host). nvtl / tp may be NULL. */
int ndt_eval_batch(ndt_ctx* ctx, const float* xyz, uint64_t num_points, const double* T34,
                   uint64_t num_poses, double* nvtl, double* transform_probability);

/* Per-alignment device timing of the last alignment call (any ndt_align* entry): start and
 * finish of each alignment in ms, relative to the earliest start of that call, by the
 * caller's result index. n must not exceed the number of alignments of that call. */
int ndt_batch_timings(ndt_ctx* ctx, double* start_ms, double* finish_ms, uint64_t n);

/* Multi-particle initial-pose search: estimate_initial_pose + align_batch_gpu +
 * select_best_particle (src/cuda_ndt_matcher/src/initial_pose.rs:115-460,
 * src/ndt_cuda/src/optimization/solver.rs:459-561, src/cuda_ndt_matcher/src/particle.rs:36-42).
 * Every query's particles are aligned in one launch (all queries together), each result is
 * scored by NVTL at its aligned pose, and the particle with the highest selection score wins:
 * NVTL when positive, else 5 exp(-score / 10) (initial_pose.rs:233-245); ties go to the later
 * particle, as Rust's max_by does. Particle k of query q starts from the query's prior pose
 * with x, y + U(-xy_range, xy_range), yaw + U(-yaw_range, yaw_range) (yaw_range = pi covers
 * the circle, like the reference's uniform yaw) and z, roll, pitch + N(0, sigma^2) — drawn
 * from a SplitMix64 stream seeded by (seed, q, k), so a search is reproducible.
 * With guided > 0 the last `guided` particles of each query are TPE-guided, as the reference's
 * guided phase (initial_pose.rs:280-420; TreeStructuredParzenEstimator, tpe.rs; its defaults
 * are 200 particles, 100 of them startup): each is the best of 100 further draws by the
 * Parzen log-likelihood ratio over the query's aligned results so far (x, y, yaw kernels of
 * 0.25 m, 0.25 m, 2.5 deg; the best max(1, min(10, n / 10)) results are the good set, score
 * exp(-score / 10)). The startup particles go in one launch; the guided ones go in rounds, one
 * particle of every query per launch. */
typedef struct ndt_particle_config {
    uint32_t num_particles;        /* particles per query (200) */
    uint32_t guided;               /* TPE-guided particles among them (0: all drawn up front;
                                      the reference: 100); < num_particles */
    double xy_range;               /* 2.0 m */
    double yaw_range;              /* pi */
    double z_sigma;                /* 0 */
    double roll_pitch_sigma;       /* 0 */
    uint64_t seed;
} ndt_particle_config;

typedef struct ndt_pose_estimate {
    double pose[6];                /* aligned pose of the best particle */
    double initial_pose[6];        /* the particle it started from */
    double nvtl;
    double score;
    double selection_score;
    int32_t particle;              /* index of the best particle within its query */
    int32_t iterations;
    int32_t converged;
    int32_t reserved;
} ndt_pose_estimate;

/* The TPE proposal of a guided particle (host only): particle `particle` of query `query`
 * from the query's prior and its num_trials aligned results so far, in the order they were
 * aligned, 4 doubles each (x, y, yaw of the aligned pose, exp(-score / 10)). */
int ndt_tpe_propose(const ndt_particle_config* cfg, uint64_t query, uint64_t particle,
                    const double prior[6], const double* trials, uint64_t num_trials,
                    double pose_out[6]);

/* out: num_queries estimates; particles (optional, may be NULL): num_queries *
 * num_particles results, query-major. Each query's ndt_scan gives its points and prior. */
int ndt_initial_pose_search(ndt_ctx* ctx, const ndt_scan* queries, uint64_t num_queries,
                            const ndt_particle_config* cfg, ndt_pose_estimate* out,
                            ndt_result* particles);

/* ---- Learned initial-pose proposals ---------------------------------------------------
 * No counterpart in the reference, which draws all initial-pose particles at random (or from
 * its sequential TPE). A small network (the "proposal network") maps a scan and a coarse
 * pose to a few candidate poses. Each candidate is refined by plain NDT and judged by NVTL;
 * when the best NVTL is below a threshold, the plain particle search runs instead.
 * - Input: a 64 x 64 x 8 occupancy grid of the scan at 1 m, rotated by the coarse yaw, plus
 *   a 64 x 64 crop at 1 m of the map's height image around the coarse position.
 * - Layers: hidden_layers x hidden (GELU), then proposals x (dx, dy, dyaw, logit).
 * - Every matrix product runs on the tcgen05 tensor cores (bf16 operands, f32 accumulate).
 * - Training pairs come from scans with known converged poses (ndt_pnet_add_scan), perturbed
 *   on the device: x, y + U(-xy_range, xy_range), yaw uniform on the circle. */
typedef struct ndt_pnet_config {
    int32_t input_dim;             /* 36864 = 64*64*8 scan grid + 64*64 map crop */
    int32_t hidden;                /* 512 */
    int32_t hidden_layers;         /* 4 */
    int32_t proposals;             /* 16 */
    int32_t batch;                 /* 256: inference chunk (queries per network launch) */
    float learning_rate;           /* Adam, 3e-4 */
    float xy_range;                /* training perturbation of x, y (m): 5 */
    float yaw_weight;              /* loss weight of the yaw error (its scale pi / yaw_weight
                                      against 4 m for x, y): 8 */
    uint64_t seed;                 /* weight initialisation and training samples */
    int32_t train_batch;           /* samples per training step, a multiple of 64 (0: batch);
                                      default 1024 */
    int32_t reserved;
} ndt_pnet_config;

typedef struct ndt_pnet ndt_pnet;

int ndt_pnet_config_default(ndt_pnet_config* cfg);
int ndt_pnet_create(const ndt_pnet_config* cfg, int32_t device, ndt_pnet** out);
int ndt_pnet_destroy(ndt_pnet* net);
int ndt_pnet_get_config(ndt_pnet* net, ndt_pnet_config* out);
/* Adds a map (host points) for features: its 1 m height image. Returns its id. */
int ndt_pnet_add_map(ndt_pnet* net, const float* xyz, uint64_t num_points, int32_t* map_id);
/* Adds a training scan (sensor frame, host) of map `map_id` with its converged pose. */
int ndt_pnet_add_scan(ndt_pnet* net, int32_t map_id, const float* xyz, uint64_t num_points,
                      const double pose[6], int32_t* scan_id);
/* `steps` Adam steps of `batch` freshly perturbed samples; loss_out (optional) per step. */
int ndt_pnet_train(ndt_pnet* net, uint64_t steps, float* loss_out);
/* Counters of a network since creation: inference_kernel_ms is the CUDA-event time of the
 * device work of ndt_pnet_propose (feature build, every layer's GEMM and activation, decode;
 * not the query upload), train_ms that of ndt_pnet_train. */
typedef struct ndt_pnet_stats {
    uint64_t inference_batches;    /* forward passes (one per `batch` queries) */
    uint64_t queries;
    double inference_kernel_ms;
    uint64_t train_steps;
    double train_ms;
} ndt_pnet_stats;
int ndt_pnet_stats_get(ndt_pnet* net, ndt_pnet_stats* out);
/* Candidate poses of each query (its ndt_scan's initial_pose is the coarse pose):
 * poses num_queries * proposals * 6, logits num_queries * proposals (optional). */
int ndt_pnet_propose(ndt_pnet* net, int32_t map_id, const ndt_scan* queries,
                     uint64_t num_queries, double* poses, double* logits);
/* One forward + backward on given inputs x (b x input_dim, rounded to bf16) and targets
 * (b x 3: dx, dy in m, dyaw in rad): mean loss and every parameter's gradient (the
 * ndt_pnet_params order), without an update. For checking against an FP64 restatement. */
int ndt_pnet_debug_grad(ndt_pnet* net, const float* x, const float* targets, uint64_t b,
                        float* loss, float* grads);
/* Parameters in f32, layer by layer (W out x in row-major, then b): read (set = 0) or
 * write (set = 1). With params NULL, *count receives the number of values. */
int ndt_pnet_params(ndt_pnet* net, float* params, uint64_t* count, int32_t set);
/* Learned initial-pose search on the context's target map (also added to the network as
 * map_id): proposals -> one alignment launch for all queries -> NVTL -> selection as in
 * ndt_initial_pose_search. With refine (optional, num_particles > 0), a second round draws
 * refine->num_particles particles around each query's winner (x, y +- xy_range, yaw +-
 * yaw_range; guided ignored), aligns them in one launch and keeps the better winner. Queries
 * whose best NVTL is then below nvtl_threshold (2.3) rerun as a plain particle search with
 * `fallback` (optional). used_fallback (optional): 1 per such query. */
int ndt_learned_pose_search(ndt_ctx* ctx, ndt_pnet* net, int32_t map_id, const ndt_scan* queries,
                            uint64_t num_queries, const ndt_particle_config* refine,
                            double nvtl_threshold, const ndt_particle_config* fallback,
                            ndt_pose_estimate* out, int32_t* used_fallback);

/* The network's GEMM: D[m x n] (f32, row-major) = A[m x k] B[n x k]^T with A, B bf16
 * row-major (device), k a multiple of 64; synchronous (checks the kernel's wait limits).
 * splits > 1 (split-K, at most k / 64): D holds `splits` partial products one after the
 * other (d_d + z * m * n covers k-blocks [z k/64/splits, (z+1) k/64/splits)); their sum is
 * the product. */
int ndt_gemm_bf16(const void* d_a, const void* d_b, float* d_d, int32_t m, int32_t n, int32_t k,
                  int32_t splits, void* stream);

/* 27-cell hash neighbour query (graph_hash_query_inline, ndt_graph_kernels.cu:47-104;
 * voxel_hash_query_kernel, voxel_hash.cu:136-210) for host query points; idx is
 * num_points * max_neighbors voxel indices (Morton order), -1 padded. */
int ndt_neighbors_query(ndt_ctx* ctx, const float* xyz, uint64_t num_points,
                        int32_t max_neighbors, int32_t* idx, int32_t* counts);

int ndt_stats_get(ndt_ctx* ctx, ndt_stats* out);
int ndt_stats_reset(ndt_ctx* ctx);
/* Enables CUDA-event timing of every kernel launch (read back through ndt_stats). */
int ndt_profile_enable(ndt_ctx* ctx, int enable);

/* Per-iteration records of the Newton loop (the K5 debug buffer of
 * src/cuda_ffi/csrc/ndt_graph_common.cuh:101-114): when enabled, every alignment records per
 * iteration 48 doubles: iteration, score, correspondences, pose before the step (6),
 * gradient (6), Hessian upper triangle (21), raw solver output (6), solver path
 * (0 Cholesky, 1 eigen), solver success, 4 reserved. ndt_debug_read copies the records of
 * result `index` of the last alignment call. */
int ndt_debug_trace(ndt_ctx* ctx, int enable);
int ndt_debug_read(ndt_ctx* ctx, uint64_t index, double* out, int32_t max_records,
                   int32_t* num_records);

/* Test hook for the work-queue kernel's no-progress limit (no counterpart in the reference,
 * whose host loop synchronises after every kernel). A work-queue CTA that finds no chunk to
 * claim while alignments are open gives up after limit_ns (default 2 s; 0 restores it) and
 * the call returns NDT_ERR_DEVICE. With withhold_next = 1, the next work-queue launch starts
 * with every chunk of every alignment already claimed, so no CTA finds work and the limit
 * runs out: the error path can be tested without a fault. The context stays usable. */
int ndt_debug_queue_stall(ndt_ctx* ctx, uint64_t limit_ns, int32_t withhold_next);

const char* ndt_last_error_string(void);

/* ---- build-stage primitives on caller device memory (the cuda_ffi roles) ------------ */
/* Temporary storage follows the two-phase convention of the reference's CUB wrappers:
 * call with d_temp == NULL to read the required *temp_bytes. `stream` is a cudaStream_t. */

/* cub_radix_sort_pairs_u64_u32 (src/cuda_ffi/csrc/radix_sort.cu:62-86): stable ascending
 * LSD sort of (u64 key, u32 value) pairs on bits [begin_bit, end_bit), in place. */
int ndt_radix_sort_pairs_u64_u32(uint64_t* d_keys, uint32_t* d_values, uint64_t n,
                                 int32_t begin_bit, int32_t end_bit, void* d_temp,
                                 uint64_t* temp_bytes, void* stream);
/* Allocation-free variant of ndt_radix_sort_pairs_u64_u32; it has no counterpart in the
 * reference. It is for callers that may not allocate device memory while they run: a
 * real-time loop where cudaMalloc/cudaFree would synchronise the device and stall the
 * pipeline, or a process held to a fixed device-memory budget. Same result as
 * ndt_radix_sort_pairs_u64_u32 (stable ascending sort of bits [begin_bit, end_bit), in place),
 * but the scratch is one fixed array inside this library (12,845,312 bytes per device), so:
 *  - n <= 1048576 pairs; larger n returns NDT_ERR_CAPACITY and touches nothing;
 *  - the first call on each device does the set-up (resolves the array's device address,
 *    which can load the library's kernels onto that device): make it, with that device
 *    current, before any stream capture. A cudaDeviceReset ends the context that address
 *    belongs to; the first call after it (in a new context) does the set-up again;
 *  - the scratch needs no initial contents (nothing in it has to start at zero);
 *  - all calls on one device share the scratch: two calls whose work overlaps on the GPU
 *    (different streams, or host threads with no ordering between their streams) race and
 *    corrupt each other's results. Issue them on one stream, or order them. */
int ndt_radix_sort_pairs_u64_u32_static(uint64_t* d_keys, uint32_t* d_values, uint64_t n,
                                        int32_t begin_bit, int32_t end_bit, void* stream);
/* detect_boundaries_kernel + InclusiveSum + Flagged (src/cuda_ffi/csrc/segment_detect.cu:
 * 27-146): segment id per element and start index per segment of sorted keys. */
int ndt_detect_segments(const uint64_t* d_sorted, uint64_t n, uint32_t* d_segment_ids,
                        uint32_t* d_segment_starts, uint32_t* d_num_segments, void* d_temp,
                        uint64_t* temp_bytes, void* stream);
/* compute_morton_codes_kernel (src/ndt_cuda/src/voxel_grid/gpu/morton.rs:45-95) with this
 * library's membership rule: key = morton(floor(p / res) - min cell), idx = identity.
 * min_cell (3 x int32, device) receives the per-axis minimum cell. */
int ndt_morton_codes(const float* d_xyz, uint64_t n, float resolution, uint64_t* d_codes,
                     uint32_t* d_indices, int32_t* d_min_cell, void* d_temp,
                     uint64_t* temp_bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* NDT_GB300_H */
