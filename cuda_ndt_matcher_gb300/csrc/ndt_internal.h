// ndt_internal.h — host-side structures shared by the library's translation units.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "ndt_common.cuh"
#include "ndt_gb300.h"

namespace ndtgb {

// Grow-only device allocation owned by a context.
// Elementwise work fused into the tcgen05 GEMM's epilogue (tc_gemm.cu), per element (row m,
// column n) of the accumulator acc:
//   GEMM_EPI_STORE        D = acc
//   GEMM_EPI_BIAS_GELU    z = acc + bias[n]: D = z, x = GELU(z) as bf16 into x [M x N] and
//                         xt [N x M] (the next layer's input in both operand layouts)
//   GEMM_EPI_BIAS         z = acc + bias[n]: D = z (the output layer)
//   GEMM_EPI_GELU_BACK    g = acc * GELU'(zin[m][n]): D = g, bf16 g into x [M x N] and
//                         xt [N x M] (the previous layer's output gradient)
// Not with split-K (a partial product has no bias and no activation).
enum { GEMM_EPI_STORE = 0, GEMM_EPI_BIAS_GELU = 1, GEMM_EPI_BIAS = 2, GEMM_EPI_GELU_BACK = 3 };
struct GemmEpilogue {
    int mode;
    const float* bias;
    const float* zin;
    __nv_bfloat16* x;
    __nv_bfloat16* xt;
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};
int dev_reserve(DevBuf& b, size_t bytes);
void dev_free(DevBuf& b);

struct PinBuf {
    void* p = nullptr;
    size_t bytes = 0;
};
int pin_reserve(PinBuf& b, size_t bytes);
void pin_free(PinBuf& b);

void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

// Device-resident voxel map.
struct Map {
    DevBuf slots, slot_icov, slot_vidx, grid, nmask;
    DevBuf vox_coord, vox_mean, vox_cov, vox_icov, vox_count;
    MapView view{};
    ndt_map_info info{};
    bool valid = false;
};

// Scratch used while building a map (kept for the next rebuild).
struct BuildScratch {
    DevBuf keys_a, keys_b, vals_a, vals_b, tmp;
    DevBuf seg_ids, seg_starts, seg_valid, seg_rank, seg_rec, small;
};

// Temporary-storage sizing of the sort / scan primitives (two-phase convention).
size_t radix_sort_temp_bytes(size_t n);
size_t scan_temp_bytes(size_t n);
int radix_sort_pairs(uint64_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                     void* temp, size_t temp_bytes, cudaStream_t s);
int radix_sort_pairs32(uint32_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                       void* temp, size_t temp_bytes, cudaStream_t s);
int detect_segments(const uint64_t* sorted, size_t n, uint32_t* seg_ids, uint32_t* seg_starts,
                    uint32_t* num_segments, void* temp, size_t temp_bytes, cudaStream_t s);
size_t detect_segments_temp_bytes(size_t n);
int morton_codes(const float* pts, size_t n, float res, uint64_t* codes, uint32_t* idx,
                 int32_t* d_minmax /* 6 ints + count */, cudaStream_t s);

// Point count and cell box of a set of segments (a point set's, or a merge of tiles').
struct SegGeometry {
    size_t nf = 0;      // finite points
    uint32_t S = 0;     // segments (occupied cells)
    int32_t mn[3] = {0, 0, 0}, mx[3] = {0, 0, 0};
};
int build_map(Map& map, BuildScratch& sc, const float* d_pts, size_t n, const ndt_config& cfg,
              uint32_t* d_status, cudaStream_t s, float* build_ms);

// Per-segment (per occupied cell) record of a build: cell, count and, for a voxel, its
// mean, regularised covariance and inverse (upper triangle).
struct SegRec {
    float mean[3];
    float cov[9];
    float icov[6];  // c00, c01, c02, c11, c12, c22
    int32_t coord[3];
    uint32_t count;
};

// A map tile's segments, built once when the tile is put: point indices in key order,
// segment starts, records and validity, with the tile's cell box.
struct TileSegs {
    DevBuf idx, starts, rec, valid;
    SegGeometry geo;
};
int build_tile_segments(BuildScratch& sc, const float* d_pts, size_t n, const ndt_config& cfg,
                        cudaStream_t s, TileSegs& out, float* ms_out);

// One tile as the merge kernels read it (device pointers; seg_off = the tile's first segment
// in the concatenation of all tiles' segments, in tile order).
struct TileSegRef {
    const SegRec* rec;
    const uint32_t* valid;
    const uint32_t* starts;
    const uint32_t* idx;
    const float* pts;
    uint64_t seg_off;
    uint32_t S, nf;
    int32_t mn[3], mx[3];
};
// The voxel map of the tiles' points concatenated in the given order, from their segments:
// the same map build_map gives for that concatenation. Cells held by one tile keep that
// tile's records; cells shared by tiles are recomputed from their points.
int merge_tiles(Map& map, BuildScratch& sc, const std::vector<TileSegRef>& refs, DevBuf& d_refs,
                const ndt_config& cfg, uint32_t* d_status, cudaStream_t s, float* build_ms);

// One alignment job of a launch.
struct AlignJob {
    uint64_t offset;   // first point (index into the concatenated xyz array)
    uint32_t n;        // points
    uint32_t slot;     // index of the caller's result
    double pose[6];    // initial pose
};

struct AlignOut {
    double pose[6];
    double score;
    double hessian[36];
    int32_t iterations;
    int32_t converged;
    int32_t ncorr;
    int32_t osc;
    int32_t status;
    int32_t pad;
    uint64_t point_iters;
    uint64_t corr_total;
    uint64_t cycles[4];  // SM cycles: points + CTA reduce, cluster wait, control, broadcast
    int32_t n_eigen;     // iterations that took the eigen (indefinite) solver path
    int32_t pad2;
    uint64_t t_start, t_end;  // global timer (ns) when the alignment started / finished
};

// Per-iteration trace record (doubles): it, score, correspondences, pose before the step (6),
// gradient (6), Hessian upper triangle (21), raw solver output (6), solver path, solver ok,
// then 4 device-only fields: SM cycles of the g/H assembly, of the 6x6 solve and of the step
// plus next frame, and the FP64 Jacobi sweeps of an eigen solve. Fields 0-43 have the same
// layout as the oracle's trace (whose last 4 are zero).
constexpr int TRACE_REC = 48;

// Largest dense cell index a map build makes (bytes); beyond it the kernels probe the hash.
constexpr uint64_t DENSE_GRID_MAX_BYTES = 4096ull << 20;
// octant neighbourhood masks (32 B per cell of the grown box) up to this size, else one
// mask per cell (4 B): the octant masks cost eight times the scatter of one mask per cell
constexpr uint64_t OCTANT_MASK_MAX_BYTES = 256ull << 20;

struct AlignParams {
    MapView map;
    double* trace;     // nullptr unless tracing is enabled
    const float* pts;
    const AlignJob* jobs;
    AlignOut* out;
    uint32_t num_jobs;
    int32_t max_iter;
    int32_t max_nb;
    int32_t semantics;
    int32_t min_corr;
    int32_t cluster;
    float d1f, d2f;
    double d1, d2;
    double step_size;
    double eps;
    uint32_t* status;
    int32_t ls_cands;      // graph-path line search: candidates per iteration (0: off)
    double ls_mu, ls_nu;   // strong Wolfe constants
    // work-queue kernel (k_ndt_queue): per-alignment claim words, controller state, frames,
    // per-chunk partial sums (offsets by alignment), counters {alignments finished}
    struct QJob* qjobs;
    struct QCtl* qctl;
    float* qframe;
    double* qpart;
    const uint32_t* qpart_off;
    uint32_t* qcount;
    int32_t qchunk;        // points per chunk (set by the launch from the shape); chunks of
                           // 1/QSPLIT_DIV of it in an alignment's late iterations
    uint32_t qchunks_total;  // chunks of one iteration of every alignment (at full size)
    uint32_t qgrid;          // CTAs of the launch (set by the launch)
    // points copied in while the work-queue kernel runs: the device word counts the points of
    // the batch resident so far (a prefix of pts, written by the copy stream after each
    // chunk); an alignment is claimable once its last point is resident. nullptr: all are.
    const uint32_t* qarrive;
    uint32_t qarrive_total;  // the word's value once every point is resident
    // 1: this launch continues an earlier one over the same state (no initialisation). With
    // qarrive set, CTAs that find nothing to claim while input is still arriving leave after
    // QSTARVE_NS without input progress, so the kernel never depends on copies that another
    // stream may only run after it (the host then launches the continuation after the last
    // copy).
    int32_t qresume;
    // work-queue kernel: a CTA that finds no work for stall_ns with alignments open (and all
    // input resident) sets ST_QUEUE_STALL and leaves (2 s unless a test shortens it); with
    // withhold, every chunk starts out claimed (a test hook: no CTA finds work)
    uint64_t stall_ns;
    int32_t withhold;
    // work-queue kernel: each chunk's points staged into shared memory by one bulk copy
    // (needs the points' buffer 16-byte aligned)
    int32_t qstage;
};
constexpr unsigned long long QSTARVE_NS = 2000000ull;
constexpr unsigned long long QSTALL_NS = 2000000000ull;

// Newton-kernel sums per iteration: 34 f32 per-thread accumulators (score, gradient and
// Hessian terms), reduced in FP64, plus the correspondence count.
constexpr int NACC = 34;
constexpr int NRED = NACC + 1;

// Work-queue kernel state, one per alignment (global memory).
struct QJob {
    // iteration << 48 | the iteration's chunk count << 32 | chunks claimed (iteration QDONE:
    // the alignment is finished)
    unsigned long long gen_claim;
    uint32_t done;                 // chunks of the current iteration finished
    uint32_t pad;
};
constexpr uint32_t QDONE = 0xFFFFu;
constexpr uint32_t QMAXCH = 0xFFFFu;  // chunks per iteration at most (16-bit count)
// Chunks of an alignment's late iterations are 1/QSPLIT_DIV of the launch's chunk size, and
// 1/(2 QSPLIT_DIV) in its last ones (the partial-sum slots are sized for those). At the
// 20k-point bench batch, 2 and 8 were slower as the first split.
constexpr uint32_t QSPLIT_DIV = 4;
// Controller state of an alignment between iterations (FP64; read and written only by the
// controller of the alignment's current iteration).
struct QCtl {
    // the FP64 block (QCTL_DOUBLES, contiguous: the controller moves it with one load and one
    // store per lane and element group)
    double pose[6], best_pose[6], best_score, last_H[36], prev[3], prev2[3];
    double W[36];
    double Ad[27], Bd[54];
    uint64_t point_iters, corr_total, t_start;
    unsigned long long cyc_chunks, cyc_ctl;
    int32_t last_corr, osc, max_osc, n_eigen, have_w, pad;
};
constexpr int QCTL_DOUBLES = 172;
static_assert(offsetof(QCtl, Bd) == 118 * sizeof(double) &&
                  offsetof(QCtl, point_iters) == QCTL_DOUBLES * sizeof(double),
              "QCtl's FP64 block is pose, best_pose, best_score, last_H, prev, prev2, W, Ad, Bd");

// Line search of the graph path: at most 8 candidates (GRAPH_MAX_LS_CANDIDATES,
// ndt_graph_common.cuh:18); Armijo and curvature constants of PipelineV2Config::default
// (full_gpu_pipeline_v2.rs:101-113)
constexpr int LS_MAX = 8;
constexpr double LS_MU = 1e-4;
constexpr double LS_NU = 0.9;
// Line search of the CPU path: the More-Thuente search with MoreThuenteConfig::default()
// (more_thuente.rs:36-46): steps in [1e-9, 0.1], at most 10 iterations after the first trial
constexpr double MT_STEP_MIN = 1e-9;
constexpr double MT_STEP_MAX = 0.1;
constexpr int MT_MAX_ITER = 10;

struct LaunchShape {
    int cluster;
    int threads;
    int regcap;  // 128 (default); 80, 64, 48: denser residency for 128/256-thread CTAs
    int queue;   // > 0: work-queue kernel, chunks of `queue` points per thread (cluster 1)
    int npw;     // work-queue kernel: lanes sharing each point's neighbour search (0, 1: one)
    int stage;   // work-queue kernel: 1 stages each chunk's points in shared memory (bulk copy)
};

int launch_align(const AlignParams& p, LaunchShape shape, cudaStream_t s);

// Per-pose scoring (NVTL + score/correspondences over all neighbours within one resolution).
struct ScoreJob {
    uint64_t offset;
    uint32_t n;
    uint32_t pose_src;   // 0: T34 given; 1: take pose from AlignOut[pose_index] (zyx quirk)
    uint32_t out_index;
    uint32_t pad;
    double T[12];
};
struct ScoreOut {
    double nvtl_sum;
    double score_sum;
    uint64_t nvtl_count;
    uint64_t ncorr;
};
size_t score_part_bytes(uint32_t num_jobs, uint32_t max_n);
int launch_score(const MapView& map, const float* pts, const ScoreJob* jobs, uint32_t num_jobs,
                 uint32_t max_n, const AlignOut* align_out, void* part, ScoreOut* out, float d1,
                 float d2, cudaStream_t s);
int launch_query(const MapView& map, const float* q, size_t n, int max_nb, int32_t* idx,
                 int32_t* cnt, cudaStream_t s);

}  // namespace ndtgb
