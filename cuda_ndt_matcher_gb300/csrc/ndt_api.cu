// ndt_api.cu — the C ABI of libndt_gb300.so (declared in include/ndt_gb300.h).
//
// A context owns one CUDA stream, the device voxel map, grow-only device buffers, pinned
// host staging buffers and a few host threads. An alignment call packs the host scans into
// pinned memory with those threads, copying each packed chunk to the device while the next
// is packed, launches the Newton kernel (one cluster per alignment, longest scans first) and
// the NVTL kernel on the final poses (as a CUDA graph when configured), copies the
// per-alignment records back and synchronises once.
#include <algorithm>
#include <memory>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <vector>

#include "ndt_internal.h"

namespace ndtgb {

static thread_local std::string g_err;

void set_error(const std::string& m) { g_err = m; }

int cuda_fail(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return 0;
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return (int)e;
}

int dev_reserve(DevBuf& b, size_t bytes) {
    if (bytes <= b.bytes && b.p) return 0;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
    size_t nb = std::max<size_t>(bytes + bytes / 4, 256);
    cudaError_t e = cudaMalloc(&b.p, nb);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    b.bytes = nb;
    return 0;
}

void dev_free(DevBuf& b) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

int pin_reserve(PinBuf& b, size_t bytes) {
    if (bytes <= b.bytes && b.p) return 0;
    if (b.p) cudaFreeHost(b.p);
    b.p = nullptr;
    b.bytes = 0;
    size_t nb = std::max<size_t>(bytes + bytes / 4, 256);
    cudaError_t e = cudaMallocHost(&b.p, nb);
    if (e != cudaSuccess) {
        b.p = nullptr;
        return cuda_fail(e, "cudaMallocHost");
    }
    b.bytes = nb;
    return 0;
}

void pin_free(PinBuf& b) {
    if (b.p) cudaFreeHost(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

static void gauss_params(double res, double outlier, double* d1, double* d2) {
    // GaussianParams::new (src/ndt_cuda/src/derivatives/types.rs:61-75)
    double c1 = 10.0 * (1.0 - outlier);
    double c2 = outlier / (res * res * res);
    double d3 = -std::log(c2);
    double g1 = -std::log(c1 + c2) - d3;
    double nom = -std::log(c1 * std::exp(-0.5) + c2) - d3;
    *d1 = g1;
    *d2 = -2.0 * std::log(nom / g1);
}

}  // namespace ndtgb

using namespace ndtgb;

// A few host threads for staging copies: run(n, f) calls f(0 .. n-1) across the workers and
// the calling thread and returns when every call is done. Workers start on first use and
// stop with the owning context.
class HostPool {
public:
    ~HostPool() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            quit_ = true;
        }
        cv_.notify_all();
        for (auto& w : workers_) w.join();
    }
    void run(uint64_t n, const std::function<void(uint64_t)>& f) {
        if (n == 0) return;
        start();
        if (workers_.empty() || n == 1) {
            for (uint64_t i = 0; i < n; ++i) f(i);
            return;
        }
        {
            std::lock_guard<std::mutex> lk(mu_);
            fn_ = &f;
            n_ = n;
            next_.store(0);
            active_ = workers_.size();
            ++gen_;
        }
        cv_.notify_all();
        drain();
        std::unique_lock<std::mutex> lk(mu_);
        done_cv_.wait(lk, [&] { return active_ == 0; });
        fn_ = nullptr;
    }

private:
    void drain() {
        for (uint64_t i; (i = next_.fetch_add(1)) < n_;) (*fn_)(i);
    }
    void start() {
        if (started_) return;
        started_ = true;
        const unsigned hw = std::thread::hardware_concurrency();
        const unsigned nt = hw > 1 ? std::min(7u, hw - 1) : 0u;
        for (unsigned t = 0; t < nt; ++t) workers_.emplace_back([this] { loop(); });
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            std::unique_lock<std::mutex> lk(mu_);
            cv_.wait(lk, [&] { return quit_ || gen_ != seen; });
            if (quit_) return;
            seen = gen_;
            lk.unlock();
            drain();
            lk.lock();
            if (--active_ == 0) done_cv_.notify_one();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void(uint64_t)>* fn_ = nullptr;
    uint64_t n_ = 0, gen_ = 0;
    std::atomic<uint64_t> next_{0};
    size_t active_ = 0;
    bool quit_ = false, started_ = false;
};

// A batch between its enqueue and its completion.
struct PendingAlign {
    std::vector<AlignJob> jobs;        // in launch order (largest scans first)
    std::vector<uint64_t> n_by_slot;   // points of each of the caller's scans
    int max_iter = 0;
    bool cpu = false;
    size_t ob = 0, sob = 0;            // byte offsets of the score outputs and status word
    bool active = false;
};

// Host scans of a batch laid out for copying in: the jobs are in launch order (largest scan
// first), job j's points go to jobs[j].offset, and the copy runs in chunks of jobs
// [chunk_job[k], chunk_job[k + 1]) of 256 KB doubling to 16 MB, each starting on a 64-point
// (768-byte) boundary.
struct StagePlan {
    const ndt_scan* scans = nullptr;
    std::vector<uint32_t> chunk_job;   // first job of each chunk, then the job count
    uint64_t total = 0;                // end of the last job's points (padding included)
};

struct ndt_ctx;

// Asynchronous batches (ndt_batch_submit / ndt_batch_wait): each slot is an internal context
// with its own stream, buffers and pinned staging, aligning against its owner's map.
struct AsyncSlot {
    ndt_ctx* ctx = nullptr;
    uint64_t ticket = 0;               // 0: free
    uint64_t m = 0;
};
constexpr int MAX_ASYNC_SLOTS = 3;

struct ndt_ctx {
    HostPool pool;
    ndt_config cfg{};
    PendingAlign pend;
    AsyncSlot slots[MAX_ASYNC_SLOTS];
    uint64_t next_ticket = 0;
    bool borrowed_map = false;         // an async slot: map.view belongs to the owner
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t cstream = nullptr;  // host batches copied in while the work-queue kernel runs
    cudaEvent_t ev_in0 = nullptr, ev_in1 = nullptr;  // counter reset / last chunk copied
    Map map;
    BuildScratch bs;
    DevBuf d_in, d_jobs, d_aout, d_sjobs, d_sout, d_part, d_status, d_q, d_qidx, d_qcnt;
    PinBuf h_pts, h_jobs, h_aout, h_sjobs, h_sout, h_misc, h_arrive;
    double d1 = 0, d2 = 0;
    ndt_stats stats{};
    bool profile = false;
    bool trace = false;
    DevBuf d_trace;
    DevBuf d_qjobs, d_qctl, d_qframe, d_qpart, d_qoff;  // work-queue kernel
    std::vector<double> h_trace;       // last call's records, by job order
    std::vector<uint32_t> trace_slot;  // job index -> caller's result index
    int trace_iters = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr, ev3 = nullptr;
    LaunchShape forced{0, 0, 0, 0};                        // set only while autotuning
    std::map<std::pair<int, int>, LaunchShape> tuned;      // (log2 jobs, log2 max points)
    // captured batches, most recently used last; a key holds everything the captured
    // launches bake in (sizes, launch shape, buffer addresses, map and parameter versions)
    struct GraphEntry {
        std::vector<uint64_t> key;
        cudaGraphExec_t exec = nullptr;
    };
    std::vector<GraphEntry> graphs;
    uint64_t map_gen = 0, cfg_gen = 0;
    std::vector<double> t_start_ms, t_finish_ms;           // last call, by result index
    // map tiles and the background rebuild into the standby map
    struct Tile {
        uint64_t id;
        DevBuf pts;
        uint64_t n;
        TileSegs segs;           // the tile's segments (built on put)
        float seg_res = 0.f;     // map parameters the segments were built with
        int32_t seg_min = 0;
        float seg_ratio = 0.f;
    };
    std::vector<Tile> tiles;
    Map map_b;
    BuildScratch bs_b, bs_tile;
    DevBuf d_gather, d_status_b, d_tile_refs;
    float tile_put_ms = 0.f;     // device time of the last put's segment build
    uint64_t stall_ns = QSTALL_NS;  // work-queue no-progress limit (ndt_debug_queue_stall)
    int32_t withhold_next = 0;
    cudaStream_t bstream = nullptr;
    std::thread builder;
    std::atomic<int> build_state{0};  // 0 idle, 1 running, 2 finished
    int build_rc = 0;
    float build_ms_b = 0.f;
    std::string build_err;
};

// Waits for the asynchronous batches in flight (their results stay for ndt_batch_wait): the
// map they read must not change under them.
static void async_drain(ndt_ctx* c) {
    for (auto& s : c->slots)
        if (s.ticket && s.ctx) cudaStreamSynchronize(s.ctx->stream);
}

// Finishes a background rebuild: joins its thread and, when it succeeded, makes the standby
// map the active one (alignment work on the old map has completed: every call synchronises,
// and asynchronous batches are drained first).
static void tiles_settle(ndt_ctx* c, bool wait) {
    if (!c->builder.joinable()) return;
    if (!wait && c->build_state.load() != 2) return;
    c->builder.join();
    c->build_state.store(0);
    if (c->build_rc == 0) {
        async_drain(c);
        std::swap(c->map, c->map_b);
        c->map_b.valid = false;
        c->map_gen++;
        c->stats.build_launches++;
        c->stats.build_ms += c->build_ms_b;
    }
}

// Packs host scans into the pinned staging buffer with the context's host threads and copies
// them to the device in chunks of about 16 MB: each chunk's copy is issued as soon as that
// chunk is packed, so the DMA overlaps the packing of the next one.
static void stage_scans(ndt_ctx* c, const ndt_scan* scans, uint64_t m,
                        const std::vector<uint64_t>& offset, uint64_t total) {
    if (total == 0) return;
    char* hp = (char*)c->h_pts.p;
    const uint64_t chunk_pts = (16ull << 20) / 12;
    uint64_t i0 = 0;
    while (i0 < m) {
        uint64_t i1 = i0, pts = 0;
        while (i1 < m && (pts < chunk_pts || i1 == i0)) pts += scans[i1++].num_points;
        c->pool.run(i1 - i0, [&](uint64_t k) {
            const uint64_t i = i0 + k;
            std::memcpy(hp + offset[i] * 12, scans[i].xyz, scans[i].num_points * 12);
        });
        const uint64_t o0 = offset[i0], o1 = i1 < m ? offset[i1] : total;
        cudaMemcpyAsync((char*)c->d_in.p + o0 * 12, hp + o0 * 12, (o1 - o0) * 12,
                        cudaMemcpyHostToDevice, c->stream);
        i0 = i1;
    }
    c->stats.h2d_bytes += total * 12;
}

// Copies a planned batch to c->d_in on stream s: the context's host threads pack the scans
// into the pinned buffer in one pass (in launch order), and the thread that packs the last
// scan of a chunk issues that chunk's copy, chunks strictly in order (under a lock), so the
// copies overlap the packing with no barrier between chunks. With d_arrive, a 4-byte copy
// after each chunk sets that device word to the points resident so far (a prefix of the
// batch; c->h_arrive holds one value per chunk and is reserved by the caller).
static void stage_plan(ndt_ctx* c, const StagePlan& pl, const std::vector<AlignJob>& jobs,
                       cudaStream_t s, uint32_t* d_arrive) {
    const size_t nch = pl.chunk_job.size() - 1;
    const uint64_t m = pl.chunk_job.back();
    if (nch == 0 || m == 0) return;
    char* hp = (char*)c->h_pts.p;
    uint32_t* ha = (uint32_t*)c->h_arrive.p;
    std::unique_ptr<std::atomic<uint32_t>[]> left(new std::atomic<uint32_t>[nch]);
    for (size_t k = 0; k < nch; ++k) left[k].store(pl.chunk_job[k + 1] - pl.chunk_job[k]);
    std::vector<char> packed(nch, 0);
    size_t next = 0;
    std::mutex mu;
    const int dev = c->device;
    auto issue = [&](size_t k) {
        const uint32_t a = pl.chunk_job[k], b = pl.chunk_job[k + 1];
        const uint64_t o0 = jobs[a].offset, o1 = jobs[b - 1].offset + jobs[b - 1].n;
        if (o1 > o0) {
            cudaMemcpyAsync((char*)c->d_in.p + o0 * 12, hp + o0 * 12, (o1 - o0) * 12,
                            cudaMemcpyHostToDevice, s);
            c->stats.h2d_bytes += (o1 - o0) * 12;
        }
        if (d_arrive) {
            ha[k] = (uint32_t)o1;
            cudaMemcpyAsync(d_arrive, ha + k, 4, cudaMemcpyHostToDevice, s);
            c->stats.h2d_bytes += 4;
        }
    };
    c->pool.run(m, [&](uint64_t t) {
        const AlignJob& jb = jobs[t];
        if (jb.n) std::memcpy(hp + jb.offset * 12, pl.scans[jb.slot].xyz, (size_t)jb.n * 12);
        const size_t k = (size_t)(std::upper_bound(pl.chunk_job.begin(), pl.chunk_job.end(),
                                                   (uint32_t)t) -
                                  pl.chunk_job.begin()) - 1;
        if (left[k].fetch_sub(1) != 1) return;  // the chunk still has scans to pack
        std::lock_guard<std::mutex> lk(mu);
        packed[k] = 1;
        if (next < nch && packed[next]) cudaSetDevice(dev);  // this thread issues copies
        while (next < nch && packed[next]) issue(next++);
    });
}

static void drop_graphs(ndt_ctx* c) {
    for (auto& g : c->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

static int check_status(ndt_ctx* c, uint32_t st) {
    if (st == 0) return 0;
    uint32_t zero = 0;
    cudaMemcpyAsync(c->d_status.p, &zero, 4, cudaMemcpyHostToDevice, c->stream);
    cudaStreamSynchronize(c->stream);
    if (st & ST_HASH_FULL) {
        set_error("hash insert found no free slot");
        return NDT_ERR_HASH_FULL;
    }
    if (st & ST_PROBE_LIMIT) {
        set_error("hash probe exceeded its bound");
        return NDT_ERR_PROBE_LIMIT;
    }
    if (st & ST_QUEUE_STALL) {
        set_error("work-queue Newton kernel found no work for " +
                  std::to_string(c->stall_ns / 1000000ull) + " ms with alignments open");
        return NDT_ERR_DEVICE;
    }
    set_error("device reported status " + std::to_string(st));
    return NDT_ERR_DEVICE;
}

extern "C" {

const char* ndt_last_error_string(void) { return g_err.c_str(); }

int ndt_config_default(ndt_config* cfg) {
    if (!cfg) return NDT_ERR_INVALID_ARGUMENT;
    std::memset(cfg, 0, sizeof *cfg);
    cfg->resolution = 2.0f;
    cfg->max_iterations = 30;
    cfg->trans_epsilon = 0.01;
    cfg->step_size = 0.1;
    cfg->outlier_ratio = 0.55;
    cfg->min_points_per_voxel = 6;
    cfg->eigenvalue_ratio = 0.01f;
    cfg->max_neighbors = MAX_NB_GPU;
    cfg->semantics = NDT_SEMANTICS_GPU_GRAPH;
    cfg->min_correspondences = 10;
    cfg->device = 0;
    cfg->cluster_size = 0;
    cfg->threads_per_cta = 0;
    cfg->hash_capacity_factor = 2;
    return NDT_OK;
}

}  // extern "C"

// Parameter ranges shared by create and configure; launch-shape knobs are 0 (automatic) or
// one of the compiled variants.
static bool config_ok(const ndt_config& c) {
    const int K = c.cluster_size, T = c.threads_per_cta, R = c.max_registers;
    return c.resolution > 0.f && c.max_iterations >= 1 && c.max_neighbors >= 1 &&
           c.max_neighbors <= MAX_NB_ALL && c.step_size > 0.0 && c.outlier_ratio > 0.0 &&
           c.outlier_ratio < 1.0 &&
           (c.semantics == NDT_SEMANTICS_GPU_GRAPH || c.semantics == NDT_SEMANTICS_CPU) &&
           (K == 0 || K == 1 || K == 2 || K == 4 || K == 8) &&
           (T == 0 || T == 128 || T == 256 || T == 512) &&
           (R == 0 || R == 48 || R == 64 || R == 80 || R == 128) &&
           (c.cell_index == NDT_CELL_INDEX_AUTO || c.cell_index == NDT_CELL_INDEX_HASH ||
            c.cell_index == NDT_CELL_INDEX_OCTANT) &&
           (c.cuda_graph == 0 || c.cuda_graph == 1) &&
           (c.use_line_search == 0 || c.use_line_search == 1) &&
           c.work_queue >= -1 && c.work_queue <= 16 &&
           (c.work_queue <= 0 || (T != 128 || R == 0 || R == 64)) &&
           (c.work_queue <= 0 || (T != 512 || R == 0 || R == 128)) &&
           (c.work_queue <= 0 || (T != 256 || R == 0 || R == 64 || R == 80)) &&
           (c.lanes_per_point == 0 || c.lanes_per_point == 1 ||
            ((c.lanes_per_point == 2 || c.lanes_per_point == 4) &&
             c.semantics == NDT_SEMANTICS_GPU_GRAPH && (T == 0 || T == 256) &&
             (R == 0 || R == 64))) &&
           (c.stage_points == 0 || c.stage_points == 1);
}

extern "C" {

int ndt_ctx_create(const ndt_config* cfg, ndt_ctx** out) {
    if (!out) return NDT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    ndt_config c;
    if (cfg)
        c = *cfg;
    else
        ndt_config_default(&c);
    if (!config_ok(c)) {
        set_error("invalid configuration");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev <= c.device) {
        set_error("no CUDA device available");
        return NDT_ERR_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if ((e = cudaGetDeviceProperties(&prop, c.device)) != cudaSuccess) return cuda_fail(e, "device");
    if (!(prop.major == 10 && prop.minor == 3)) {
        set_error("libndt_gb300 is built for sm_103a; device " + std::string(prop.name) +
                  " has compute capability " + std::to_string(prop.major) + "." +
                  std::to_string(prop.minor));
        return NDT_ERR_NO_DEVICE;
    }
    if ((e = cudaSetDevice(c.device)) != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    ndt_ctx* x = new ndt_ctx();
    x->cfg = c;
    x->device = c.device;
    x->num_sms = prop.multiProcessorCount;
    if ((e = cudaStreamCreateWithFlags(&x->stream, cudaStreamNonBlocking)) != cudaSuccess) {
        delete x;
        return cuda_fail(e, "stream");
    }
    cudaEventCreate(&x->ev0);
    cudaEventCreate(&x->ev1);
    cudaEventCreate(&x->ev2);
    cudaEventCreate(&x->ev3);
    cudaStreamCreateWithFlags(&x->bstream, cudaStreamNonBlocking);
    cudaStreamCreateWithFlags(&x->cstream, cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&x->ev_in0, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&x->ev_in1, cudaEventDisableTiming);
    int rc = dev_reserve(x->d_status, 16);
    if (!rc) rc = dev_reserve(x->d_status_b, 16);
    if (rc) {
        delete x;
        return rc;
    }
    cudaMemsetAsync(x->d_status.p, 0, 16, x->stream);
    cudaMemsetAsync(x->d_status_b.p, 0, 16, x->stream);
    gauss_params((double)c.resolution, c.outlier_ratio, &x->d1, &x->d2);
    *out = x;
    return NDT_OK;
}

int ndt_ctx_destroy(ndt_ctx* c) {
    if (!c) return NDT_OK;
    cudaSetDevice(c->device);
    async_drain(c);
    for (auto& s : c->slots)
        if (s.ctx) ndt_ctx_destroy(s.ctx);  // a slot's map is borrowed: its Map owns nothing
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->cstream) cudaStreamSynchronize(c->cstream);
    if (c->builder.joinable()) c->builder.join();
    for (auto& t : c->tiles)
        for (DevBuf* b : {&t.pts, &t.segs.idx, &t.segs.starts, &t.segs.rec, &t.segs.valid})
            dev_free(*b);
    for (DevBuf* b : {&c->bs_tile.keys_a, &c->bs_tile.keys_b, &c->bs_tile.vals_a,
                      &c->bs_tile.vals_b, &c->bs_tile.tmp, &c->bs_tile.seg_ids,
                      &c->bs_tile.seg_starts, &c->bs_tile.seg_valid, &c->bs_tile.seg_rank,
                      &c->bs_tile.seg_rec, &c->bs_tile.small, &c->d_tile_refs})
        dev_free(*b);
    for (DevBuf* b : {&c->map_b.slots, &c->map_b.slot_icov, &c->map_b.slot_vidx, &c->map_b.grid,
                      &c->map_b.nmask,
                      &c->map_b.vox_coord, &c->map_b.vox_mean, &c->map_b.vox_cov,
                      &c->map_b.vox_icov, &c->map_b.vox_count, &c->bs_b.keys_a, &c->bs_b.keys_b,
                      &c->bs_b.vals_a, &c->bs_b.vals_b, &c->bs_b.tmp, &c->bs_b.seg_ids,
                      &c->bs_b.seg_starts, &c->bs_b.seg_valid, &c->bs_b.seg_rank,
                      &c->bs_b.seg_rec, &c->bs_b.small, &c->d_gather, &c->d_status_b})
        dev_free(*b);
    if (c->bstream) cudaStreamDestroy(c->bstream);
    drop_graphs(c);
    for (DevBuf* b : {&c->map.slots, &c->map.slot_icov, &c->map.slot_vidx, &c->map.grid,
                      &c->map.nmask,
                      &c->map.vox_coord,
                      &c->map.vox_mean, &c->map.vox_cov, &c->map.vox_icov, &c->map.vox_count,
                      &c->bs.keys_a, &c->bs.keys_b, &c->bs.vals_a, &c->bs.vals_b, &c->bs.tmp,
                      &c->bs.seg_ids, &c->bs.seg_starts, &c->bs.seg_valid, &c->bs.seg_rank,
                      &c->bs.seg_rec, &c->bs.small, &c->d_in, &c->d_jobs, &c->d_aout,
                      &c->d_sjobs, &c->d_sout, &c->d_part, &c->d_status, &c->d_q, &c->d_qidx,
                      &c->d_qcnt, &c->d_trace, &c->d_qjobs, &c->d_qctl, &c->d_qframe,
                      &c->d_qpart, &c->d_qoff})
        dev_free(*b);
    for (PinBuf* b : {&c->h_pts, &c->h_jobs, &c->h_aout, &c->h_sjobs, &c->h_sout, &c->h_misc,
                      &c->h_arrive})
        pin_free(*b);
    for (cudaEvent_t ev : {c->ev0, c->ev1, c->ev2, c->ev3, c->ev_in0, c->ev_in1})
        if (ev) cudaEventDestroy(ev);
    if (c->cstream) cudaStreamDestroy(c->cstream);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return NDT_OK;
}

void* ndt_ctx_stream(ndt_ctx* c) { return c ? (void*)c->stream : nullptr; }

int ndt_ctx_configure(ndt_ctx* c, const ndt_config* cfg) {
    if (!c || !cfg) return NDT_ERR_INVALID_ARGUMENT;
    tiles_settle(c, true);  // a running rebuild reads the configuration
    const ndt_config& n = *cfg;
    if (!config_ok(n) || n.device != c->cfg.device) {
        set_error("invalid configuration");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    if (c->map.valid && n.resolution != c->map.view.res) {
        set_error("resolution changes need a new set_target");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    c->cfg = n;
    c->cfg_gen++;
    gauss_params((double)n.resolution, n.outlier_ratio, &c->d1, &c->d2);
    return NDT_OK;
}

int ndt_profile_enable(ndt_ctx* c, int enable) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    c->profile = enable != 0;
    return NDT_OK;
}

int ndt_debug_queue_stall(ndt_ctx* c, uint64_t limit_ns, int32_t withhold_next) {
    if (!c || (withhold_next != 0 && withhold_next != 1)) return NDT_ERR_INVALID_ARGUMENT;
    c->stall_ns = limit_ns ? limit_ns : QSTALL_NS;
    c->withhold_next = withhold_next;
    c->cfg_gen++;  // captured batches bake the limit in
    return NDT_OK;
}

int ndt_debug_trace(ndt_ctx* c, int enable) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    c->trace = enable != 0;
    return NDT_OK;
}

int ndt_debug_read(ndt_ctx* c, uint64_t index, double* out, int32_t max_records,
                   int32_t* num_records) {
    if (!c || !out || !num_records) return NDT_ERR_INVALID_ARGUMENT;
    *num_records = 0;
    for (size_t j = 0; j < c->trace_slot.size(); ++j) {
        if (c->trace_slot[j] != index) continue;
        const double* src = c->h_trace.data() + j * (size_t)c->trace_iters * TRACE_REC;
        int n = 0;
        for (int it = 0; it < c->trace_iters && it < max_records; ++it) {
            if (src[it * TRACE_REC] != src[it * TRACE_REC]) break;  // NaN: not run
            std::memcpy(out + (size_t)it * TRACE_REC, src + (size_t)it * TRACE_REC,
                        TRACE_REC * sizeof(double));
            n++;
        }
        *num_records = n;
        return NDT_OK;
    }
    set_error("no trace for that result index (enable ndt_debug_trace before aligning)");
    return NDT_ERR_INVALID_ARGUMENT;
}

int ndt_stats_get(ndt_ctx* c, ndt_stats* out) {
    if (!c || !out) return NDT_ERR_INVALID_ARGUMENT;
    *out = c->stats;
    return NDT_OK;
}

int ndt_stats_reset(ndt_ctx* c) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    std::memset(&c->stats, 0, sizeof c->stats);
    return NDT_OK;
}

static int set_target_dev(ndt_ctx* c, const float* d_xyz, uint64_t n) {
    tiles_settle(c, true);
    async_drain(c);  // batches in flight read the map being rebuilt in place
    c->map.valid = false;
    c->map_gen++;  // captured batches bake the map in
    float ms = 0.f;
    int rc = build_map(c->map, c->bs, d_xyz, (size_t)n, c->cfg, (uint32_t*)c->d_status.p,
                       c->stream, &ms);
    if (rc) return rc;
    uint32_t st = 0;
    cudaMemcpyAsync(&st, c->d_status.p, 4, cudaMemcpyDeviceToHost, c->stream);
    if ((rc = cuda_fail(cudaStreamSynchronize(c->stream), "set_target"))) return rc;
    if ((rc = check_status(c, st))) {
        c->map.valid = false;
        return rc;
    }
    c->stats.build_launches++;
    c->stats.build_ms += ms;
    return NDT_OK;
}

int ndt_set_target(ndt_ctx* c, const float* xyz, uint64_t n) {
    if (!c || (!xyz && n)) return NDT_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    cudaSetDevice(c->device);
    int rc = dev_reserve(c->d_in, n * 12);
    if (rc) return rc;
    rc = cuda_fail(cudaMemcpyAsync(c->d_in.p, xyz, n * 12, cudaMemcpyHostToDevice, c->stream),
                   "target upload");
    if (rc) return rc;
    c->stats.h2d_bytes += n * 12;
    return set_target_dev(c, (const float*)c->d_in.p, n);
}

int ndt_set_target_device(ndt_ctx* c, const float* d_xyz, uint64_t n) {
    if (!c || (!d_xyz && n)) return NDT_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    cudaSetDevice(c->device);
    return set_target_dev(c, d_xyz, n);
}

// Builds a tile's segments (cells, counts, FP64 statistics) with the context's current map
// parameters, on the tile stream.
static int tile_segments(ndt_ctx* c, ndt_ctx::Tile& t) {
    float ms = 0.f;
    const int rc = build_tile_segments(c->bs_tile, (const float*)t.pts.p, (size_t)t.n, c->cfg,
                                       c->bstream, t.segs, &ms);
    if (rc) return rc;
    t.seg_res = c->cfg.resolution;
    t.seg_min = c->cfg.min_points_per_voxel;
    t.seg_ratio = c->cfg.eigenvalue_ratio;
    c->tile_put_ms = ms;
    c->stats.build_ms += ms;
    return 0;
}

int ndt_tile_put(ndt_ctx* c, uint64_t tile_id, const float* xyz, uint64_t n) {
    if (!c || (!xyz && n)) return NDT_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    if (n >= 0xFFFFFFF0ull) {
        set_error("a tile holds fewer than 2^32 points");
        return NDT_ERR_CAPACITY;
    }
    cudaSetDevice(c->device);
    ndt_ctx::Tile* t = nullptr;
    for (auto& x : c->tiles)
        if (x.id == tile_id) t = &x;
    if (t) {
        tiles_settle(c, true);  // a running merge reads this tile's buffers
    } else {
        c->tiles.push_back(ndt_ctx::Tile{});
        t = &c->tiles.back();
        t->id = tile_id;
    }
    int rc = dev_reserve(t->pts, n * 12);
    if (rc) return rc;
    t->n = n;
    cudaMemcpyAsync(t->pts.p, xyz, n * 12, cudaMemcpyHostToDevice, c->bstream);
    c->stats.h2d_bytes += n * 12;
    if ((rc = cuda_fail(cudaStreamSynchronize(c->bstream), "tile upload"))) return rc;
    return tile_segments(c, *t);
}

int ndt_tile_remove(ndt_ctx* c, uint64_t tile_id) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < c->tiles.size(); ++i)
        if (c->tiles[i].id == tile_id) {
            tiles_settle(c, true);  // a running merge reads the tile's buffers
            ndt_ctx::Tile& t = c->tiles[i];
            for (DevBuf* b : {&t.pts, &t.segs.idx, &t.segs.starts, &t.segs.rec, &t.segs.valid})
                dev_free(*b);
            c->tiles.erase(c->tiles.begin() + (long)i);
            return NDT_OK;
        }
    set_error("no such tile");
    return NDT_ERR_INVALID_ARGUMENT;
}

int ndt_tiles_commit(ndt_ctx* c, int32_t wait) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    tiles_settle(c, true);  // one rebuild at a time
    async_drain(c);         // the rebuild reuses the standby map's buffers
    uint64_t total = 0;
    for (auto& t : c->tiles) total += t.n;
    if (total == 0) {
        set_error("no tiles to build a map from");
        return NDT_ERR_EMPTY_INPUT;
    }
    cudaSetDevice(c->device);
    int rc;
    // tiles whose segments were built with other map parameters are rebuilt first
    for (auto& t : c->tiles)
        if (t.seg_res != c->cfg.resolution || t.seg_min != c->cfg.min_points_per_voxel ||
            t.seg_ratio != c->cfg.eigenvalue_ratio)
            if ((rc = tile_segments(c, t))) return rc;
    std::vector<TileSegRef> refs;
    uint64_t off = 0;
    for (auto& t : c->tiles) {
        TileSegRef r{};
        r.rec = (const SegRec*)t.segs.rec.p;
        r.valid = (const uint32_t*)t.segs.valid.p;
        r.starts = (const uint32_t*)t.segs.starts.p;
        r.idx = (const uint32_t*)t.segs.idx.p;
        r.pts = (const float*)t.pts.p;
        r.seg_off = off;
        r.S = t.segs.geo.S;
        r.nf = (uint32_t)t.segs.geo.nf;
        for (int a = 0; a < 3; ++a) {
            r.mn[a] = t.segs.geo.mn[a];
            r.mx[a] = t.segs.geo.mx[a];
        }
        off += r.S;
        refs.push_back(r);
    }
    c->build_state.store(1);
    const ndt_config cfg = c->cfg;
    c->builder = std::thread([c, refs, cfg]() {
        cudaSetDevice(c->device);
        float ms = 0.f;
        int r = merge_tiles(c->map_b, c->bs_b, refs, c->d_tile_refs, cfg,
                            (uint32_t*)c->d_status_b.p, c->bstream, &ms);
        uint32_t st = 0;
        if (!r) {
            cudaMemcpyAsync(&st, c->d_status_b.p, 4, cudaMemcpyDeviceToHost, c->bstream);
            r = cuda_fail(cudaStreamSynchronize(c->bstream), "tile rebuild");
        }
        if (!r && st) {
            uint32_t zero = 0;
            cudaMemcpyAsync(c->d_status_b.p, &zero, 4, cudaMemcpyHostToDevice, c->bstream);
            cudaStreamSynchronize(c->bstream);
            set_error("device reported status " + std::to_string(st) + " during a tile rebuild");
            r = NDT_ERR_DEVICE;
        }
        c->build_rc = r;
        c->build_ms_b = ms;
        c->build_err = r ? std::string(ndt_last_error_string()) : std::string();
        c->build_state.store(2);
    });
    if (wait) {
        tiles_settle(c, true);
        if (c->build_rc) {
            set_error(c->build_err);
            return c->build_rc;
        }
    }
    return NDT_OK;
}

int ndt_tiles_status(ndt_ctx* c, uint64_t* num_tiles, uint64_t* num_points, int32_t* pending,
                     int32_t* last_rc, float* build_ms, float* put_ms) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    if (put_ms) *put_ms = c->tile_put_ms;
    uint64_t n = 0;
    for (auto& t : c->tiles) n += t.n;
    if (num_tiles) *num_tiles = c->tiles.size();
    if (num_points) *num_points = n;
    if (pending) *pending = c->build_state.load() == 1 ? 1 : 0;
    if (last_rc) *last_rc = c->build_state.load() == 1 ? 0 : c->build_rc;
    if (build_ms) *build_ms = c->build_ms_b;
    return NDT_OK;
}

int ndt_map_info_get(ndt_ctx* c, ndt_map_info* out) {
    if (!c || !out) return NDT_ERR_INVALID_ARGUMENT;
    tiles_settle(c, false);
    if (!c->map.valid) {
        set_error("No target set. Call set_target() first.");
        return NDT_ERR_NO_TARGET;
    }
    *out = c->map.info;
    return NDT_OK;
}

int ndt_map_voxels(ndt_ctx* c, int32_t* coords, float* means, float* covs, float* icovs,
                   uint32_t* counts, uint64_t capacity) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    tiles_settle(c, false);
    if (!c->map.valid) {
        set_error("No target set. Call set_target() first.");
        return NDT_ERR_NO_TARGET;
    }
    uint64_t V = c->map.info.num_voxels;
    if (capacity < V) {
        set_error("output capacity below the number of voxels");
        return NDT_ERR_CAPACITY;
    }
    cudaSetDevice(c->device);
    cudaStream_t s = c->stream;
    if (coords) cudaMemcpyAsync(coords, c->map.vox_coord.p, V * 12, cudaMemcpyDeviceToHost, s);
    if (covs) cudaMemcpyAsync(covs, c->map.vox_cov.p, V * 36, cudaMemcpyDeviceToHost, s);
    if (icovs) cudaMemcpyAsync(icovs, c->map.vox_icov.p, V * 36, cudaMemcpyDeviceToHost, s);
    if (counts) cudaMemcpyAsync(counts, c->map.vox_count.p, V * 4, cudaMemcpyDeviceToHost, s);
    std::vector<float> m4;
    if (means) {
        m4.resize(V * 4);
        cudaMemcpyAsync(m4.data(), c->map.vox_mean.p, V * 16, cudaMemcpyDeviceToHost, s);
    }
    int rc = cuda_fail(cudaStreamSynchronize(s), "map readback");
    if (rc) return rc;
    if (means)
        for (uint64_t v = 0; v < V; ++v) {
            means[3 * v] = m4[4 * v];
            means[3 * v + 1] = m4[4 * v + 1];
            means[3 * v + 2] = m4[4 * v + 2];
        }
    return NDT_OK;
}

}  // extern "C"

// Launch shape: enough CTAs to fill the GPU twice over, at least ~1k points per CTA.
static int log2_bucket(uint64_t v) {
    int b = 0;
    while ((1ull << b) < v && b < 63) ++b;
    return b;
}

// Launch shape: an explicit configuration wins, then an autotuned entry for this
// (batch size, scan size) bucket, then the default: 512-thread CTAs for large scans, and
// clusters doubled until the launch covers about three CTAs per SM while keeping at least
// two points per thread per CTA.
// The work-queue kernel is used when the configuration asks for it (work_queue > 0) or the
// autotuner picked it, never with line search.
static LaunchShape choose_shape(ndt_ctx* c, uint32_t jobs, uint32_t max_n) {
    LaunchShape sh{0, 0, 128, 0};
    if (c->forced.cluster > 0) return c->forced;
    const bool ls = c->cfg.use_line_search != 0;
    if (c->cfg.work_queue > 0 && !ls) {
        sh.cluster = 1;
        sh.threads = c->cfg.threads_per_cta > 0 ? c->cfg.threads_per_cta : 256;
        sh.regcap = c->cfg.max_registers > 0 ? c->cfg.max_registers : (sh.threads == 512 ? 128 : 64);
        sh.queue = c->cfg.work_queue;
        sh.npw = c->cfg.lanes_per_point > 1 ? c->cfg.lanes_per_point : 1;
        sh.stage = c->cfg.stage_points > 0 ? 1 : 0;
        return sh;
    }
    auto it = c->tuned.find({log2_bucket(jobs), log2_bucket(max_n)});
    if (it != c->tuned.end() && c->cfg.cluster_size <= 0 && c->cfg.threads_per_cta <= 0 &&
        !(it->second.queue > 0 && (ls || c->cfg.work_queue < 0)))
        return it->second;
    sh.threads = c->cfg.threads_per_cta > 0
                     ? c->cfg.threads_per_cta
                     : (max_n >= 4096 ? 512 : (max_n >= 1024 ? 256 : 128));
    if (c->cfg.max_registers > 0 && sh.threads <= 256) sh.regcap = c->cfg.max_registers;
    if (c->cfg.cluster_size > 0) {
        sh.cluster = c->cfg.cluster_size;
        return sh;
    }
    int K = 1;
    while (K < 8 && (uint64_t)jobs * K < 3ull * (uint64_t)c->num_sms &&
           max_n / (uint32_t)(2 * K) >= (uint32_t)sh.threads * 2)
        K *= 2;
    sh.cluster = K;
    return sh;
}

// Core: align jobs whose points are at d_pts (device, concatenated), or, with a plan, host
// scans that are copied to d_pts (c->d_in) first. Enqueues the batch on the context's stream
// (job tables in, Newton kernel, NVTL scoring, results out) and records what
// run_align_finish needs in c->pend. With the work-queue kernel, a planned batch of more than
// one copy chunk is copied in on c->cstream while the kernel already runs (see k_ndt_queue);
// otherwise its copies precede the launch on the stream.
static int run_align_enqueue(ndt_ctx* c, const float* d_pts, std::vector<AlignJob>& jobs,
                             const std::vector<uint64_t>& n_by_slot,
                             const StagePlan* plan = nullptr) {
    uint32_t nj = (uint32_t)jobs.size();
    c->pend.active = false;
    if (nj == 0) return NDT_OK;
    std::stable_sort(jobs.begin(), jobs.end(),
                     [](const AlignJob& a, const AlignJob& b) { return a.n > b.n; });
    uint32_t max_n = jobs.front().n;
    int rc;
    size_t jb = nj * sizeof(AlignJob), ob = nj * sizeof(AlignOut), sjb = nj * sizeof(ScoreJob),
           sob = nj * sizeof(ScoreOut);
    if ((rc = dev_reserve(c->d_jobs, jb)) || (rc = dev_reserve(c->d_aout, ob)) ||
        (rc = dev_reserve(c->d_sjobs, sjb)) || (rc = dev_reserve(c->d_sout, sob)) ||
        (rc = dev_reserve(c->d_part, score_part_bytes(nj, max_n))) ||
        (rc = pin_reserve(c->h_jobs, jb + sjb)) || (rc = pin_reserve(c->h_aout, ob + sob + 16)))
        return rc;
    AlignJob* hj = (AlignJob*)c->h_jobs.p;
    ScoreJob* hs = (ScoreJob*)((char*)c->h_jobs.p + jb);
    for (uint32_t j = 0; j < nj; ++j) {
        hj[j] = jobs[j];
        ScoreJob s{};
        s.offset = jobs[j].offset;
        s.n = jobs[j].n;
        s.pose_src = 1;
        s.out_index = j;
        hs[j] = s;
    }
    cudaStream_t st = c->stream;
    c->stats.h2d_bytes += jb + sjb;
    AlignParams p{};
    p.map = c->map.view;
    p.pts = d_pts;
    p.jobs = (const AlignJob*)c->d_jobs.p;
    p.out = (AlignOut*)c->d_aout.p;
    p.num_jobs = nj;
    p.max_iter = c->cfg.max_iterations;
    bool cpu = c->cfg.semantics == NDT_SEMANTICS_CPU;
    p.semantics = c->cfg.semantics;
    p.max_nb = cpu ? MAX_NB_ALL : c->cfg.max_neighbors;
    p.min_corr = c->cfg.min_correspondences;
    p.d1 = c->d1;
    p.d2 = c->d2;
    p.d1f = (float)c->d1;
    p.d2f = (float)c->d2;
    p.step_size = c->cfg.step_size;
    if (cpu) {
        p.eps = c->cfg.trans_epsilon;
    } else {  // K5: step_len < sqrtf(epsilon_sq), epsilon_sq = (f32 eps)^2
        float ef = (float)c->cfg.trans_epsilon;
        p.eps = (double)sqrtf(ef * ef);
    }
    p.status = (uint32_t*)c->d_status.p;
    p.stall_ns = c->stall_ns;
    p.withhold = c->withhold_next;
    c->withhold_next = 0;
    // line search: the graph path's candidates, or (CPU path) the More-Thuente search
    p.ls_cands = c->cfg.use_line_search ? LS_MAX : 0;
    p.ls_mu = LS_MU;
    p.ls_nu = LS_NU;
    p.trace = nullptr;
    if (c->trace) {
        size_t tb = (size_t)nj * p.max_iter * TRACE_REC * sizeof(double);
        if ((rc = dev_reserve(c->d_trace, tb))) return rc;
        cudaMemsetAsync(c->d_trace.p, 0xFF, tb, st);  // NaN marks iterations not run
        p.trace = (double*)c->d_trace.p;
    }
    LaunchShape shape = choose_shape(c, nj, max_n);
    // work-queue kernel: chunk counts and partial-sum offsets per alignment (host, in the
    // pinned job block), per-alignment state and the partials (device)
    size_t qob = 0;
    uint32_t* hq = nullptr;
    if (shape.queue > 0) {
        const uint32_t chunk = (uint32_t)(shape.threads * shape.queue);
        qob = (size_t)nj * sizeof(uint32_t);
        if ((rc = pin_reserve(c->h_jobs, jb + sjb + qob))) return rc;
        hj = (AlignJob*)c->h_jobs.p;  // the block may have moved: refill it
        hs = (ScoreJob*)((char*)c->h_jobs.p + jb);
        for (uint32_t j = 0; j < nj; ++j) {
            hj[j] = jobs[j];
            ScoreJob s{};
            s.offset = jobs[j].offset;
            s.n = jobs[j].n;
            s.pose_src = 1;
            s.out_index = j;
            hs[j] = s;
        }
        hq = (uint32_t*)((char*)c->h_jobs.p + jb + sjb);
        // partial-sum slots per alignment: its chunk count at the smallest (last iterations')
        // chunk size, the most an iteration uses, capped at the 16-bit count of the claim word
        const uint32_t small = std::max(1u, chunk / (2 * QSPLIT_DIV));
        uint64_t total = 0, full = 0;
        for (uint32_t j = 0; j < nj; ++j) {
            hq[j] = (uint32_t)total;
            const uint64_t n = jobs[j].n;
            total += std::min<uint64_t>(n ? (n + small - 1) / small : 1, QMAXCH);
            full += std::min<uint64_t>(n ? (n + chunk - 1) / chunk : 1, QMAXCH);
        }
        if (total > 0xFFFFFFFFull) {
            set_error("too many chunks in one batch");
            return NDT_ERR_CAPACITY;
        }
        if ((rc = dev_reserve(c->d_qjobs, (size_t)nj * sizeof(QJob))) ||
            (rc = dev_reserve(c->d_qctl, (size_t)nj * sizeof(QCtl))) ||
            (rc = dev_reserve(c->d_qframe, (size_t)nj * 52 * sizeof(float))) ||
            (rc = dev_reserve(c->d_qoff, qob)) ||
            (rc = dev_reserve(c->d_qpart, (size_t)total * NRED * sizeof(double))))
            return rc;
        p.qjobs = (QJob*)c->d_qjobs.p;
        p.qctl = (QCtl*)c->d_qctl.p;
        p.qframe = (float*)c->d_qframe.p;
        p.qpart = (double*)c->d_qpart.p;
        p.qpart_off = (const uint32_t*)c->d_qoff.p;
        p.qcount = (uint32_t*)c->d_status.p + 2;  // word 2 of the status block
        p.qchunks_total = (uint32_t)full;
        c->stats.h2d_bytes += qob;
    }
    AlignOut* ho = (AlignOut*)c->h_aout.p;
    ScoreOut* hso = (ScoreOut*)((char*)c->h_aout.p + ob);
    uint32_t* hst = (uint32_t*)((char*)c->h_aout.p + ob + sob);
    // host batch copied in during the launch: the kernel reads the resident-point count from
    // word 3 of the status block (32-bit: the batch holds fewer than 2^32 points)
    const bool stream_in = plan && shape.queue > 0 && !c->trace &&
                           plan->chunk_job.size() > 2 && plan->total < 0xFFFFFFFFull;
    if (plan && !stream_in) stage_plan(c, *plan, jobs, st, nullptr);
    uint32_t* d_arrive = nullptr;
    if (stream_in) {
        if ((rc = pin_reserve(c->h_arrive, plan->chunk_job.size() * 4))) return rc;
        d_arrive = (uint32_t*)c->d_status.p + 3;
        p.qarrive = d_arrive;
        p.qarrive_total = (uint32_t)plan->total;
    }
    // the batch on the stream: job tables in, Newton kernel, NVTL scoring, results out (the
    // events are graph nodes when captured)
    auto enqueue = [&](unsigned evf) -> int {
        cudaMemcpyAsync(c->d_jobs.p, hj, jb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(c->d_sjobs.p, hs, sjb, cudaMemcpyHostToDevice, st);
        if (shape.queue > 0) {
            cudaMemcpyAsync(c->d_qoff.p, hq, qob, cudaMemcpyHostToDevice, st);
            cudaMemsetAsync(p.qcount, 0, d_arrive ? 8 : 4, st);  // words 2 (and 3)
        }
        if (d_arrive) cudaEventRecord(c->ev_in0, st);  // the counter is reset
        cudaEventRecordWithFlags(c->ev0, st, evf);
        int r = launch_align(p, shape, st);
        if (r) return r;
        cudaEventRecordWithFlags(c->ev1, st, evf);
        if (d_arrive) {
            // the points, while the kernel runs; then, after the last chunk, the continuation
            // launch (it finds nothing left unless the first launch ran out of input) and
            // scoring
            cudaStreamWaitEvent(c->cstream, c->ev_in0, 0);
            stage_plan(c, *plan, jobs, c->cstream, d_arrive);
            cudaEventRecord(c->ev_in1, c->cstream);
            cudaStreamWaitEvent(st, c->ev_in1, 0);
            AlignParams pr = p;
            pr.qarrive = nullptr;
            pr.qresume = 1;
            if ((r = launch_align(pr, shape, st))) return r;
            cudaEventRecordWithFlags(c->ev1, st, evf);
        }
        r = launch_score(c->map.view, d_pts, (const ScoreJob*)c->d_sjobs.p, nj, max_n,
                         (const AlignOut*)c->d_aout.p, c->d_part.p, (ScoreOut*)c->d_sout.p,
                         (float)c->d1, (float)c->d2, st);
        if (r) return r;
        cudaEventRecordWithFlags(c->ev2, st, evf);
        cudaMemcpyAsync(ho, c->d_aout.p, ob, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(hso, c->d_sout.p, sob, cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(hst, c->d_status.p, 4, cudaMemcpyDeviceToHost, st);
        return cuda_fail(cudaGetLastError(), "align enqueue");
    };
    if (c->cfg.cuda_graph && !c->trace && !stream_in) {
        const std::vector<uint64_t> key = {
            nj, max_n, (uint64_t)shape.cluster, (uint64_t)shape.threads, (uint64_t)shape.regcap,
            (uint64_t)shape.queue, (uint64_t)shape.npw, (uint64_t)shape.stage,
            (uint64_t)(uintptr_t)c->d_qjobs.p,
            (uint64_t)(uintptr_t)c->d_qctl.p, (uint64_t)(uintptr_t)c->d_qframe.p,
            (uint64_t)(uintptr_t)c->d_qpart.p, (uint64_t)(uintptr_t)c->d_qoff.p,
            c->map_gen, c->cfg_gen, (uint64_t)(uintptr_t)d_pts, (uint64_t)(uintptr_t)c->d_jobs.p,
            (uint64_t)(uintptr_t)c->d_aout.p, (uint64_t)(uintptr_t)c->d_sjobs.p,
            (uint64_t)(uintptr_t)c->d_sout.p, (uint64_t)(uintptr_t)c->d_part.p,
            (uint64_t)(uintptr_t)c->h_jobs.p, (uint64_t)(uintptr_t)c->h_aout.p};
        size_t gi = c->graphs.size();
        for (size_t i = 0; i < c->graphs.size(); ++i)
            if (c->graphs[i].key == key) gi = i;
        if (gi == c->graphs.size()) {
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return cuda_fail(e, "graph capture");
            rc = enqueue(cudaEventRecordExternal);  // event nodes inside the graph
            e = cudaStreamEndCapture(st, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e != cudaSuccess) return cuda_fail(e, "graph capture");
            cudaGraphExec_t exec = nullptr;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
            if (c->graphs.size() >= 8) {
                cudaGraphExecDestroy(c->graphs.front().exec);
                c->graphs.erase(c->graphs.begin());
            }
            c->graphs.push_back({key, exec});
            gi = c->graphs.size() - 1;
        } else if (gi + 1 != c->graphs.size()) {  // most recently used last
            auto g = c->graphs[gi];
            c->graphs.erase(c->graphs.begin() + (long)gi);
            c->graphs.push_back(g);
            gi = c->graphs.size() - 1;
        }
        if ((rc = cuda_fail(cudaGraphLaunch(c->graphs[gi].exec, st), "graph launch"))) return rc;
    } else if ((rc = enqueue(cudaEventRecordDefault))) {
        return rc;
    }
    c->stats.d2h_bytes += ob + sob + 4;
    PendingAlign& pd = c->pend;
    pd.jobs = jobs;
    pd.n_by_slot = n_by_slot;
    pd.max_iter = p.max_iter;
    pd.cpu = cpu;
    pd.ob = ob;
    pd.sob = sob;
    pd.active = true;
    return NDT_OK;
}

// Waits for the batch run_align_enqueue put on the stream and writes its results (caller's
// order) to out.
static int run_align_finish(ndt_ctx* c, ndt_result* out) {
    PendingAlign& pd = c->pend;
    if (!pd.active) return NDT_OK;
    pd.active = false;
    int rc;
    const std::vector<AlignJob>& jobs = pd.jobs;
    const std::vector<uint64_t>& n_by_slot = pd.n_by_slot;
    const uint32_t nj = (uint32_t)jobs.size();
    const bool cpu = pd.cpu;
    const AlignOut* ho = (const AlignOut*)c->h_aout.p;
    const ScoreOut* hso = (const ScoreOut*)((char*)c->h_aout.p + pd.ob);
    const uint32_t* hst = (const uint32_t*)((char*)c->h_aout.p + pd.ob + pd.sob);
    if ((rc = cuda_fail(cudaStreamSynchronize(c->stream), "align"))) return rc;
    if ((rc = check_status(c, *hst))) return rc;
    if (c->trace) {
        c->trace_iters = pd.max_iter;
        c->h_trace.resize((size_t)nj * pd.max_iter * TRACE_REC);
        cudaMemcpy(c->h_trace.data(), c->d_trace.p, c->h_trace.size() * sizeof(double),
                   cudaMemcpyDeviceToHost);
        c->trace_slot.resize(nj);
        for (uint32_t j = 0; j < nj; ++j) c->trace_slot[j] = jobs[j].slot;
    }
    float ams = 0.f, sms = 0.f;
    cudaEventElapsedTime(&ams, c->ev0, c->ev1);
    cudaEventElapsedTime(&sms, c->ev1, c->ev2);
    c->stats.align_launches++;
    c->stats.align_kernel_ms += ams;
    c->stats.score_launches++;
    c->stats.score_kernel_ms += sms;
    uint64_t t0 = UINT64_MAX;
    for (uint32_t j = 0; j < nj; ++j) t0 = std::min(t0, ho[j].t_start);
    c->t_start_ms.assign(nj, 0.0);
    c->t_finish_ms.assign(nj, 0.0);
    for (uint32_t j = 0; j < nj; ++j) {
        const AlignOut& o = ho[j];
        const ScoreOut& so = hso[j];
        c->t_start_ms[jobs[j].slot] = (double)(o.t_start - t0) * 1e-6;
        c->t_finish_ms[jobs[j].slot] = (double)(o.t_end - t0) * 1e-6;
        ndt_result& r = out[jobs[j].slot];
        std::memset(&r, 0, sizeof r);
        for (int i = 0; i < 6; ++i) r.pose[i] = o.pose[i];
        r.score = o.score;
        for (int i = 0; i < 36; ++i) r.hessian[i] = o.hessian[i];
        r.converged = o.converged;
        r.iterations = o.iterations;
        r.num_correspondences = o.ncorr;
        r.oscillation_count = o.osc;
        r.status = o.status;
        uint64_t nsrc = n_by_slot[jobs[j].slot];
        bool nocorr_early = cpu && o.status == NDT_STATUS_NO_CORRESPONDENCES;
        r.transform_probability = (nsrc && !nocorr_early) ? o.score / (double)nsrc : 0.0;
        r.nvtl = (!nocorr_early && so.nvtl_count) ? so.nvtl_sum / (double)so.nvtl_count : 0.0;
        c->stats.alignments++;
        c->stats.iterations += (uint64_t)std::max(o.iterations, 0);
        c->stats.point_iterations += o.point_iters;
        c->stats.correspondences += o.corr_total;
        c->stats.cycles_points += o.cycles[0];
        c->stats.cycles_cluster_wait += o.cycles[1];
        c->stats.cycles_control += o.cycles[2];
        c->stats.cycles_broadcast += o.cycles[3];
        c->stats.eigen_solves += (uint64_t)o.n_eigen;
    }
    return NDT_OK;
}

static int run_align(ndt_ctx* c, const float* d_pts, std::vector<AlignJob>& jobs,
                     const std::vector<uint64_t>& n_by_slot, ndt_result* out,
                     const StagePlan* plan = nullptr) {
    const int rc = run_align_enqueue(c, d_pts, jobs, n_by_slot, plan);
    return rc ? rc : run_align_finish(c, out);
}

static int need_target(ndt_ctx* c) {
    tiles_settle(c, false);
    if (!c->map.valid) {
        set_error("No target set. Call set_target() first.");
        return NDT_ERR_NO_TARGET;
    }
    return 0;
}

extern "C" {

}  // extern "C"

// Host scans of a batch: checked, described as jobs in launch order (largest scan first,
// the caller's order among equal sizes) and laid out in x->d_in for copying in chunks (the
// copies are issued by run_align_enqueue).
static int prepare_batch(ndt_ctx* x, const ndt_scan* scans, uint64_t m,
                         std::vector<AlignJob>& jobs, std::vector<uint64_t>& ns,
                         StagePlan& plan) {
    if (m > 0xFFFFFFull) {
        set_error("too many scans in one batch");
        return NDT_ERR_CAPACITY;
    }
    for (uint64_t i = 0; i < m; ++i) {
        if (scans[i].num_points && !scans[i].xyz) return NDT_ERR_INVALID_ARGUMENT;
        if (scans[i].num_points > 0xFFFFFFF0ull) {
            set_error("scan exceeds 2^32 points");
            return NDT_ERR_CAPACITY;
        }
    }
    std::vector<uint32_t> order(m);
    for (uint64_t i = 0; i < m; ++i) order[i] = (uint32_t)i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        return scans[a].num_points > scans[b].num_points;
    });
    jobs.assign(m, AlignJob{});
    ns.assign(m, 0);
    plan.scans = scans;
    plan.chunk_job.clear();
    const uint64_t max_chunk = (16ull << 20) / 12;
    uint64_t off = 0, in_chunk = 0, chunk = (256ull << 10) / 12;
    for (uint64_t t = 0; t < m; ++t) {
        const uint32_t i = order[t];
        if (t == 0 || in_chunk >= chunk) {
            if (t) chunk = std::min(2 * chunk, max_chunk);
            off = (off + 63) & ~63ull;
            plan.chunk_job.push_back((uint32_t)t);
            in_chunk = 0;
        }
        jobs[t].offset = off;
        jobs[t].n = (uint32_t)scans[i].num_points;
        jobs[t].slot = i;
        for (int k = 0; k < 6; ++k) jobs[t].pose[k] = scans[i].initial_pose[k];
        ns[i] = scans[i].num_points;
        off += scans[i].num_points;
        in_chunk += scans[i].num_points;
    }
    plan.chunk_job.push_back((uint32_t)m);
    plan.total = off;
    int rc;
    if ((rc = pin_reserve(x->h_pts, off * 12 + 16)) || (rc = dev_reserve(x->d_in, off * 12 + 16)))
        return rc;
    return NDT_OK;
}

static void stats_add(ndt_stats& a, const ndt_stats& b) {
    a.align_launches += b.align_launches;
    a.alignments += b.alignments;
    a.iterations += b.iterations;
    a.point_iterations += b.point_iterations;
    a.correspondences += b.correspondences;
    a.align_kernel_ms += b.align_kernel_ms;
    a.score_launches += b.score_launches;
    a.score_kernel_ms += b.score_kernel_ms;
    a.build_launches += b.build_launches;
    a.build_ms += b.build_ms;
    a.h2d_bytes += b.h2d_bytes;
    a.d2h_bytes += b.d2h_bytes;
    a.cycles_points += b.cycles_points;
    a.cycles_cluster_wait += b.cycles_cluster_wait;
    a.cycles_control += b.cycles_control;
    a.cycles_broadcast += b.cycles_broadcast;
    a.eigen_solves += b.eigen_solves;
    a.proposal_launches += b.proposal_launches;
    a.proposal_kernel_ms += b.proposal_kernel_ms;
}

static AsyncSlot* find_ticket(ndt_ctx* c, uint64_t ticket) {
    for (auto& s : c->slots)
        if (ticket && s.ticket == ticket) return &s;
    set_error("no asynchronous batch with that ticket");
    return nullptr;
}

extern "C" {

int ndt_align_batch(ndt_ctx* c, const ndt_scan* scans, uint64_t m, ndt_result* out) {
    if (!c || (!scans && m) || (!out && m)) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (m == 0) return NDT_OK;
    cudaSetDevice(c->device);
    std::vector<AlignJob> jobs;
    std::vector<uint64_t> ns;
    StagePlan plan;
    if ((rc = prepare_batch(c, scans, m, jobs, ns, plan))) return rc;
    return run_align(c, (const float*)c->d_in.p, jobs, ns, out, &plan);
}

int ndt_batch_submit(ndt_ctx* c, const ndt_scan* scans, uint64_t m, uint64_t* ticket) {
    if (!c || !ticket || (!scans && m)) return NDT_ERR_INVALID_ARGUMENT;
    *ticket = 0;
    int rc = need_target(c);
    if (rc) return rc;
    cudaSetDevice(c->device);
    AsyncSlot* s = nullptr;
    for (auto& x : c->slots)
        if (x.ticket == 0) {
            s = &x;
            break;
        }
    if (!s) {
        set_error("every asynchronous slot holds a batch: wait for one first");
        return NDT_ERR_CAPACITY;
    }
    if (!s->ctx) {
        if ((rc = ndt_ctx_create(&c->cfg, &s->ctx))) return rc;
        s->ctx->borrowed_map = true;
    }
    ndt_ctx* x = s->ctx;
    // the owner's map (borrowed, never freed by the slot), parameters and tuned shapes
    x->cfg = c->cfg;
    x->cfg_gen = c->cfg_gen;
    x->d1 = c->d1;
    x->d2 = c->d2;
    x->tuned = c->tuned;
    x->map.view = c->map.view;
    x->map.info = c->map.info;
    x->map.valid = true;
    x->map_gen = c->map_gen;
    x->trace = false;
    std::vector<AlignJob> jobs;
    std::vector<uint64_t> ns;
    StagePlan plan;
    if ((rc = prepare_batch(x, scans, m, jobs, ns, plan))) return rc;
    if ((rc = run_align_enqueue(x, (const float*)x->d_in.p, jobs, ns, &plan))) return rc;
    s->ticket = ++c->next_ticket;
    s->m = m;
    *ticket = s->ticket;
    return NDT_OK;
}

int ndt_batch_poll(ndt_ctx* c, uint64_t ticket, int32_t* ready) {
    if (!c || !ready) return NDT_ERR_INVALID_ARGUMENT;
    AsyncSlot* s = find_ticket(c, ticket);
    if (!s) return NDT_ERR_INVALID_ARGUMENT;
    const cudaError_t e = cudaStreamQuery(s->ctx->stream);
    *ready = e == cudaSuccess;
    if (e == cudaErrorNotReady) return NDT_OK;
    return cuda_fail(e, "batch poll");
}

int ndt_batch_wait(ndt_ctx* c, uint64_t ticket, ndt_result* out) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    AsyncSlot* s = find_ticket(c, ticket);
    if (!s) return NDT_ERR_INVALID_ARGUMENT;
    if (s->m && !out) return NDT_ERR_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    ndt_ctx* x = s->ctx;
    const int rc = run_align_finish(x, out);
    stats_add(c->stats, x->stats);
    std::memset(&x->stats, 0, sizeof x->stats);
    c->t_start_ms = x->t_start_ms;
    c->t_finish_ms = x->t_finish_ms;
    s->ticket = 0;
    s->m = 0;
    return rc;
}

int ndt_batch_timings(ndt_ctx* c, double* start_ms, double* finish_ms, uint64_t n) {
    if (!c || (n && (!start_ms || !finish_ms))) return NDT_ERR_INVALID_ARGUMENT;
    if (n > c->t_start_ms.size()) {
        set_error("more timings requested than alignments in the last call");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    for (uint64_t i = 0; i < n; ++i) {
        start_ms[i] = c->t_start_ms[i];
        finish_ms[i] = c->t_finish_ms[i];
    }
    return NDT_OK;
}

}  // extern "C"

// SplitMix64 (Steele, Lea, Flood 2014): the particle generator's stream
static inline uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static inline double unit_double(uint64_t& s) {  // [0, 1), 53 bits
    return (double)(splitmix64(s) >> 11) * 0x1.0p-53;
}

// Particle k of query q (documented with ndt_initial_pose_search): stream seeded by
// (seed, q, k); draws in the order x, y, yaw, then z, roll, pitch (Box-Muller normals).
static void make_particle(const ndt_particle_config& pc, uint64_t q, uint64_t k,
                          const double* prior, double* pose) {
    uint64_t s = pc.seed ^ (0x9e3779b97f4a7c15ull * (q + 1)) ^ (0xd1b54a32d192ed03ull * (k + 1));
    splitmix64(s);
    for (int i = 0; i < 6; ++i) pose[i] = prior[i];
    pose[0] += (2.0 * unit_double(s) - 1.0) * pc.xy_range;
    pose[1] += (2.0 * unit_double(s) - 1.0) * pc.xy_range;
    pose[5] += (2.0 * unit_double(s) - 1.0) * pc.yaw_range;
    const double sig[3] = {pc.z_sigma, pc.roll_pitch_sigma, pc.roll_pitch_sigma};
    const int dim[3] = {2, 3, 4};
    for (int i = 0; i < 3; ++i) {
        const double u1 = 1.0 - unit_double(s), u2 = unit_double(s);
        const double nrm = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
        if (sig[i] > 0.0) pose[dim[i]] += sig[i] * nrm;
    }
}

// Particle k of query q, candidate c of a TPE proposal (c = 0: the particle's own draw, the
// one make_particle gives): the same sampler on a stream whose seed mixes in c.
static void draw_particle(const ndt_particle_config& pc, uint64_t q, uint64_t k, uint64_t c,
                          const double* prior, double* pose) {
    ndt_particle_config p = pc;
    p.seed = pc.seed ^ (0x94d049bb133111ebull * c);
    make_particle(p, q, k, prior, pose);
}

// ---- TPE-guided particles (estimate_initial_pose's guided phase, initial_pose.rs:280-420;
// TreeStructuredParzenEstimator, cuda_ndt_matcher/src/tpe.rs) ----
// A trial is an aligned particle: x, y, yaw of its result and exp(-score / 10); a query's
// trials are kept best first, equal scores in arrival order (a stable sort).
struct TpeTrial {
    double x, y, yaw, score;
};

constexpr double TPE_PI = 3.14159265358979323846;
constexpr int TPE_CANDIDATES = 100;  // N_EI_CANDIDATES

static double tpe_log_sum_exp(const std::vector<double>& v) {
    if (v.empty()) return -INFINITY;
    double m = -INFINITY;
    for (double x : v) m = std::max(m, x);
    if (std::isinf(m)) return m;
    double s = 0.0;
    for (double x : v) s += std::exp(x - m);
    return m + std::log(s);
}

// compute_log_likelihood_ratio (tpe.rs:160-196): Gaussian kernels of widths 0.25 m, 0.25 m
// and 2.5 deg on x, y and the wrapped yaw difference around every trial; the best `above`
// trials form the good set, the rest the bad set, each weighted by its size; the ratio is
// log p_good - 5 log p_bad.
static double tpe_ratio(const std::vector<TpeTrial>& t, size_t above, const double* in) {
    const size_t n = t.size();
    if (n == 0 || above == 0 || above >= n) return 0.0;
    const double sig[3] = {0.25, 0.25, 2.5 * TPE_PI / 180.0};
    const double lsig = std::log(sig[0]) + std::log(sig[1]) + std::log(sig[2]);
    const double wa = std::log(1.0 / (double)above), wb = std::log(1.0 / (double)(n - above));
    std::vector<double> a, b;
    a.reserve(above);
    b.reserve(n - above);
    for (size_t i = 0; i < n; ++i) {
        double d[3] = {in[0] - t[i].x, in[1] - t[i].y, in[5] - t[i].yaw};
        while (d[2] >= TPE_PI) d[2] -= 2.0 * TPE_PI;
        while (d[2] < -TPE_PI) d[2] += 2.0 * TPE_PI;
        double lp = 0.0;
        for (int k = 0; k < 3; ++k) {
            const double r = d[k] / sig[k];
            lp += -0.5 * r * r;
        }
        lp -= lsig;
        if (i < above)
            a.push_back(lp + wa);
        else
            b.push_back(lp + wb);
    }
    return tpe_log_sum_exp(a) - tpe_log_sum_exp(b) * 5.0;
}

// get_next_input (tpe.rs:98-150): a random draw while the good set is empty, else the best of
// 100 further draws by the likelihood ratio (the first draw stands when no ratio beats it)
static void tpe_propose(const ndt_particle_config& pc, uint64_t q, uint64_t k,
                        const double* prior, const std::vector<TpeTrial>& trials, double* pose) {
    const size_t n = trials.size();
    const size_t above = n ? std::min<size_t>(std::max<size_t>(n / 10, 1), 10) : 0;
    draw_particle(pc, q, k, 0, prior, pose);
    if (above == 0) return;
    double best = -INFINITY, cand[6];
    for (int c = 1; c <= TPE_CANDIDATES; ++c) {
        draw_particle(pc, q, k, (uint64_t)c, prior, cand);
        const double r = tpe_ratio(trials, above, cand);
        if (r > best) {
            best = r;
            for (int i = 0; i < 6; ++i) pose[i] = cand[i];
        }
    }
}

static void tpe_add(std::vector<TpeTrial>& t, const ndt_result& r) {
    const TpeTrial x{r.pose[0], r.pose[1], r.pose[5], std::exp(-r.score / 10.0)};
    t.insert(std::upper_bound(t.begin(), t.end(), x,
                              [](const TpeTrial& a, const TpeTrial& b) { return a.score > b.score; }),
             x);
}

static int check_queries(const ndt_scan* queries, uint64_t nq) {
    for (uint64_t q = 0; q < nq; ++q) {
        if (queries[q].num_points == 0) {
            set_error("Source point cloud is empty");
            return NDT_ERR_EMPTY_INPUT;
        }
        if (!queries[q].xyz) return NDT_ERR_INVALID_ARGUMENT;
        if (queries[q].num_points > 0xFFFFFFF0ull) {
            set_error("scan exceeds 2^32 points");
            return NDT_ERR_CAPACITY;
        }
    }
    return 0;
}

// np starting poses per query (starts: nq * np * 6) aligned in one launch, each scored by
// NVTL at its aligned pose, then select_best_particle per query.
// Uploads the queries' points once (c->d_in; qoff: each query's first point) for the
// particle alignments that follow.
static int stage_queries(ndt_ctx* c, const ndt_scan* queries, uint64_t nq,
                         std::vector<uint64_t>& qoff) {
    int rc;
    cudaSetDevice(c->device);
    uint64_t total = 0;
    for (uint64_t q = 0; q < nq; ++q) {
        if (queries[q].num_points == 0) {
            set_error("Source point cloud is empty");
            return NDT_ERR_EMPTY_INPUT;
        }
        if (!queries[q].xyz) return NDT_ERR_INVALID_ARGUMENT;
        if (queries[q].num_points > 0xFFFFFFF0ull) {
            set_error("scan exceeds 2^32 points");
            return NDT_ERR_CAPACITY;
        }
        total += queries[q].num_points;
    }
    if ((rc = pin_reserve(c->h_pts, total * 12 + 16)) || (rc = dev_reserve(c->d_in, total * 12 + 16)))
        return rc;
    qoff.assign(nq, 0);
    uint64_t off = 0;
    for (uint64_t q = 0; q < nq; ++q) {
        qoff[q] = off;
        off += queries[q].num_points;
    }
    stage_scans(c, queries, nq, qoff, total);
    return NDT_OK;
}

// np particles per query from starts (query-major, 6 per particle) against the staged
// points, in one launch; results query-major into res.
static int align_starts(ndt_ctx* c, const ndt_scan* queries, uint64_t nq,
                        const std::vector<uint64_t>& qoff, uint64_t np, const double* starts,
                        ndt_result* res) {
    std::vector<AlignJob> jobs(nq * np);
    std::vector<uint64_t> ns(nq * np);
    for (uint64_t q = 0; q < nq; ++q)
        for (uint64_t k = 0; k < np; ++k) {
            AlignJob& j = jobs[q * np + k];
            j.offset = qoff[q];
            j.n = (uint32_t)queries[q].num_points;
            j.slot = (uint32_t)(q * np + k);
            for (int d = 0; d < 6; ++d) j.pose[d] = starts[6 * (q * np + k) + d];
            ns[q * np + k] = queries[q].num_points;
        }
    return run_align(c, (const float*)c->d_in.p, jobs, ns, res);
}

// select_best_particle (particle.rs:36-42): the highest selection score (NVTL when positive,
// else 5 exp(-score / 10)), the later particle on ties
static void select_best(const ndt_result* res, uint64_t nq, uint64_t np, const double* starts,
                        ndt_pose_estimate* out) {
    for (uint64_t q = 0; q < nq; ++q) {
        int64_t best = -1;
        double best_sel = -INFINITY;
        for (uint64_t k = 0; k < np; ++k) {
            const ndt_result& r = res[q * np + k];
            const double sel = r.nvtl > 0.0 ? r.nvtl : 5.0 * std::exp(-r.score / 10.0);
            if (best < 0 || sel >= best_sel) {
                best = (int64_t)k;
                best_sel = sel;
            }
        }
        const ndt_result& r = res[q * np + (uint64_t)best];
        ndt_pose_estimate& e = out[q];
        std::memset(&e, 0, sizeof e);
        for (int i = 0; i < 6; ++i) {
            e.pose[i] = r.pose[i];
            e.initial_pose[i] = starts[6 * (q * np + (uint64_t)best) + i];
        }
        e.nvtl = r.nvtl;
        e.score = r.score;
        e.selection_score = best_sel;
        e.particle = (int32_t)best;
        e.iterations = r.iterations;
        e.converged = r.converged;
    }
}

static int search_from_starts(ndt_ctx* c, const ndt_scan* queries, uint64_t nq, uint64_t np,
                              const double* starts, ndt_pose_estimate* out,
                              ndt_result* particles) {
    if (nq * np > 0xFFFFFFull) {
        set_error("too many particles in one search (queries x particles > 2^24)");
        return NDT_ERR_CAPACITY;
    }
    std::vector<uint64_t> qoff;
    int rc;
    if ((rc = stage_queries(c, queries, nq, qoff))) return rc;
    std::vector<ndt_result> local;
    ndt_result* res = particles;
    if (!res) {
        local.resize(nq * np);
        res = local.data();
    }
    if ((rc = align_starts(c, queries, nq, qoff, np, starts, res))) return rc;
    select_best(res, nq, np, starts, out);
    return NDT_OK;
}

// The guided search: every query's first np - ng particles (startup) in one launch, then ng
// rounds; in each, every query's TPE proposes its next particle from all of that query's
// results so far (on the context's host threads), and the round's particles are aligned in
// one launch. Each query's particles follow the reference's sequential loop; the queries
// share the launches.
static int search_guided(ndt_ctx* c, const ndt_scan* queries, uint64_t nq,
                         const ndt_particle_config& pc, ndt_pose_estimate* out,
                         ndt_result* particles) {
    const uint64_t np = pc.num_particles, ng = pc.guided, n0 = np - ng;
    std::vector<uint64_t> qoff;
    int rc;
    if ((rc = stage_queries(c, queries, nq, qoff))) return rc;
    std::vector<ndt_result> local;
    ndt_result* res = particles;
    if (!res) {
        local.resize(nq * np);
        res = local.data();
    }
    std::vector<double> starts(nq * np * 6);
    std::vector<std::vector<TpeTrial>> trials(nq);
    if (n0 > 0) {
        std::vector<double> s0(nq * n0 * 6);
        std::vector<ndt_result> r0(nq * n0);
        for (uint64_t q = 0; q < nq; ++q)
            for (uint64_t k = 0; k < n0; ++k)
                make_particle(pc, q, k, queries[q].initial_pose, &s0[6 * (q * n0 + k)]);
        if ((rc = align_starts(c, queries, nq, qoff, n0, s0.data(), r0.data()))) return rc;
        for (uint64_t q = 0; q < nq; ++q)
            for (uint64_t k = 0; k < n0; ++k) {
                res[q * np + k] = r0[q * n0 + k];
                std::memcpy(&starts[6 * (q * np + k)], &s0[6 * (q * n0 + k)], 6 * sizeof(double));
                tpe_add(trials[q], r0[q * n0 + k]);
            }
    }
    std::vector<double> sr(nq * 6);
    std::vector<ndt_result> rr(nq);
    for (uint64_t k = n0; k < np; ++k) {
        c->pool.run(nq, [&](uint64_t q) {
            tpe_propose(pc, q, k, queries[q].initial_pose, trials[q], &sr[6 * q]);
        });
        if ((rc = align_starts(c, queries, nq, qoff, 1, sr.data(), rr.data()))) return rc;
        for (uint64_t q = 0; q < nq; ++q) {
            res[q * np + k] = rr[q];
            std::memcpy(&starts[6 * (q * np + k)], &sr[6 * q], 6 * sizeof(double));
            tpe_add(trials[q], rr[q]);
        }
    }
    select_best(res, nq, np, starts.data(), out);
    return NDT_OK;
}

extern "C" {

int ndt_initial_pose_search(ndt_ctx* c, const ndt_scan* queries, uint64_t nq,
                            const ndt_particle_config* pc, ndt_pose_estimate* out,
                            ndt_result* particles) {
    if (!c || !pc || (nq && (!queries || !out))) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (nq == 0) return NDT_OK;
    const uint64_t np = pc->num_particles;
    if (np == 0 || pc->guided >= np || !(pc->xy_range >= 0.0) || !(pc->yaw_range >= 0.0) ||
        !(pc->z_sigma >= 0.0) || !(pc->roll_pitch_sigma >= 0.0)) {
        set_error("invalid particle configuration");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    if ((rc = check_queries(queries, nq))) return rc;
    if (nq * np > 0xFFFFFFull) {
        set_error("too many particles in one search (queries x particles > 2^24)");
        return NDT_ERR_CAPACITY;
    }
    if (pc->guided > 0) return search_guided(c, queries, nq, *pc, out, particles);
    std::vector<double> starts(nq * np * 6);
    for (uint64_t q = 0; q < nq; ++q)
        for (uint64_t k = 0; k < np; ++k)
            make_particle(*pc, q, k, queries[q].initial_pose, &starts[6 * (q * np + k)]);
    return search_from_starts(c, queries, nq, np, starts.data(), out, particles);
}

int ndt_tpe_propose(const ndt_particle_config* pc, uint64_t query, uint64_t particle,
                    const double prior[6], const double* trials, uint64_t num_trials,
                    double pose_out[6]) {
    if (!pc || !prior || !pose_out || (num_trials && !trials)) return NDT_ERR_INVALID_ARGUMENT;
    std::vector<TpeTrial> t;
    t.reserve(num_trials);
    for (uint64_t i = 0; i < num_trials; ++i) {
        const TpeTrial x{trials[4 * i], trials[4 * i + 1], trials[4 * i + 2], trials[4 * i + 3]};
        t.insert(std::upper_bound(t.begin(), t.end(), x,
                                  [](const TpeTrial& a, const TpeTrial& b) {
                                      return a.score > b.score;
                                  }),
                 x);
    }
    tpe_propose(*pc, query, particle, prior, t, pose_out);
    return NDT_OK;
}

int ndt_learned_pose_search(ndt_ctx* c, ndt_pnet* net, int32_t map_id, const ndt_scan* queries,
                            uint64_t nq, const ndt_particle_config* refine,
                            double nvtl_threshold, const ndt_particle_config* fallback,
                            ndt_pose_estimate* out, int32_t* used_fallback) {
    if (!c || !net || (nq && (!queries || !out))) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (nq == 0) return NDT_OK;
    if ((rc = check_queries(queries, nq))) return rc;
    ndt_pnet_config pcfg;
    if ((rc = ndt_pnet_get_config(net, &pcfg))) return rc;
    const uint64_t np = (uint64_t)pcfg.proposals;
    std::vector<double> starts(nq * np * 6);
    ndt_pnet_stats before, after;
    ndt_pnet_stats_get(net, &before);
    if ((rc = ndt_pnet_propose(net, map_id, queries, nq, starts.data(), nullptr))) return rc;
    ndt_pnet_stats_get(net, &after);
    c->stats.proposal_launches += after.inference_batches - before.inference_batches;
    c->stats.proposal_kernel_ms += after.inference_kernel_ms - before.inference_kernel_ms;
    if ((rc = search_from_starts(c, queries, nq, np, starts.data(), out, nullptr))) return rc;
    if (refine && refine->num_particles > 0) {
        // a second round around each query's best proposal result: refine->num_particles
        // particles drawn around it (the particle search's rule, seeded), all aligned in one
        // launch; the better of the two rounds' winners is kept
        std::vector<ndt_scan> around(queries, queries + nq);
        for (uint64_t q = 0; q < nq; ++q)
            for (int k = 0; k < 6; ++k) around[q].initial_pose[k] = out[q].pose[k];
        ndt_particle_config rc2 = *refine;
        rc2.guided = 0;
        std::vector<ndt_pose_estimate> second(nq);
        if ((rc = ndt_initial_pose_search(c, around.data(), nq, &rc2, second.data(), nullptr)))
            return rc;
        for (uint64_t q = 0; q < nq; ++q)
            if (second[q].selection_score > out[q].selection_score) out[q] = second[q];
    }
    std::vector<uint64_t> redo;
    for (uint64_t q = 0; q < nq; ++q) {
        const bool fb = fallback && out[q].nvtl < nvtl_threshold;
        if (used_fallback) used_fallback[q] = fb ? 1 : 0;
        if (fb) redo.push_back(q);
    }
    if (redo.empty()) return NDT_OK;
    std::vector<ndt_scan> sub(redo.size());
    for (size_t i = 0; i < redo.size(); ++i) sub[i] = queries[redo[i]];
    std::vector<ndt_pose_estimate> sub_out(redo.size());
    if ((rc = ndt_initial_pose_search(c, sub.data(), sub.size(), fallback, sub_out.data(),
                                      nullptr)))
        return rc;
    for (size_t i = 0; i < redo.size(); ++i) out[redo[i]] = sub_out[i];
    return NDT_OK;
}

int ndt_align(ndt_ctx* c, const float* xyz, uint64_t n, const double pose_in[6], ndt_result* out) {
    if (!c || !pose_in || !out || (!xyz && n)) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (n == 0) {
        set_error("Source point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    ndt_scan s;
    s.xyz = xyz;
    s.num_points = n;
    for (int k = 0; k < 6; ++k) s.initial_pose[k] = pose_in[k];
    return ndt_align_batch(c, &s, 1, out);
}

int ndt_align_multi_pose(ndt_ctx* c, const float* xyz, uint64_t n, const double* poses,
                         uint64_t m, ndt_result* out) {
    if (!c || (!poses && m) || (!out && m) || (!xyz && n)) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (n == 0) {
        set_error("Source point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    if (m == 0) return NDT_OK;
    if (n > 0xFFFFFFF0ull || m > 0xFFFFFFull) {
        set_error("scan or pose count too large");
        return NDT_ERR_CAPACITY;
    }
    cudaSetDevice(c->device);
    if ((rc = pin_reserve(c->h_pts, n * 12)) || (rc = dev_reserve(c->d_in, n * 12))) return rc;
    std::memcpy(c->h_pts.p, xyz, n * 12);
    cudaMemcpyAsync(c->d_in.p, c->h_pts.p, n * 12, cudaMemcpyHostToDevice, c->stream);
    c->stats.h2d_bytes += n * 12;
    std::vector<AlignJob> jobs(m);
    std::vector<uint64_t> ns(m, n);
    for (uint64_t i = 0; i < m; ++i) {
        jobs[i].offset = 0;
        jobs[i].n = (uint32_t)n;
        jobs[i].slot = (uint32_t)i;
        for (int k = 0; k < 6; ++k) jobs[i].pose[k] = poses[6 * i + k];
    }
    return run_align(c, (const float*)c->d_in.p, jobs, ns, out);
}

int ndt_align_batch_device(ndt_ctx* c, const float* d_xyz, const uint64_t* offsets,
                           const double* poses, uint64_t m, ndt_result* out) {
    if (!c || (m && (!d_xyz || !offsets || !poses || !out))) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (m == 0) return NDT_OK;
    if (m > 0xFFFFFFull) {
        set_error("too many scans in one batch");
        return NDT_ERR_CAPACITY;
    }
    cudaSetDevice(c->device);
    std::vector<AlignJob> jobs(m);
    std::vector<uint64_t> ns(m);
    for (uint64_t i = 0; i < m; ++i) {
        if (offsets[i + 1] < offsets[i] || offsets[i + 1] - offsets[i] > 0xFFFFFFF0ull)
            return NDT_ERR_INVALID_ARGUMENT;
        jobs[i].offset = offsets[i];
        jobs[i].n = (uint32_t)(offsets[i + 1] - offsets[i]);
        jobs[i].slot = (uint32_t)i;
        for (int k = 0; k < 6; ++k) jobs[i].pose[k] = poses[6 * i + k];
        ns[i] = jobs[i].n;
    }
    return run_align(c, d_xyz, jobs, ns, out);
}

int ndt_autotune(ndt_ctx* c, const float* d_xyz, const uint64_t* offsets, const double* poses,
                 uint64_t m, int32_t repeats, ndt_tune_result* out) {
    if (!c || !d_xyz || !offsets || !poses || m == 0 || !out) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (repeats < 1) repeats = 1;
    uint64_t max_n = 0;
    for (uint64_t i = 0; i < m; ++i) max_n = std::max(max_n, offsets[i + 1] - offsets[i]);
    std::vector<ndt_result> tmp(m);
    ndt_stats saved = c->stats;
    const int Ks[4] = {1, 2, 4, 8};
    const int TC[8][2] = {{128, 128}, {128, 80}, {128, 64}, {256, 128},
                          {256, 80},  {256, 64}, {256, 48}, {512, 128}};
    // work-queue candidates: (threads, registers, points per thread per chunk, lanes sharing
    // each point's neighbour search, chunk points staged in shared memory)
    const int QC[14][5] = {{256, 64, 2, 1, 0}, {256, 64, 4, 1, 0}, {256, 64, 8, 1, 0},
                           {256, 80, 4, 1, 0}, {128, 64, 4, 1, 0}, {512, 128, 2, 1, 0},
                           {256, 64, 4, 2, 0}, {256, 64, 4, 4, 0}, {256, 64, 8, 4, 0},
                           {256, 64, 2, 1, 1}, {256, 64, 4, 1, 1}, {256, 64, 8, 1, 1},
                           {256, 64, 4, 2, 1}, {256, 64, 4, 4, 1}};
    const bool graph_sem = c->cfg.semantics != NDT_SEMANTICS_CPU;
    const bool ls = c->cfg.use_line_search != 0;
    std::vector<LaunchShape> cands;
    if (c->cfg.work_queue <= 0 || ls)
        for (int K : Ks)
            for (const auto& tc : TC) cands.push_back(LaunchShape{K, tc[0], tc[1], 0});
    if (c->cfg.work_queue >= 0 && !ls)
        for (const auto& qc : QC)
            if (qc[3] == 1 || graph_sem)
                cands.push_back(LaunchShape{1, qc[0], qc[1], qc[2], qc[3], qc[4]});
    LaunchShape best{0, 0, 128, 0};
    double best_ms = 1e300;
    int tried = 0;
    for (const LaunchShape& cand : cands) {
        c->forced = cand;
        rc = ndt_align_batch_device(c, d_xyz, offsets, poses, m, tmp.data());  // warm
        if (rc) break;
        double before = c->stats.align_kernel_ms;
        for (int r = 0; r < repeats && !rc; ++r)
            rc = ndt_align_batch_device(c, d_xyz, offsets, poses, m, tmp.data());
        if (rc) break;
        double ms = (c->stats.align_kernel_ms - before) / repeats;
        tried++;
        if (ms < best_ms) {
            best_ms = ms;
            best = c->forced;
        }
    }
    c->forced = LaunchShape{0, 0, 0, 0};
    c->stats = saved;
    if (rc) return rc;
    c->tuned[{log2_bucket(m), log2_bucket(max_n)}] = best;
    out->cluster_size = best.cluster;
    out->threads_per_cta = best.threads;
    out->registers = best.regcap;
    out->work_queue = best.queue;
    out->lanes_per_point = best.queue > 0 ? std::max(1, best.npw) : 0;
    out->stage_points = best.queue > 0 ? best.stage : 0;
    out->reserved = 0;
    out->kernel_ms = best_ms;
    out->aligns_per_s = best_ms > 0 ? 1000.0 * (double)m / best_ms : 0.0;
    out->candidates = tried;
    return NDT_OK;
}

int ndt_eval_batch(ndt_ctx* c, const float* xyz, uint64_t n, const double* T34, uint64_t m,
                   double* nvtl, double* tp) {
    if (!c || (!T34 && m) || (!xyz && n)) return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (m == 0) return NDT_OK;
    if (n > 0xFFFFFFF0ull || m > 0xFFFFFFull) {
        set_error("scan or pose count too large");
        return NDT_ERR_CAPACITY;
    }
    cudaSetDevice(c->device);
    size_t sjb = m * sizeof(ScoreJob), sob = m * sizeof(ScoreOut);
    if ((rc = pin_reserve(c->h_pts, n * 12 + 16)) || (rc = dev_reserve(c->d_in, n * 12 + 16)) ||
        (rc = dev_reserve(c->d_sjobs, sjb)) || (rc = dev_reserve(c->d_sout, sob)) ||
        (rc = dev_reserve(c->d_part, score_part_bytes((uint32_t)m, (uint32_t)n))) ||
        (rc = pin_reserve(c->h_sjobs, sjb)) || (rc = pin_reserve(c->h_sout, sob)))
        return rc;
    if (n) std::memcpy(c->h_pts.p, xyz, n * 12);
    ScoreJob* hs = (ScoreJob*)c->h_sjobs.p;
    for (uint64_t j = 0; j < m; ++j) {
        ScoreJob s{};
        s.offset = 0;
        s.n = (uint32_t)n;
        s.pose_src = 0;
        s.out_index = (uint32_t)j;
        for (int k = 0; k < 12; ++k) s.T[k] = T34[12 * j + k];
        hs[j] = s;
    }
    cudaStream_t st = c->stream;
    if (n) cudaMemcpyAsync(c->d_in.p, c->h_pts.p, n * 12, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(c->d_sjobs.p, hs, sjb, cudaMemcpyHostToDevice, st);
    cudaEventRecord(c->ev0, st);
    if ((rc = launch_score(c->map.view, (const float*)c->d_in.p, (const ScoreJob*)c->d_sjobs.p,
                           (uint32_t)m, (uint32_t)n, nullptr, c->d_part.p, (ScoreOut*)c->d_sout.p,
                           (float)c->d1, (float)c->d2, st)))
        return rc;
    cudaEventRecord(c->ev1, st);
    cudaMemcpyAsync(c->h_sout.p, c->d_sout.p, sob, cudaMemcpyDeviceToHost, st);
    if ((rc = cuda_fail(cudaStreamSynchronize(st), "eval"))) return rc;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    c->stats.score_launches++;
    c->stats.score_kernel_ms += ms;
    c->stats.h2d_bytes += n * 12 + sjb;
    c->stats.d2h_bytes += sob;
    const ScoreOut* so = (const ScoreOut*)c->h_sout.p;
    for (uint64_t j = 0; j < m; ++j) {
        if (nvtl) nvtl[j] = so[j].nvtl_count ? so[j].nvtl_sum / (double)so[j].nvtl_count : 0.0;
        if (tp) tp[j] = so[j].ncorr ? so[j].score_sum / (double)so[j].ncorr : 0.0;
    }
    return NDT_OK;
}

int ndt_neighbors_query(ndt_ctx* c, const float* xyz, uint64_t n, int32_t max_nb, int32_t* idx,
                        int32_t* counts) {
    if (!c || (n && (!xyz || !idx || !counts)) || max_nb < 1 || max_nb > MAX_NB_ALL)
        return NDT_ERR_INVALID_ARGUMENT;
    int rc = need_target(c);
    if (rc) return rc;
    if (n == 0) return NDT_OK;
    cudaSetDevice(c->device);
    if ((rc = dev_reserve(c->d_q, n * 12)) || (rc = dev_reserve(c->d_qidx, n * 4 * max_nb)) ||
        (rc = dev_reserve(c->d_qcnt, n * 4)))
        return rc;
    cudaStream_t st = c->stream;
    cudaMemcpyAsync(c->d_q.p, xyz, n * 12, cudaMemcpyHostToDevice, st);
    if ((rc = launch_query(c->map.view, (const float*)c->d_q.p, n, max_nb, (int32_t*)c->d_qidx.p,
                           (int32_t*)c->d_qcnt.p, st)))
        return rc;
    cudaMemcpyAsync(idx, c->d_qidx.p, n * 4 * max_nb, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(counts, c->d_qcnt.p, n * 4, cudaMemcpyDeviceToHost, st);
    return cuda_fail(cudaStreamSynchronize(st), "neighbour query");
}

int ndt_radix_sort_pairs_u64_u32(uint64_t* d_keys, uint32_t* d_values, uint64_t n,
                                 int32_t begin_bit, int32_t end_bit, void* d_temp,
                                 uint64_t* temp_bytes, void* stream) {
    if (!temp_bytes || begin_bit < 0 || end_bit > 64 || begin_bit > end_bit)
        return NDT_ERR_INVALID_ARGUMENT;
    size_t need = radix_sort_temp_bytes((size_t)n);
    if (!d_temp) {
        *temp_bytes = need;
        return NDT_OK;
    }
    if (*temp_bytes < need || (n && (!d_keys || !d_values))) return NDT_ERR_INVALID_ARGUMENT;
    return radix_sort_pairs(d_keys, d_values, (size_t)n, begin_bit, end_bit, d_temp,
                            (size_t)*temp_bytes, (cudaStream_t)stream);
}

int ndt_detect_segments(const uint64_t* d_sorted, uint64_t n, uint32_t* d_segment_ids,
                        uint32_t* d_segment_starts, uint32_t* d_num_segments, void* d_temp,
                        uint64_t* temp_bytes, void* stream) {
    if (!temp_bytes) return NDT_ERR_INVALID_ARGUMENT;
    size_t need = detect_segments_temp_bytes((size_t)n);
    if (!d_temp) {
        *temp_bytes = need;
        return NDT_OK;
    }
    if (*temp_bytes < need || !d_num_segments || (n && (!d_sorted || !d_segment_starts)))
        return NDT_ERR_INVALID_ARGUMENT;
    return detect_segments(d_sorted, (size_t)n, d_segment_ids, d_segment_starts, d_num_segments,
                           d_temp, (size_t)*temp_bytes, (cudaStream_t)stream);
}

int ndt_morton_codes(const float* d_xyz, uint64_t n, float res, uint64_t* d_codes,
                     uint32_t* d_indices, int32_t* d_min_cell, void* d_temp,
                     uint64_t* temp_bytes, void* stream) {
    if (!temp_bytes || !(res > 0.f)) return NDT_ERR_INVALID_ARGUMENT;
    if (!d_temp) {
        *temp_bytes = 256;
        return NDT_OK;
    }
    if (*temp_bytes < 256 || (n && (!d_xyz || !d_codes || !d_indices)))
        return NDT_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = morton_codes(d_xyz, (size_t)n, res, d_codes, d_indices, (int32_t*)d_temp, s);
    if (rc) return rc;
    if (d_min_cell)
        cudaMemcpyAsync(d_min_cell, d_temp, 12, cudaMemcpyDeviceToDevice, s);
    return cuda_fail(cudaGetLastError(), "morton codes");
}

}  // extern "C"
