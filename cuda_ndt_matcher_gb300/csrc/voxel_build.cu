// voxel_build.cu — GPU voxel-map build for sm_103a (the `set_target` hot path).
//
// Pipeline (one CUDA stream, no host work between kernels except the size reads that pick
// the key width and size the allocations):
//   1. cells + bounds      : cell = floor(p / res) per finite point (f32 IEEE division, the
//                            membership rule of VoxelCoord::from_point,
//                            src/ndt_cuda/src/voxel_grid/types.rs:206-212); min/max cell.
//   2. Morton keys         : key = morton(cell - min cell), 21 bits per axis
//                            (src/ndt_cuda/src/voxel_grid/gpu/morton.rs:45-95 layout); the
//                            non-finite points get key ~0 and sort last.
//   3. LSD radix sort      : stable, 8-bit digits, only the significant key bits, 32-bit
//                            keys when they fit (replaces cub::DeviceRadixSort,
//                            src/cuda_ffi/csrc/radix_sort.cu).
//   4. segments            : per-tile counts of key changes, scanned, then the starts
//                            (src/cuda_ffi/csrc/segment_detect.cu:27-146; the API's
//                            ndt_detect_segments keeps flags + scan for the segment ids).
//   5. voxel statistics    : segments visited largest first; segments of 48 points or more
//                            summed by a warp each (k_segment_sums), the rest by a thread
//                            each, every voxel finished by a thread (k_voxel_stats); exact
//                            integer moments of the segment's points (the FP64
//                            running sum's mean bit for bit, the centred covariance from an
//                            exact numerator), FP64 two-pass moments where the exact bounds
//                            do not hold; eigenvector directions by an f32 Jacobi, refined
//                            in FP64; regularisation to the min-ratio and inverse in FP64,
//                            f32 outputs (Voxel::from_statistics / regularize_covariance,
//                            src/ndt_cuda/src/voxel_grid/types.rs:54-190).
//   6. compaction          : valid voxels keep their Morton order.
//   7. hash insert         : bounded linear probing with atomicCAS, displacement recorded
//                            (voxel_hash_build_kernel, src/cuda_ffi/csrc/voxel_hash.cu:69-114).
//   8. dense cell index    : when it fits, {centroid, slot} per cell of the map's box, and
//                            the neighbourhood masks (one per octant of each cell while they
//                            fit their budget, else one per cell) that list the neighbours a
//                            point there can accept.
// Bit-exact parts (cells, keys, counts, means) use no multiply-add: cells are an f32 division,
// means an FP64 division of an exact sum (or a running sum of adds), so FMA contraction
// cannot change them; the regularised covariances, compared in f32 ULPs, use FMAs freely.
#include <algorithm>
#include <cstdio>
#include <mutex>

#include <cuda.h>

#include "ndt_internal.h"

namespace ndtgb {

constexpr int BT = 256;        // threads per block for tile kernels
constexpr int ITEMS = 16;      // items per thread
constexpr int TILE = BT * ITEMS;

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
static inline uint32_t ntiles(size_t n) { return (uint32_t)((n + TILE - 1) / TILE); }

// ---------------------------------------------------------------------------------------
// Block-wide exclusive scan of one value per thread (256 threads).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* ws,
                                                         uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (BT / 32) ? ws[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < BT / 32) ws[lane] = w;
    }
    __syncthreads();
    uint32_t pre = warp ? ws[warp - 1] : 0u;
    *total = ws[BT / 32 - 1];
    __syncthreads();
    return pre + x - v;
}

__global__ void __launch_bounds__(BT) k_tile_reduce(const uint32_t* __restrict__ in, size_t n,
                                                    uint32_t* __restrict__ bsum) {
    __shared__ uint32_t ws[BT / 32];
    size_t base = (size_t)blockIdx.x * TILE;
    uint32_t s = 0;
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
        size_t i = base + (size_t)r * BT + threadIdx.x;
        if (i < n) s += in[i];
    }
    uint32_t tot;
    block_exclusive_scan(s, ws, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(BT) k_scan_bsums(uint32_t* __restrict__ bsum, uint32_t nb) {
    __shared__ uint32_t ws[BT / 32];
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += TILE) {
        uint32_t v[ITEMS];
        uint32_t s = 0;
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            uint32_t i = base + threadIdx.x * ITEMS + k;
            v[k] = i < nb ? bsum[i] : 0u;
            s += v[k];
        }
        uint32_t tot;
        uint32_t run = carry + block_exclusive_scan(s, ws, &tot);
#pragma unroll
        for (int k = 0; k < ITEMS; ++k) {
            uint32_t i = base + threadIdx.x * ITEMS + k;
            if (i < nb) bsum[i] = run;
            run += v[k];
        }
        carry += tot;
        __syncthreads();
    }
}

// exclusive scan of a tile; element order: thread t holds items t*ITEMS .. t*ITEMS+15
__global__ void __launch_bounds__(BT) k_tile_scan(const uint32_t* __restrict__ in,
                                                  uint32_t* __restrict__ out, size_t n,
                                                  const uint32_t* __restrict__ bsum) {
    __shared__ uint32_t ws[BT / 32];
    size_t base = (size_t)blockIdx.x * TILE + (size_t)threadIdx.x * ITEMS;
    uint32_t v[ITEMS];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0u;
        s += v[k];
    }
    uint32_t tot;
    uint32_t run = bsum[blockIdx.x] + block_exclusive_scan(s, ws, &tot);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
}

size_t scan_temp_bytes(size_t n) { return align_up((size_t)ntiles(n) * 4 + 4, 256); }

// exclusive scan in -> out (may alias); temp >= scan_temp_bytes(n)
static int exclusive_scan(const uint32_t* in, uint32_t* out, size_t n, void* temp,
                          cudaStream_t s) {
    if (n == 0) return 0;
    uint32_t nb = ntiles(n);
    uint32_t* bsum = (uint32_t*)temp;
    k_tile_reduce<<<nb, BT, 0, s>>>(in, n, bsum);
    k_scan_bsums<<<1, BT, 0, s>>>(bsum, nb);
    k_tile_scan<<<nb, BT, 0, s>>>(in, out, n, bsum);
    return cuda_fail(cudaGetLastError(), "scan launch");
}

// ---------------------------------------------------------------------------------------
// Stable LSD radix sort of (key, u32 value) pairs, 8-bit digits; keys u64 or, when the
// significant bits fit, u32 (half the key traffic per pass).
// ---------------------------------------------------------------------------------------
// Digit counts of each TILE-key tile: shared-memory atomics into one counter set per warp
// (keys of one digit then queue only within their warp), summed per digit at the end.
template <typename K>
__global__ void __launch_bounds__(BT) k_radix_hist(const K* __restrict__ keys, size_t n,
                                                   int shift, uint32_t dmask,
                                                   uint32_t* __restrict__ hist, uint32_t nb) {
    __shared__ uint32_t h[BT / 32][256];
#pragma unroll
    for (int w = 0; w < BT / 32; ++w) h[w][threadIdx.x] = 0;
    __syncthreads();
    uint32_t* const hw = h[threadIdx.x >> 5];
    const size_t base = (size_t)blockIdx.x * TILE;
    K kv[ITEMS];
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
        const size_t i = base + (size_t)r * BT + threadIdx.x;
        kv[r] = i < n ? keys[i] : K(0);
    }
#pragma unroll
    for (int r = 0; r < ITEMS; ++r)
        if (base + (size_t)r * BT + threadIdx.x < n)
            atomicAdd(&hw[(uint32_t)(kv[r] >> shift) & dmask], 1u);
    __syncthreads();
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < BT / 32; ++w) c += h[w][threadIdx.x];
    hist[(size_t)threadIdx.x * nb + blockIdx.x] = c;
}

// Lanes of the warp whose 9-bit value d (an 8-bit digit, or 0x100 for no key) equals this
// lane's: one ballot per bit, each narrowing the set to the lanes that agree on that bit.
__device__ __forceinline__ uint32_t digit_peers(uint32_t d) {
    uint32_t m = 0xffffffffu;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const bool bit = (d >> k) & 1u;
        const uint32_t b = __ballot_sync(0xffffffffu, bit);
        m &= bit ? b : ~b;
    }
    return m;
}

// One block per TILE-key tile. Warp w owns the tile's keys [w * 512, (w + 1) * 512), held in
// registers as 16 rounds of 32. Pass 1: each warp counts its digits into its own counters
// (same-digit lanes found by digit_peers). Then per digit: the tile-local start (block
// scan) plus the counts of the earlier warps give each warp's first position. Pass 2: each
// key goes to shared memory at its warp's running position of its digit plus its rank among
// the round's same-digit lanes: tile order within each digit, so the sort is stable. Last, the
// keys leave in that order: the keys of one digit as one contiguous run at base[digit] (the
// scanned histogram), so the stores coalesce.
template <typename K>
__global__ void __launch_bounds__(BT, sizeof(K) == 4 ? 4 : 3) k_radix_scatter(
    const K* __restrict__ kin, const uint32_t* __restrict__ vin, K* __restrict__ kout,
    uint32_t* __restrict__ vout, size_t n, int shift, uint32_t dmask,
    const uint32_t* __restrict__ offs, uint32_t nb) {
    constexpr int NWARP = BT / 32;
    constexpr int WROUNDS = TILE / BT;  // rounds of 32 keys per warp
    extern __shared__ __align__(16) unsigned char sc_smem[];
    K* skey = reinterpret_cast<K*>(sc_smem);
    uint32_t* sval = reinterpret_cast<uint32_t*>(sc_smem + TILE * sizeof(K));
    __shared__ uint32_t wpos[NWARP][256];  // per warp: digit counts, then running positions
    __shared__ uint32_t base[256];         // global position of the tile's first key of each digit
    __shared__ uint32_t loff[256];         // tile-local position of the first key of each digit
    __shared__ uint32_t ws[NWARP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t tbase = (size_t)blockIdx.x * TILE;
    const uint32_t tn = (uint32_t)min((size_t)TILE, n - tbase);
    const uint32_t wbase = (uint32_t)warp * (WROUNDS * 32);
#pragma unroll
    for (int w = 0; w < NWARP; ++w) wpos[w][threadIdx.x] = 0;
    __syncthreads();
    K key[WROUNDS];
#pragma unroll
    for (int r = 0; r < WROUNDS; ++r) {
        const uint32_t li = wbase + (uint32_t)r * 32 + lane;
        key[r] = li < tn ? kin[tbase + li] : K(0);
    }
#pragma unroll
    for (int r = 0; r < WROUNDS; ++r) {
        const uint32_t li = wbase + (uint32_t)r * 32 + lane;
        const uint32_t d = li < tn ? ((uint32_t)(key[r] >> shift) & dmask) : 0x100u;
        const uint32_t peers = digit_peers(d);
        if (d != 0x100u && lane == __ffs(peers) - 1) wpos[warp][d] += (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        const uint32_t d = threadIdx.x;  // one thread per digit (BT == 256)
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < NWARP; ++w) {
            const uint32_t c = wpos[w][d];
            wpos[w][d] = run;
            run += c;
        }
        uint32_t tot;
        const uint32_t lo = block_exclusive_scan(run, ws, &tot);
        loff[d] = lo;
#pragma unroll
        for (int w = 0; w < NWARP; ++w) wpos[w][d] += lo;
        base[d] = offs[(size_t)d * nb + blockIdx.x];
    }
    __syncthreads();
    const uint32_t lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < WROUNDS; ++r) {
        const uint32_t li = wbase + (uint32_t)r * 32 + lane;
        const bool valid = li < tn;
        const uint32_t d = valid ? ((uint32_t)(key[r] >> shift) & dmask) : 0x100u;
        const uint32_t peers = digit_peers(d);
        if (valid) {
            const uint32_t pos = wpos[warp][d] + (uint32_t)__popc(peers & lt);
            skey[pos] = key[r];
            sval[pos] = vin[tbase + li];
        }
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wpos[warp][d] += (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < tn; i += BT) {
        const K k = skey[i];
        const uint32_t d = (uint32_t)(k >> shift) & dmask;
        const uint32_t pos = base[d] + (i - loff[d]);
        kout[pos] = k;
        vout[pos] = sval[i];
    }
}

template <typename K>
static size_t radix_temp_bytes(size_t n) {
    size_t nb = ntiles(n);
    return align_up(n * sizeof(K), 256) + align_up(n * 4, 256) + align_up(256 * nb * 4, 256) +
           scan_temp_bytes(256 * nb);
}

size_t radix_sort_temp_bytes(size_t n) { return radix_temp_bytes<uint64_t>(n); }

template <typename K>
static int radix_sort_t(K* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                        void* temp, size_t temp_bytes, cudaStream_t s) {
    if (n <= 1 || end_bit <= begin_bit) return 0;
    if (temp_bytes < radix_temp_bytes<K>(n)) {
        set_error("radix sort: temporary storage too small");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    uint32_t nb = ntiles(n);
    char* t = (char*)temp;
    K* kalt = (K*)t;
    t += align_up(n * sizeof(K), 256);
    uint32_t* valt = (uint32_t*)t;
    t += align_up(n * 4, 256);
    uint32_t* hist = (uint32_t*)t;
    t += align_up(256 * (size_t)nb * 4, 256);
    void* stemp = t;
    K* kin = keys;
    uint32_t* vin = vals;
    K* kout = kalt;
    uint32_t* vout = valt;
    int passes = 0;
    // the scatter's tile staging may exceed the default dynamic shared-memory limit (set on
    // the current device at every call: a host-side attribute, no allocation)
    constexpr int smem = TILE * (int)(sizeof(K) + 4);
    cudaFuncSetAttribute(k_radix_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    for (int shift = begin_bit; shift < end_bit; shift += 8, ++passes) {
        int width = std::min(8, end_bit - shift);
        uint32_t dmask = (1u << width) - 1u;
        k_radix_hist<K><<<nb, BT, 0, s>>>(kin, n, shift, dmask, hist, nb);
        int rc = exclusive_scan(hist, hist, 256 * (size_t)nb, stemp, s);
        if (rc) return rc;
        k_radix_scatter<K><<<nb, BT, smem, s>>>(kin, vin, kout, vout, n, shift, dmask, hist, nb);
        int e = cuda_fail(cudaGetLastError(), "radix scatter launch");
        if (e) return e;
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    if (passes & 1) {
        cudaMemcpyAsync(keys, kin, n * sizeof(K), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(vals, vin, n * 4, cudaMemcpyDeviceToDevice, s);
    }
    return cuda_fail(cudaGetLastError(), "radix sort");
}

int radix_sort_pairs(uint64_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                     void* temp, size_t temp_bytes, cudaStream_t s) {
    return radix_sort_t(keys, vals, n, begin_bit, end_bit, temp, temp_bytes, s);
}

int radix_sort_pairs32(uint32_t* keys, uint32_t* vals, size_t n, int begin_bit, int end_bit,
                       void* temp, size_t temp_bytes, cudaStream_t s) {
    return radix_sort_t(keys, vals, n, begin_bit, std::min(end_bit, 32), temp, temp_bytes, s);
}

// ---------------------------------------------------------------------------------------
// Allocation-free radix sort: the passes above with their scratch (alternate key/value
// buffers, digit histograms, scan block sums) in one fixed device array of this module.
// Sized for STATIC_SORT_MAX_PAIRS pairs: 8 + 4 bytes per pair + 256 counters per 4096-pair
// tile + the scan's block sums = 12,845,312 bytes. Nothing in it needs to start at zero:
// every pass writes each word of the scratch before it reads it.
// ---------------------------------------------------------------------------------------
constexpr size_t STATIC_SORT_MAX_PAIRS = size_t(1) << 20;
constexpr size_t STATIC_SORT_SCRATCH_BYTES = STATIC_SORT_MAX_PAIRS * 8 + STATIC_SORT_MAX_PAIRS * 4 +
                                             256 * (STATIC_SORT_MAX_PAIRS / TILE) * 4 + 256;
constexpr int STATIC_SORT_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_static_sort_scratch[STATIC_SORT_SCRATCH_BYTES];

static std::mutex g_static_sort_mu;
static void* g_static_sort_ptr[STATIC_SORT_MAX_DEVICES];
static unsigned long long g_static_sort_ctx[STATIC_SORT_MAX_DEVICES];

// Unique id of the calling thread's current CUDA context (cuCtxGetId through the runtime's
// driver entry points), 0 when it cannot be read. A device reset or a new primary context
// gives a new id, and the module (with its __device__ array) is loaded again at a new address.
static unsigned long long current_context_id() {
    using GetCurrent = CUresult (*)(CUcontext*);
    using GetId = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (GetId)p;
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device. It is resolved once per device
// and context: the first call on a device (and the first after a cudaDeviceReset, which ends
// the context the address belonged to) calls cudaGetSymbolAddress, which can load this
// module onto the device. When the context id cannot be read, the address is resolved on
// every call (a lookup, no allocation).
static int static_sort_scratch(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "static radix sort: no current device");
    if (dev < 0 || dev >= STATIC_SORT_MAX_DEVICES) {
        set_error("static radix sort: device ordinal out of range");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    // makes the device's primary context current (created if needed), so its id is readable
    e = cudaSetDevice(dev);
    if (e != cudaSuccess) return cuda_fail(e, "static radix sort: device set-up");
    const unsigned long long ctx_id = current_context_id();
    std::lock_guard<std::mutex> lock(g_static_sort_mu);
    if (!g_static_sort_ptr[dev] || ctx_id == 0 || g_static_sort_ctx[dev] != ctx_id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_sort_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "static radix sort: scratch set-up");
        if (radix_sort_temp_bytes(STATIC_SORT_MAX_PAIRS) > STATIC_SORT_SCRATCH_BYTES) {
            set_error("static radix sort: scratch array smaller than the sort needs");
            return NDT_ERR_CAPACITY;
        }
        g_static_sort_ptr[dev] = p;
        g_static_sort_ctx[dev] = ctx_id;
    }
    *out = g_static_sort_ptr[dev];
    return NDT_OK;
}

}  // namespace ndtgb

extern "C" int ndt_radix_sort_pairs_u64_u32_static(uint64_t* d_keys, uint32_t* d_values,
                                                   uint64_t n, int32_t begin_bit,
                                                   int32_t end_bit, void* stream) {
    using namespace ndtgb;
    if (begin_bit < 0 || end_bit > 64 || begin_bit > end_bit) {
        set_error("static radix sort: bit range must satisfy 0 <= begin_bit <= end_bit <= 64");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    if (n > STATIC_SORT_MAX_PAIRS) {
        set_error("static radix sort: at most 1048576 pairs (fixed 12.25 MiB device scratch)");
        return NDT_ERR_CAPACITY;
    }
    if (n && (!d_keys || !d_values)) {
        set_error("static radix sort: null key or value pointer");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    void* scratch = nullptr;
    int rc = static_sort_scratch(&scratch);
    if (rc) return rc;
    return radix_sort_pairs(d_keys, d_values, (size_t)n, begin_bit, end_bit, scratch,
                            STATIC_SORT_SCRATCH_BYTES, (cudaStream_t)stream);
}

namespace ndtgb {

// ---------------------------------------------------------------------------------------
// Segments of sorted keys.
// ---------------------------------------------------------------------------------------
template <typename K>
__global__ void k_seg_flags(const K* __restrict__ keys, size_t n, uint32_t* __restrict__ flags) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = (i > 0 && keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void k_seg_finish(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ ex,
                             size_t n, uint32_t* __restrict__ seg_ids,
                             uint32_t* __restrict__ starts, uint32_t* __restrict__ num) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t f = flags[i];
    uint32_t sid = ex[i] + f;
    if (seg_ids) seg_ids[i] = sid;
    if (i == 0 || f) starts[sid] = (uint32_t)i;
    if (i == n - 1) *num = sid + 1;
}

size_t detect_segments_temp_bytes(size_t n) {
    return 2 * align_up(n * 4 + 4, 256) + scan_temp_bytes(n);
}

// Segment starts without per-key flags (the map build's form, no segment ids): one block
// per TILE keys counts the tile's segment starts (key != previous key), the tile counts are
// scanned, and the blocks write their starts at the scanned offsets in key order.
template <typename K>
__global__ void __launch_bounds__(BT) k_seg_count(const K* __restrict__ keys, size_t n,
                                                  uint32_t* __restrict__ tile_cnt) {
    __shared__ uint32_t ws[BT / 32];
    const size_t base = (size_t)blockIdx.x * TILE + (size_t)threadIdx.x * ITEMS;
    uint32_t c = 0;
    K prev = base > 0 && base - 1 < n ? keys[base - 1] : K(0);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const size_t i = base + k;
        if (i < n) {
            const K key = keys[i];
            c += (i == 0 || key != prev) ? 1u : 0u;
            prev = key;
        }
    }
    uint32_t tot;
    block_exclusive_scan(c, ws, &tot);
    if (threadIdx.x == 0) tile_cnt[blockIdx.x] = tot;
}

template <typename K>
__global__ void __launch_bounds__(BT) k_seg_write(const K* __restrict__ keys, size_t n,
                                                  const uint32_t* __restrict__ tile_off,
                                                  uint32_t* __restrict__ starts,
                                                  uint32_t* __restrict__ num) {
    __shared__ uint32_t ws[BT / 32];
    const size_t base = (size_t)blockIdx.x * TILE + (size_t)threadIdx.x * ITEMS;
    K kv[ITEMS];
    uint32_t flags = 0, c = 0;
    K prev = base > 0 && base - 1 < n ? keys[base - 1] : K(0);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
        const size_t i = base + k;
        kv[k] = i < n ? keys[i] : K(0);
        const bool f = i < n && (i == 0 || kv[k] != prev);
        prev = kv[k];
        flags |= (f ? 1u : 0u) << k;
        c += f ? 1u : 0u;
    }
    uint32_t tot;
    uint32_t r = tile_off[blockIdx.x] + block_exclusive_scan(c, ws, &tot);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k)
        if (flags >> k & 1u) starts[r++] = (uint32_t)(base + k);
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *num = tile_off[blockIdx.x] + tot;
}

// starts of the runs of equal keys in sorted[0..n), their count in *num_segments;
// temp >= ntiles(n) * 4 bytes
template <typename K>
static int segment_starts(const K* sorted, size_t n, uint32_t* seg_starts,
                          uint32_t* num_segments, void* temp, cudaStream_t s) {
    cudaMemsetAsync(num_segments, 0, 4, s);
    if (n == 0) return cuda_fail(cudaGetLastError(), "segments");
    const uint32_t nb = ntiles(n);
    uint32_t* cnt = (uint32_t*)temp;
    k_seg_count<K><<<nb, BT, 0, s>>>(sorted, n, cnt);
    k_scan_bsums<<<1, BT, 0, s>>>(cnt, nb);
    k_seg_write<K><<<nb, BT, 0, s>>>(sorted, n, cnt, seg_starts, num_segments);
    return cuda_fail(cudaGetLastError(), "segments");
}

template <typename K>
static int detect_segments_t(const K* sorted, size_t n, uint32_t* seg_ids, uint32_t* seg_starts,
                             uint32_t* num_segments, void* temp, size_t temp_bytes,
                             cudaStream_t s) {
    cudaMemsetAsync(num_segments, 0, 4, s);
    if (n == 0) return cuda_fail(cudaGetLastError(), "segments");
    if (temp_bytes < detect_segments_temp_bytes(n)) {
        set_error("detect segments: temporary storage too small");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    char* t = (char*)temp;
    uint32_t* flags = (uint32_t*)t;
    t += align_up(n * 4 + 4, 256);
    uint32_t* ex = (uint32_t*)t;
    t += align_up(n * 4 + 4, 256);
    unsigned g = (unsigned)((n + BT - 1) / BT);
    k_seg_flags<<<g, BT, 0, s>>>(sorted, n, flags);
    int rc = exclusive_scan(flags, ex, n, t, s);
    if (rc) return rc;
    k_seg_finish<<<g, BT, 0, s>>>(flags, ex, n, seg_ids, seg_starts, num_segments);
    return cuda_fail(cudaGetLastError(), "segments");
}

int detect_segments(const uint64_t* sorted, size_t n, uint32_t* seg_ids, uint32_t* seg_starts,
                    uint32_t* num_segments, void* temp, size_t temp_bytes, cudaStream_t s) {
    return detect_segments_t(sorted, n, seg_ids, seg_starts, num_segments, temp, temp_bytes, s);
}

// ---------------------------------------------------------------------------------------
// Cells, bounds and Morton keys.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool finite3(float x, float y, float z) {
    return isfinite(x) && isfinite(y) && isfinite(z);
}

__device__ __forceinline__ void cell_of(const float* p, float res, int32_t* c) {
    c[0] = sat_i32(floorf(p[0] / res));
    c[1] = sat_i32(floorf(p[1] / res));
    c[2] = sat_i32(floorf(p[2] / res));
}

// mm: [0..2] min cell, [3..5] max cell, [6] finite count
__global__ void __launch_bounds__(BT) k_cells_minmax(const float* __restrict__ pts, size_t n,
                                                     float res, int32_t* __restrict__ mm) {
    int32_t mn[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, mx[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    uint32_t cnt = 0;
    for (size_t i = (size_t)blockIdx.x * BT + threadIdx.x; i < n; i += (size_t)gridDim.x * BT) {
        float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        if (!finite3(p[0], p[1], p[2])) continue;
        int32_t c[3];
        cell_of(p, res, c);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = min(mn[a], c[a]);
            mx[a] = max(mx[a], c[a]);
        }
        cnt++;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
            mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
        }
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(&mm[a], mn[a]);
            atomicMax(&mm[3 + a], mx[a]);
        }
        atomicAdd(&mm[6], (int32_t)cnt);
    }
}

__global__ void k_minmax_init(int32_t* mm) {
    if (threadIdx.x < 3) mm[threadIdx.x] = INT32_MAX;
    else if (threadIdx.x < 6) mm[threadIdx.x] = INT32_MIN;
    else if (threadIdx.x == 6) mm[6] = 0;
}

// Morton key of each point's cell relative to the minimum cell, all ones for a non-finite
// point (it sorts last). K = uint32_t when the key's significant bits fit.
template <typename K>
__global__ void __launch_bounds__(BT) k_morton(const float* __restrict__ pts, size_t n, float res,
                                               const int32_t* __restrict__ mm,
                                               K* __restrict__ codes,
                                               uint32_t* __restrict__ idx) {
    size_t i = (size_t)blockIdx.x * BT + threadIdx.x;
    if (i >= n) return;
    float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    K code = ~K(0);
    if (finite3(p[0], p[1], p[2])) {
        int32_t c[3];
        cell_of(p, res, c);
        uint32_t q[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            int64_t d = (int64_t)c[a] - (int64_t)mm[a];
            q[a] = d > 0x1FFFFF ? 0x1FFFFFu : (uint32_t)d;
        }
        code = (K)morton3(q[0], q[1], q[2]);
    }
    codes[i] = code;
    idx[i] = (uint32_t)i;
}

// min / max cell and finite count of the points into mm
static void cell_bounds(const float* pts, size_t n, float res, int32_t* mm, cudaStream_t s) {
    k_minmax_init<<<1, 32, 0, s>>>(mm);
    if (n) {
        unsigned g = (unsigned)std::min<size_t>((n + BT - 1) / BT, 152 * 8);
        k_cells_minmax<<<g, BT, 0, s>>>(pts, n, res, mm);
    }
}

int morton_codes(const float* pts, size_t n, float res, uint64_t* codes, uint32_t* idx,
                 int32_t* mm, cudaStream_t s) {
    cell_bounds(pts, n, res, mm, s);
    if (n) k_morton<uint64_t><<<(unsigned)((n + BT - 1) / BT), BT, 0, s>>>(pts, n, res, mm, codes, idx);
    return cuda_fail(cudaGetLastError(), "morton codes");
}

// ---------------------------------------------------------------------------------------
// Voxel statistics (one thread per segment) and regularisation.
// ---------------------------------------------------------------------------------------

// Cyclic Jacobi for a symmetric 3x3 in f32 (row-major a, eigenvectors in the columns of v).
// It only has to find the eigenvector directions to f32 accuracy: the eigenvalues and the
// regularised covariance and inverse are then formed in FP64 (k_voxel_stats).
__device__ void jacobi3f(float* a, float* v) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) v[i * 3 + j] = (i == j) ? 1.f : 0.f;
#pragma unroll 1
    for (int sweep = 0; sweep < 12; ++sweep) {
        const float off = a[1] * a[1] + a[2] * a[2] + a[5] * a[5];
        const float dg = a[0] * a[0] + a[4] * a[4] + a[8] * a[8];
        if (!(off > 1e-14f * dg)) break;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            const float apq = a[p * 3 + q];
            if (apq == 0.f) continue;
            const float theta = (a[q * 3 + q] - a[p * 3 + p]) / (2.f * apq);
            float t = 1.f / (fabsf(theta) + sqrtf(theta * theta + 1.f));
            if (theta < 0.f) t = -t;
            const float c = 1.f / sqrtf(t * t + 1.f);
            const float sn = t * c;
            a[p * 3 + p] -= t * apq;
            a[q * 3 + q] += t * apq;
            a[p * 3 + q] = a[q * 3 + p] = 0.f;
            const int r = 3 - p - q;
            const float arp = a[r * 3 + p], arq = a[r * 3 + q];
            a[r * 3 + p] = a[p * 3 + r] = c * arp - sn * arq;
            a[r * 3 + q] = a[q * 3 + r] = sn * arp + c * arq;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float vp = v[k * 3 + p], vq = v[k * 3 + q];
                v[k * 3 + p] = c * vp - sn * vq;
                v[k * 3 + q] = sn * vp + c * vq;
            }
        }
    }
}

// FP64 cyclic Jacobi sweeps on B = V^T A V, rotating V along (B and V row-major, V's columns
// the eigenvector estimates), until the reference's rule 2 off^2 < 1e-28 diag^2 holds or
// max_sweeps pass. Started from an orthonormalised f32 solution, B is diagonal to about 1e-7
// of its scale and one or two sweeps reach FP64 accuracy.
__device__ void jacobi3_refine(double* B, double* V, int max_sweeps) {
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        const double off = B[1] * B[1] + B[2] * B[2] + B[5] * B[5];
        const double dg = B[0] * B[0] + B[4] * B[4] + B[8] * B[8];
        if (2.0 * off <= 1e-28 * dg) break;
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
            const double bpq = B[p * 3 + q];
            if (bpq == 0.0) continue;
            const double theta = (B[q * 3 + q] - B[p * 3 + p]) / (2.0 * bpq);
            double t = 1.0 / (fabs(theta) + sqrt(theta * theta + 1.0));
            if (theta < 0.0) t = -t;
            const double c = 1.0 / sqrt(t * t + 1.0);
            const double sn = t * c;
            B[p * 3 + p] -= t * bpq;
            B[q * 3 + q] += t * bpq;
            B[p * 3 + q] = B[q * 3 + p] = 0.0;
            const int r = 3 - p - q;
            const double brp = B[r * 3 + p], brq = B[r * 3 + q];
            B[r * 3 + p] = B[p * 3 + r] = c * brp - sn * brq;
            B[r * 3 + q] = B[q * 3 + r] = sn * brp + c * brq;
            for (int k = 0; k < 3; ++k) {
                const double vp = V[k * 3 + p], vq = V[k * 3 + q];
                V[k * 3 + p] = c * vp - sn * vq;
                V[k * 3 + q] = sn * vp + c * vq;
            }
        }
    }
}

// FP64 Rayleigh quotient v^T A v / v^T v of an f32 unit vector v (|v|^2 = 1 +- 1e-7, so
// 1 / v^T v = 2 - v^T v to FP64 rounding): FP64-accurate for an eigenvalue, since its error
// is quadratic in v's direction error. *w receives 1 / v^T v.
__device__ __forceinline__ double rayleigh(const double* A, const double* v, double* w) {
    double num = 0.0;
    for (int rr = 0; rr < 3; ++rr)
        num += v[rr] * (A[rr * 3] * v[0] + A[rr * 3 + 1] * v[1] + A[rr * 3 + 2] * v[2]);
    const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    *w = 2.0 - vv;
    return num * *w;
}

// Inverse of a symmetric positive definite 3x3 by its adjugate (FP64); false unless det > 0.
__device__ __forceinline__ bool inverse_sym3(const double* C, float* icov6) {
    const double c00 = C[4] * C[8] - C[5] * C[5];
    const double c01 = C[2] * C[5] - C[1] * C[8];
    const double c02 = C[1] * C[5] - C[2] * C[4];
    const double c11 = C[0] * C[8] - C[2] * C[2];
    const double c12 = C[1] * C[2] - C[0] * C[5];
    const double c22 = C[0] * C[4] - C[1] * C[1];
    const double det = C[0] * c00 + C[1] * c01 + C[2] * c02;
    if (!(det > 0.0)) return false;
    const double id = 1.0 / det;
    icov6[0] = (float)(c00 * id);
    icov6[1] = (float)(c01 * id);
    icov6[2] = (float)(c02 * id);
    icov6[3] = (float)(c11 * id);
    icov6[4] = (float)(c12 * id);
    icov6[5] = (float)(c22 * id);
    return true;
}

// First-order correction of an f32 eigenvector v (eigenvalue lam) against the eigenvectors
// v_j of the set `others` (bit mask): v += sum_j (v_j^T (A v - lam v)) / (lam - lam_j) v_j
// (w_j = 1 / v_j^T v_j). The direction error drops from about 1e-7 lambda_max / gap to its
// square; the 1 / gap factors need only f32 accuracy.
__device__ __forceinline__ void refine_vector(const double* A, double* v, double lam,
                                              const double (*vs)[3], const double* lams,
                                              const double* ws, int others) {
    double r[3];
    for (int rr = 0; rr < 3; ++rr)
        r[rr] = A[rr * 3] * v[0] + A[rr * 3 + 1] * v[1] + A[rr * 3 + 2] * v[2] - lam * v[rr];
    double dv[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < 3; ++j) {
        if (!(others >> j & 1)) continue;
        const double proj = vs[j][0] * r[0] + vs[j][1] * r[1] + vs[j][2] * r[2];
        const double inv = (double)(1.f / (float)(lam - lams[j]));
        const double c = proj * ws[j] * inv;
        for (int k = 0; k < 3; ++k) dv[k] += c * vs[j][k];
    }
    for (int k = 0; k < 3; ++k) v[k] += dv[k];
}

// Regularised covariance and inverse of the FP64 covariance A (Voxel::from_statistics /
// regularize_covariance, src/ndt_cuda/src/voxel_grid/types.rs:54-190): eigenvalues below
// ratio * lambda_max are raised to it; cov' = V diag(clamped) V^T when any was, else A;
// inverse V diag(1 / clamped) V^T. a32 / V32: the f32 Jacobi's eigenvalues (diagonal) and
// eigenvectors (columns). Which eigenvalues clamp is read from the f32 eigenvalues when they
// lie clear of the threshold (1e-4 relative, against their 1e-5 error there), and the clamped
// ones lie at least lambda_max / 1000 below the others (an f32 direction error of 1e-4 at most,
// 1e-8 after the first-order refinement); then, with FP64 Rayleigh quotients as
// the eigenvalues:
//   - nothing clamps: cov' = A, inverse by the adjugate (A's condition number <= 1 / ratio);
//   - one clamps: cov' = A + (thr - lambda_c) v_c v_c^T, v_c refined against the other two;
//   - two clamp: cov' = thr I + (lambda_u - thr) v_u v_u^T, v_u refined against the other
//     two (mixing inside the clamped pair then cannot matter);
//   and the inverse by the adjugate of cov'.
// Anything else takes the full FP64 route: the f32 eigenvectors orthonormalised
// (Gram-Schmidt), Jacobi sweeps on V^T A V to the reference's stopping rule, and the
// reconstruction from the eigen-decomposition. Every route is FP64-accurate, so the f32
// outputs agree with an FP64 eigen-decomposition to f32 rounding.
__device__ bool regularize(const double* A, const float* a32, const float* V32, float ratio,
                           SegRec& r) {
    const float e32[3] = {a32[0], a32[4], a32[8]};
    const float mx32 = fmaxf(e32[0], fmaxf(e32[1], e32[2]));
    bool fast = mx32 > 0.f;
    int clamp = 0;  // bit i: eigenvalue i clamps
    if (fast) {
        const float thr32 = mx32 * ratio;
        for (int i = 0; i < 3; ++i) {
            if (e32[i] <= thr32 * 0.9999f) {
                clamp |= 1 << i;
            } else if (!(e32[i] >= thr32 * 1.0001f)) {
                fast = false;
            }
        }
        for (int i = 0; i < 3 && fast; ++i)
            for (int j = 0; j < 3; ++j)
                if ((clamp >> i & 1) && !(clamp >> j & 1) && e32[j] - e32[i] < 0.001f * mx32)
                    fast = false;
    }
    if (fast) {
        if (!clamp) {
            for (int q = 0; q < 9; ++q) r.cov[q] = (float)A[q];
            return inverse_sym3(A, r.icov);
        }
        double v[3][3], w[3], lam[3];
        for (int i = 0; i < 3; ++i) {
            for (int k = 0; k < 3; ++k) v[i][k] = (double)V32[k * 3 + i];
            lam[i] = rayleigh(A, v[i], &w[i]);
        }
        const double mx = fmax(lam[0], fmax(lam[1], lam[2]));
        if (!(mx > 0.0)) return false;
        const double thr = mx * (double)ratio;
        const int one = __popc(clamp) == 1;
        const int t = one ? __ffs(clamp) - 1 : __ffs(7 & ~clamp) - 1;  // the vector to refine
        double u[3] = {v[t][0], v[t][1], v[t][2]};
        refine_vector(A, u, lam[t], v, lam, w, 7 & ~(1 << t));
        const double wu = 2.0 - (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        double C[9];
        const double c = one ? (thr - lam[t]) * wu : (lam[t] - thr) * wu;
        for (int rr = 0; rr < 3; ++rr)
            for (int cc = rr; cc < 3; ++cc) {  // upper triangle, mirrored: C stays symmetric
                const double base = one ? A[rr * 3 + cc] : (rr == cc ? thr : 0.0);
                C[rr * 3 + cc] = C[cc * 3 + rr] = base + c * u[rr] * u[cc];
            }
        for (int q = 0; q < 9; ++q) r.cov[q] = (float)C[q];
        return inverse_sym3(C, r.icov);
    }
    // full FP64 route: orthonormal basis from the f32 eigenvectors, Jacobi sweeps on V^T A V
    double V[9];
    for (int q = 0; q < 9; ++q) V[q] = (double)V32[q];
    for (int i = 0; i < 3; ++i) {
        for (int j = 0; j < i; ++j) {
            const double d = V[i] * V[j] + V[3 + i] * V[3 + j] + V[6 + i] * V[6 + j];
            for (int k = 0; k < 3; ++k) V[k * 3 + i] -= d * V[k * 3 + j];
        }
        const double inv = 1.0 / sqrt(V[i] * V[i] + V[3 + i] * V[3 + i] + V[6 + i] * V[6 + i]);
        for (int k = 0; k < 3; ++k) V[k * 3 + i] *= inv;
    }
    double AV[9], B[9];
    for (int rr = 0; rr < 3; ++rr)
        for (int cc = 0; cc < 3; ++cc)
            AV[rr * 3 + cc] =
                A[rr * 3] * V[cc] + A[rr * 3 + 1] * V[3 + cc] + A[rr * 3 + 2] * V[6 + cc];
    for (int rr = 0; rr < 3; ++rr)
        for (int cc = rr; cc < 3; ++cc)
            B[rr * 3 + cc] = B[cc * 3 + rr] =
                V[rr] * AV[cc] + V[3 + rr] * AV[3 + cc] + V[6 + rr] * AV[6 + cc];
    jacobi3_refine(B, V, 4);
    const double ev[3] = {B[0], B[4], B[8]};
    const double mx = fmax(ev[0], fmax(ev[1], ev[2]));
    if (!(mx > 0.0)) return false;
    const double thr = mx * (double)ratio;
    int needs = 0;
    double cl[3], icl[3];
    for (int i = 0; i < 3; ++i) {
        cl[i] = ev[i] < thr ? thr : ev[i];
        if (ev[i] < thr) needs = 1;
        icl[i] = 1.0 / cl[i];
    }
    for (int rr = 0; rr < 3; ++rr)
        for (int cc = rr; cc < 3; ++cc) {
            double sr = 0.0, si = 0.0;
            for (int k = 0; k < 3; ++k) {
                const double vv = V[rr * 3 + k] * V[cc * 3 + k];
                sr += vv * cl[k];
                si += vv * icl[k];
            }
            const float fc = (float)(needs ? sr : A[rr * 3 + cc]);
            r.cov[rr * 3 + cc] = r.cov[cc * 3 + rr] = fc;
            r.icov[rr == 0 ? cc : (rr == 1 ? 2 + cc : 5)] = (float)si;
        }
    return true;
}

// ---- Exact moments ------------------------------------------------------------------------
// Per axis, a quantum 2^e0 from the voxel's cell k: its points lie within
// B = max(|k|, |k + 1|) resolutions of zero, below 2^EB (B < 2^EB with a 1e-3 margin for the
// f32 cell rule). For a cell at least one resolution from zero every point is at least about
// B / 2, a multiple of its ulp >= 2^(EB - 26): e0 = EB - 26. A cell next to zero (k = 0 or
// -1) holds values of any size: e0 = EB - 40. Each point is then m 2^e0 with an integer
// |m| < 2^40, exact unless it is a value below 2^(e0 + 23) whose low bits fall under the
// quantum (it is rounded then, by at most 2^-41 of the cell's reach). With d = m - m_first
// (|d| < 2^41) the sums S1 = sum d (int64) and S2 = sum d d^T (128-bit) are exact for up to
// 65536 points and independent of the order of the points. From them:
//   - the mean of an axis whose points were all exact and whose sum (S1 + n m_first) has at
//     most 53 significant bits above the coarsest power of two dividing every point: every
//     partial sum of these same-sign values (one cell) is then an FP64 number, so the FP64
//     running sum in input order (build_voxel_grid_cpu, src/ndt_cuda/src/voxel_grid/cpu.rs:
//     51-75) never rounds and equals it, and fl(sum / n) is its mean bit for bit. Any other
//     axis takes that running sum in input order (moments_mean_fp64);
//   - the centred covariance (n S2 - S1 S1^T) 2^(e0a + e0b) / (n (n - 1)) from the 128-bit
//     numerator rounded once to FP64 and the FP64 reciprocal of n (n - 1): within a few
//     roundings of the exact value whatever the order of the points (a tile merge and a full
//     build of the same cell agree bit for bit).
// A value beyond the cell's reach or non-finite sends the voxel to the FP64 two-pass formula.
struct ExactMoments {
    int32_t e0[3];            // quantum exponent per axis
    int32_t tz[3];            // fewest trailing zero bits of a non-zero m (the coarse quantum)
    long long m0[3];          // the first point in quanta
    long long s1[3];
    long long s2h[6];         // xx, xy, xz, yy, yz, zz as 128-bit (hi, lo)
    unsigned long long s2l[6];
    bool rep[3];              // every point of the axis an exact multiple of 2^e0
    bool ok;                  // every point within the cell's reach
};

// m of one coordinate in quanta 2^e0 (rounded to nearest; rep cleared when inexact, ok when
// beyond 2^(e0 + 40))
__device__ __forceinline__ long long exact_units(float x, int32_t e0, bool& rep, int32_t& tz,
                                                 bool& ok) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t ex = (b >> 23) & 0xFFu;
    if (ex == 0u) {  // +-0 is exact; a subnormal rounds to 0 quanta
        rep &= (b << 1) == 0u;
        return 0;
    }
    ok &= ex != 0xFFu;
    const int32_t sh = (int32_t)ex - 150 - e0;
    ok &= sh <= 16;
    const unsigned long long M = (b & 0x7FFFFFu) | 0x800000u;
    unsigned long long m;
    if (sh >= 0) {
        m = M << (sh & 63);
    } else if (sh > -25) {
        const int r = -sh;
        rep &= (M & ((1ull << r) - 1ull)) == 0ull;
        m = (M + (1ull << (r - 1))) >> r;
    } else {
        rep = false;
        m = 0;
    }
    if (m) tz = min(tz, __ffsll((long long)m) - 1);
    return (b >> 31) ? -(long long)m : (long long)m;
}

__device__ __forceinline__ void add_prod128(long long& hi, unsigned long long& lo, long long a,
                                            long long b) {
    const unsigned long long pl = (unsigned long long)a * (unsigned long long)b;
    const long long ph = __mul64hi(a, b);
    const unsigned long long s = lo + pl;
    hi += ph + (s < lo ? 1ll : 0ll);
    lo = s;
}

// quanta of the cell `coord` (the f32 cell index of the voxel) and the first point
__device__ __forceinline__ void exact_begin(ExactMoments& em, const float* p, const int32_t* coord,
                                            float res) {
    em.ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float k = (float)coord[a];
        const float reach = fmaxf(fabsf(k), fabsf(k + 1.f)) * res * 1.001f;
        int eb;
        frexpf(reach, &eb);  // reach < 2^eb
        em.e0[a] = eb - ((coord[a] == 0 || coord[a] == -1) ? 40 : 26);
        em.tz[a] = 64;
        em.rep[a] = true;
        em.s1[a] = 0;
        em.m0[a] = exact_units(p[a], em.e0[a], em.rep[a], em.tz[a], em.ok);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        em.s2h[k] = 0;
        em.s2l[k] = 0ull;
    }
}

__device__ __forceinline__ void exact_add(ExactMoments& em, const float* p) {
    long long d[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        d[a] = exact_units(p[a], em.e0[a], em.rep[a], em.tz[a], em.ok) - em.m0[a];
        em.s1[a] += d[a];
    }
    add_prod128(em.s2h[0], em.s2l[0], d[0], d[0]);
    add_prod128(em.s2h[1], em.s2l[1], d[0], d[1]);
    add_prod128(em.s2h[2], em.s2l[2], d[0], d[2]);
    add_prod128(em.s2h[3], em.s2l[3], d[1], d[1]);
    add_prod128(em.s2h[4], em.s2l[4], d[1], d[2]);
    add_prod128(em.s2h[5], em.s2l[5], d[2], d[2]);
}

// 2^e as an FP64 (normal range)
__device__ __forceinline__ double pow2d(int e) {
    return __longlong_as_double((long long)(e + 1023) << 52);
}

// A signed 128-bit integer (hi, lo) rounded once to the nearest FP64 (ties to even)
__device__ __forceinline__ double i128_to_double(long long hi, unsigned long long lo) {
    const bool neg = hi < 0;
    unsigned long long uh = (unsigned long long)hi, ul = lo;
    if (neg) {
        ul = ~ul + 1ull;
        uh = ~uh + (ul == 0ull ? 1ull : 0ull);
    }
    if (uh == 0ull) {
        const double v = __ull2double_rn(ul);
        return neg ? -v : v;
    }
    const int lz = __clzll((long long)uh);
    unsigned long long top = lz ? (uh << lz) | (ul >> (64 - lz)) : uh;
    const unsigned long long rest = lz ? ul << lz : ul;
    if (rest != 0ull) top |= 1ull;  // sticky: the discarded bits decide ties and halves
    const double v = __ull2double_rn(top) * pow2d(64 - lz);
    return neg ? -v : v;
}

// Mean and covariance from exact sums over n points. Returns a mask of the axes whose mean
// the exact sums cannot give (bit a set: take the FP64 running sum of axis a).
__device__ __forceinline__ int exact_finish(const ExactMoments& em, uint32_t n, double* mean,
                                            double* A) {
    const double nn = (double)n;
    int redo = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const long long tot = em.s1[a] + (long long)n * em.m0[a];
        const unsigned long long mag = tot < 0 ? (unsigned long long)(-tot) : (unsigned long long)tot;
        const int sig = mag ? 64 - __clzll((long long)mag) - min(em.tz[a], 63) : 0;
        if (em.rep[a] && sig <= 53) {
            mean[a] = (__ll2double_rn(tot) * pow2d(em.e0[a])) / nn;
        } else {
            redo |= 1 << a;
        }
    }
    const double inv_den = 1.0 / (nn * (double)(n - 1u));
    const int ia[6] = {0, 0, 0, 1, 1, 2}, ib[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        // n S2 (128-bit times a small unsigned) minus S1_a S1_b (64 x 64 -> 128), exact
        const unsigned long long nl = em.s2l[k] * (unsigned long long)n;
        const long long nh = em.s2h[k] * (long long)n +
                             (long long)__umul64hi(em.s2l[k], (unsigned long long)n);
        const long long pa = em.s1[ia[k]], pb = em.s1[ib[k]];
        const unsigned long long ql = (unsigned long long)pa * (unsigned long long)pb;
        const long long qh = __mul64hi(pa, pb);
        const unsigned long long rl = nl - ql;
        const long long rh = nh - qh - (nl < ql ? 1ll : 0ll);
        const double v =
            i128_to_double(rh, rl) * pow2d(em.e0[ia[k]] + em.e0[ib[k]]) * inv_den;
        A[ia[k] * 3 + ib[k]] = A[ib[k] * 3 + ia[k]] = v;
    }
    return redo;
}

// The FP64 running sums of the axes in `axes` (bit mask) over the points in input order, the
// means fl(sum / n) (build_voxel_grid_cpu's accumulation)
template <class Each>
__device__ __noinline__ void moments_mean_fp64(Each each, uint32_t cnt, int axes, double* mean) {
    double sum[3] = {0.0, 0.0, 0.0};
    each([&](const float* p) {
        sum[0] += (double)p[0];
        sum[1] += (double)p[1];
        sum[2] += (double)p[2];
    });
    for (int a = 0; a < 3; ++a)
        if (axes >> a & 1) mean[a] = sum[a] / (double)cnt;
}

// FP64 centred two-pass moments of one voxel's points, visited in input order by each(f) (f
// called with a pointer to each point's xyz): mean = sum / n, covariance = sum of the centred
// products / (n - 1). The route for voxels the exact sums cannot take.
template <class Each>
__device__ __noinline__ void moments_two_pass(Each each, uint32_t cnt, double* mean, double* A) {
    double sum[3] = {0.0, 0.0, 0.0};
    each([&](const float* p) {
        sum[0] += (double)p[0];
        sum[1] += (double)p[1];
        sum[2] += (double)p[2];
    });
    const double nn = (double)cnt;
    for (int a = 0; a < 3; ++a) mean[a] = sum[a] / nn;
    // upper triangle xx, xy, xz, yy, yz, zz (the products are symmetric bit for bit)
    double sq[6] = {0, 0, 0, 0, 0, 0};
    each([&](const float* p) {
        const double d0 = (double)p[0] - mean[0], d1 = (double)p[1] - mean[1],
                     d2 = (double)p[2] - mean[2];
        sq[0] += d0 * d0;
        sq[1] += d0 * d1;
        sq[2] += d0 * d2;
        sq[3] += d1 * d1;
        sq[4] += d1 * d2;
        sq[5] += d2 * d2;
    });
    const double nm1 = nn - 1.0;
    A[0] = sq[0] / nm1;
    A[1] = A[3] = sq[1] / nm1;
    A[2] = A[6] = sq[2] / nm1;
    A[4] = sq[3] / nm1;
    A[5] = A[7] = sq[4] / nm1;
    A[8] = sq[5] / nm1;
}

// Regularised covariance, inverse and mean of a voxel from its FP64 mean and covariance
// A. GB300's FP64 rate is a small fraction of its FP32 rate: the eigenvector directions come
// from an f32 Jacobi, and FP64 is spent only where the outputs depend on it (regularize).
__device__ __forceinline__ bool voxel_finish(const double* mean, const double* A, float ratio,
                                             SegRec& r) {
    float a32[9], V32[9];
    for (int q = 0; q < 9; ++q) a32[q] = (float)A[q];
    jacobi3f(a32, V32);
    if (!regularize(A, a32, V32, ratio, r)) return false;
    for (int q = 0; q < 3; ++q) r.mean[q] = (float)mean[q];
    return true;
}

// Largest voxel whose sums stay exact (S1 below 2^57, S2 below 2^98 with |d| < 2^41)
constexpr uint32_t EXACT_MAX_POINTS = 65536;

// Statistics of one voxel by one thread: count, then exact moments (FP64 running sums for
// the axes whose mean they cannot give) when the voxel has at most EXACT_MAX_POINTS points
// within the exact bounds, else FP64 two-pass moments; then voxel_finish. each(f) visits the
// voxel's points in input order; first: its first point. r.coord (the voxel's cell) is the
// caller's.
template <class Each>
__device__ __forceinline__ bool voxel_stats(Each each, const float* first, uint32_t cnt,
                                            int min_points, float ratio, float res, SegRec& r) {
    r.count = cnt;
    if ((int)cnt < min_points) return false;
    double mean[3], A[9];
    bool exact = cnt <= EXACT_MAX_POINTS;
    ExactMoments em;
    if (exact) {
        exact_begin(em, first, r.coord, res);
        each([&](const float* p) { exact_add(em, p); });
        exact = em.ok;
    }
    if (exact) {
        const int redo = exact_finish(em, cnt, mean, A);
        if (redo) moments_mean_fp64(each, cnt, redo, mean);
    } else {
        moments_two_pass(each, cnt, mean, A);
    }
    return voxel_finish(mean, A, ratio, r);
}

// Segment sizes as sort keys: segments visited largest first (key 0xFFFF - min(count,
// 0xFFFF)), so the threads of a warp take segments of nearly equal size and the longest
// start first.
__global__ void k_seg_size_keys(const uint32_t* __restrict__ starts, uint32_t S, uint32_t nf,
                                uint32_t* __restrict__ keys, uint32_t* __restrict__ order) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const uint32_t e = s + 1 < S ? starts[s + 1] : nf;
    keys[s] = 0xFFFFu - min(e - starts[s], 0xFFFFu);
    order[s] = s;
}

// Voxels of at least WARP_SEG_MIN points are summed by a whole warp (exact sums of the lanes'
// strided shares, added over the lanes in 128-bit), up to EXACT_MAX_POINTS points.
constexpr uint32_t WARP_SEG_MIN = 48;

// 128-bit (hi, lo) sum over the warp's lanes (every lane ends with the total)
__device__ __forceinline__ void warp_sum128(long long& hi, unsigned long long& lo) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ol = __shfl_xor_sync(0xffffffffu, lo, o);
        const long long oh = __shfl_xor_sync(0xffffffffu, hi, o);
        const unsigned long long s = lo + ol;
        hi = hi + oh + (s < lo ? 1ll : 0ll);
        lo = s;
    }
}

// f(point) for the points sidx[k], k = b, b + step, ... < e, in that order, with the loads of
// four points issued together (the gathers are random reads of the map: four in flight per
// thread instead of one)
template <class F>
__device__ __forceinline__ void visit_points(const float* __restrict__ pts,
                                             const uint32_t* __restrict__ sidx, uint32_t b,
                                             uint32_t e, uint32_t step, F f) {
    uint32_t k = b;
    for (; k + 3 * step < e; k += 4 * step) {
        float v[4][3];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float* q = pts + 3 * (size_t)sidx[k + j * step];
            v[j][0] = q[0];
            v[j][1] = q[1];
            v[j][2] = q[2];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) f(v[j]);
    }
    for (; k < e; k += step) f(pts + 3 * (size_t)sidx[k]);
}

// Exact sums of one large segment, as a warp leaves them for the thread that finishes it
struct SegSums {
    long long s1[3];
    long long hi[6];
    unsigned long long lo[6];
    int32_t tz[3];
    int32_t flags;  // bit 0: the exact route holds; bits 1-3: axis a's points all exact
};

// Number of visit-order segments with at least WARP_SEG_MIN points (sorted size keys ascend)
__device__ __forceinline__ uint32_t large_segments(const uint32_t* __restrict__ skey, uint32_t S) {
    uint32_t lo = 0, hi = S;
    const uint32_t lim = 0xFFFFu - WARP_SEG_MIN;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (skey[mid] <= lim) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Exact sums of the large segments (the first W in visit order, order[t], largest first),
// one warp per segment at a time (lanes take strided shares, the 128-bit sums are added over
// the lanes), into sums[t]. k_voxel_stats finishes them one per thread.
__global__ void __launch_bounds__(128) k_segment_sums(
    const float* __restrict__ pts, const uint32_t* __restrict__ sidx,
    const uint32_t* __restrict__ starts, const uint32_t* __restrict__ order,
    const uint32_t* __restrict__ skey, uint32_t S, uint32_t nf, float res, int min_points,
    SegSums* __restrict__ sums) {
    __shared__ uint32_t sW;
    if (threadIdx.x == 0) sW = large_segments(skey, S);
    __syncthreads();
    const uint32_t W = sW;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < W; t += warps) {
        const uint32_t s = order[t];
        const uint32_t b = starts[s];
        const uint32_t e = (s + 1 < S) ? starts[s + 1] : nf;
        const uint32_t cnt = e - b;
        if ((int)cnt < min_points) continue;
        const float* first = pts + 3 * (size_t)sidx[b];
        int32_t coord[3];
        cell_of(first, res, coord);
        ExactMoments em;
        exact_begin(em, first, coord, res);
        visit_points(pts, sidx, b + lane, e, 32u, [&](const float* p) { exact_add(em, p); });
        const bool exact = __all_sync(0xffffffffu, em.ok) && cnt <= EXACT_MAX_POINTS;
        int flags = exact ? 1 : 0;
        SegSums& o = sums[t];
        if (exact) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
#pragma unroll
                for (int k = 16; k > 0; k >>= 1) {
                    em.s1[a] += __shfl_xor_sync(0xffffffffu, em.s1[a], k);
                    em.tz[a] = min(em.tz[a], __shfl_xor_sync(0xffffffffu, em.tz[a], k));
                }
                if (__all_sync(0xffffffffu, em.rep[a])) flags |= 2 << a;
            }
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                long long h = em.s2h[k];
                unsigned long long l = em.s2l[k];
                warp_sum128(h, l);
                if (lane == 0) {
                    o.hi[k] = h;
                    o.lo[k] = l;
                }
            }
            if (lane == 0)
                for (int a = 0; a < 3; ++a) {
                    o.s1[a] = em.s1[a];
                    o.tz[a] = em.tz[a];
                }
        }
        if (lane == 0) o.flags = flags;
    }
}

// One thread per segment in visit order (order[t], largest first; skey[t] its sorted size
// key). The first W (WARP_SEG_MIN points or more) are finished from their sums in sums[t]
// (k_segment_sums); the others are summed here. Every segment's record gets its cell and
// count (a tile merge reads them for cells shared between tiles); valid[s] marks the voxels.
__global__ void __launch_bounds__(128) k_voxel_stats(
    const float* __restrict__ pts, const uint32_t* __restrict__ sidx,
    const uint32_t* __restrict__ starts, const uint32_t* __restrict__ order,
    const uint32_t* __restrict__ skey, const SegSums* __restrict__ sums, uint32_t S,
    uint32_t nf, float res, int min_points, float ratio, SegRec* __restrict__ rec,
    uint32_t* __restrict__ valid) {
    __shared__ uint32_t sW;
    if (threadIdx.x == 0) sW = large_segments(skey, S);
    __syncthreads();
    const uint32_t W = sW;
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S) return;
    const uint32_t s = order[t];
    const uint32_t b = starts[s];
    const uint32_t e = (s + 1 < S) ? starts[s + 1] : nf;
    const uint32_t cnt = e - b;
    const float* first = pts + 3 * (size_t)sidx[b];
    SegRec r;
    cell_of(first, res, r.coord);
    auto each = [&](auto f) { visit_points(pts, sidx, b, e, 1u, f); };
    bool ok;
    if (t < W) {
        r.count = cnt;
        ok = false;
        if ((int)cnt >= min_points) {
            double mean[3], A[9];
            const SegSums& ss = sums[t];
            const int flags = ss.flags;
            if (flags & 1) {
                ExactMoments em;
                exact_begin(em, first, r.coord, res);
                for (int a = 0; a < 3; ++a) {
                    em.s1[a] = ss.s1[a];
                    em.tz[a] = ss.tz[a];
                    em.rep[a] = (flags >> (a + 1)) & 1;
                }
                for (int k = 0; k < 6; ++k) {
                    em.s2h[k] = ss.hi[k];
                    em.s2l[k] = ss.lo[k];
                }
                const int redo = exact_finish(em, cnt, mean, A);
                if (redo) moments_mean_fp64(each, cnt, redo, mean);
            } else {
                moments_two_pass(each, cnt, mean, A);
            }
            ok = voxel_finish(mean, A, ratio, r);
        }
    } else {
        ok = voxel_stats(each, first, cnt, min_points, ratio, res, r);
    }
    rec[s] = r;
    valid[s] = ok ? 1u : 0u;
}

__global__ void k_voxel_compact(const SegRec* __restrict__ rec, const uint32_t* __restrict__ valid,
                                const uint32_t* __restrict__ rank,
                                const uint32_t* __restrict__ num_seg, int32_t* __restrict__ coord,
                                float4* __restrict__ mean4, float* __restrict__ cov,
                                float* __restrict__ icov, uint32_t* __restrict__ count) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= *num_seg || !valid[s]) return;
    uint32_t v = rank[s];
    const SegRec& r = rec[s];
    coord[3 * v] = r.coord[0];
    coord[3 * v + 1] = r.coord[1];
    coord[3 * v + 2] = r.coord[2];
    mean4[v] = make_float4(r.mean[0], r.mean[1], r.mean[2], __uint_as_float(r.count));
    for (int q = 0; q < 9; ++q) cov[9 * (size_t)v + q] = r.cov[q];
    const float* c = r.icov;
    float full[9] = {c[0], c[1], c[2], c[1], c[3], c[4], c[2], c[4], c[5]};
    for (int q = 0; q < 9; ++q) icov[9 * (size_t)v + q] = full[q];
    count[v] = r.count;
}

__global__ void k_hash_insert(const int32_t* __restrict__ coord, const float4* __restrict__ mean4,
                              const float* __restrict__ icov, uint32_t nv, MapView m,
                              uint4* __restrict__ slots, float4* __restrict__ slot_icov,
                              int32_t* __restrict__ slot_vidx, uint32_t* __restrict__ max_probe,
                              uint32_t* __restrict__ status) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t disp = 0;  // this voxel's displacement from its home slot
    if (v < nv) {
        const int32_t gx = coord[3 * v], gy = coord[3 * v + 1], gz = coord[3 * v + 2];
        uint32_t key, s;
        cell_slot(m, gx, gy, gz, key, s);  // every voxel lies inside the map's bounding box
        bool placed = false;
        for (uint32_t j = 0; j <= m.mask; ++j) {
            const uint32_t old = atomicCAS(&slots[s].x, EMPTY_KEY, key);
            if (old == EMPTY_KEY) {
                const float4 mu = mean4[v];
                slots[s].y = __float_as_uint(mu.x);
                slots[s].z = __float_as_uint(mu.y);
                slots[s].w = __float_as_uint(mu.z);
                const float* c = icov + 9 * (size_t)v;
                slot_icov[2 * (size_t)s] = make_float4(c[0], c[1], c[2], c[4]);
                slot_icov[2 * (size_t)s + 1] = make_float4(c[5], c[8], 0.f, 0.f);
                slot_vidx[s] = (int32_t)v;
                disp = j;
                placed = true;
                break;
            }
            s = (s + 1) & m.mask;
        }
        if (!placed) atomicOr(status, ST_HASH_FULL);
    }
    // the largest displacement: one atomic per warp that has a displaced voxel (3M threads on
    // one counter would queue at its L2 slice)
    disp = __reduce_max_sync(0xffffffffu, disp);
    if ((threadIdx.x & 31u) == 0 && disp) atomicMax(max_probe, disp);
}

// Dense cell index: every occupied hash slot writes {centroid, slot} into the entry of its
// cell (the grid was set to all-ones first: slot -1 marks an empty cell).
__global__ void k_grid_fill(MapView m, float4* __restrict__ grid) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > m.mask) return;
    const uint4 v = m.slots[s];
    if (v.x == EMPTY_KEY) return;
    const uint32_t lx = v.x & ((1u << m.bits[0]) - 1u);
    const uint32_t ly = (v.x >> m.bits[0]) & ((1u << m.bits[1]) - 1u);
    const uint32_t lz = v.x >> (m.bits[0] + m.bits[1]);
    const size_t idx = ((size_t)lx * m.ext[1] + ly) * m.ext[2] + lz;
    grid[idx] = make_float4(__uint_as_float(v.y), __uint_as_float(v.z), __uint_as_float(v.w),
                            __int_as_float((int32_t)s));
}

// Neighbourhood masks (layout in MapView::nmask), scattered from the voxels: the voxel in
// local cell v is neighbour d = (dx, dy, dz) of cell v - d, so it sets bit
// 9 (dx + 1) + 3 (dy + 1) + (dz + 1) of that cell's mask (or octant masks), at grown-box
// position v - d + 1 (always inside the grown box). One thread per hash slot; the masks start
// at zero, and OR is order-free, so the result does not depend on the threads' order. The
// work goes with the number of voxels, not with the box.
// A bit is set only where the voxel's centroid can pass the radius test from some point of
// cell v - d (of that octant of it): its distance to the cell's (octant's) box is at most the
// radius, widened by 1e-5 of it and by 1e-6 cell widths per cell of distance from the origin
// (the f32 rounding of a point's cell and octant and of the f32 distance test). A cleared bit
// names a neighbour no point there accepts, so neighbour lists are those of the full 27-cell
// search. On the 5M-point 400 m map at 2 m a scan point tests 16.3 candidates with one mask
// per cell and 9.0 with octant masks, of which it accepts 5.45.
template <bool OCT>
__global__ void k_grid_mask(MapView m, uint32_t* __restrict__ nmask) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s > m.mask) return;
    const uint4 sv = m.slots[s];
    const uint32_t key = sv.x;
    if (key == EMPTY_KEY) return;
    const uint32_t v[3] = {key & ((1u << m.bits[0]) - 1u),
                           (key >> m.bits[0]) & ((1u << m.bits[1]) - 1u),
                           key >> (m.bits[0] + m.bits[1])};
    const float mu[3] = {__uint_as_float(sv.y), __uint_as_float(sv.z), __uint_as_float(sv.w)};
    const float res = m.res, half = 0.5f * res;
    // gap[a][d_a + 1][h]: distance along axis a from the centroid to the box of the cell at
    // offset -d (h = 0: the whole cell, or with octants its lower half; h = 1: its upper half)
    float gap[3][3][2], far = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float c = (float)((int64_t)v[a] + m.min_cell[a]);
        const float lo = fmaxf(mu[a] - c * res, 0.f);          // above the voxel's cell floor
        const float hi = fmaxf((c + 1.f) * res - mu[a], 0.f);  // below its ceiling
        far = fmaxf(far, fabsf(c) + 2.f);
        if constexpr (!OCT) {
            gap[a][2][0] = gap[a][2][1] = lo;  // d_a = +1: the cell below the voxel's
            gap[a][0][0] = gap[a][0][1] = hi;  // d_a = -1: the cell above
            gap[a][1][0] = gap[a][1][1] = 0.f;
        } else {
            gap[a][2][0] = lo + half;
            gap[a][2][1] = lo;
            gap[a][0][0] = hi;
            gap[a][0][1] = hi + half;
            gap[a][1][0] = fmaxf(lo - half, 0.f);  // the voxel's own slab: the other half
            gap[a][1][1] = fmaxf(hi - half, 0.f);
        }
    }
    // f32 evaluation: the cell corners and gaps carry at most a few ulps of far * res, well
    // inside the 1e-6 far * res widening
    const float lim = res * (1.f + 1e-5f) + 1e-6f * far * res;
    const float lim2 = lim * lim;
    const uint32_t E1 = m.ext[1] + 2u, E2 = m.ext[2] + 2u;
    if constexpr (!OCT) {  // one mask per cell (m.msh = 0): a rolled loop over the 27 neighbours
#pragma unroll 1
        for (uint32_t b = 0; b < 27u; ++b) {
            const uint32_t dx = b / 9u, dy = b / 3u % 3u, dz = b % 3u;
            const float gx = dx == 2u ? gap[0][2][0] : (dx == 0u ? gap[0][0][0] : 0.f);
            const float gy = dy == 2u ? gap[1][2][0] : (dy == 0u ? gap[1][0][0] : 0.f);
            const float gz = dz == 2u ? gap[2][2][0] : (dz == 0u ? gap[2][0][0] : 0.f);
            if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) > lim2) continue;
            atomicOr(nmask + ((size_t)(v[0] + 2u - dx) * E1 + (v[1] + 2u - dy)) * E2 +
                         (v[2] + 2u - dz),
                     1u << b);
        }
    } else {
        // octant masks (m.msh = 3): every loop unrolled, so the gap table stays in registers
#pragma unroll
        for (uint32_t dx = 0; dx < 3u; ++dx)  // d + 1 per axis
#pragma unroll
            for (uint32_t dy = 0; dy < 3u; ++dy)
#pragma unroll
                for (uint32_t dz = 0; dz < 3u; ++dz) {
                    const uint32_t b = dx * 9u + dy * 3u + dz;
                    // grown-box position of cell v - d, plus one: v + 2 - (d + 1)
                    uint32_t* w = nmask + ((((size_t)(v[0] + 2u - dx) * E1 + (v[1] + 2u - dy)) *
                                                E2 +
                                            (v[2] + 2u - dz))
                                           << 3);
#pragma unroll
                    for (uint32_t o = 0; o < 8u; ++o) {
                        const float gx = gap[0][dx][(o >> 2) & 1u],
                                    gy = gap[1][dy][(o >> 1) & 1u], gz = gap[2][dz][o & 1u];
                        if (fmaf(gx, gx, fmaf(gy, gy, gz * gz)) > lim2) continue;
                        atomicOr(w + o, 1u << b);
                    }
                }
    }
}

static uint32_t bit_width(uint32_t x) {
    uint32_t b = 0;
    while (b < 32 && (x >> b)) ++b;
    return b;
}

// Key width of a cell box: bits per axis of (max - min), checked against the key limits.
static int box_bits(const int32_t* mn, const int32_t* mx, uint32_t* bits) {
    for (int a = 0; a < 3; ++a) {
        int64_t range = (int64_t)mx[a] - (int64_t)mn[a];
        if (range > 0x1FFFFF) {
            set_error("map extent exceeds 2^21 voxels along an axis");
            return NDT_ERR_RANGE;
        }
        bits[a] = std::max<uint32_t>(1, bit_width((uint32_t)range));
    }
    if (bits[0] + bits[1] + bits[2] > 31) {
        set_error("map bounding box exceeds 2^31 voxel cells (tile the map)");
        return NDT_ERR_RANGE;
    }
    return 0;
}

// Stages 1-5 of a build: cells and bounds, Morton keys, sort, segments, per-segment
// statistics. Leaves in sc: vals (point indices in key order), seg_starts, seg_rec,
// seg_valid; returns the counts and the cell box in g.
int build_segments(BuildScratch& sc, const float* d_pts, size_t n, const ndt_config& cfg,
                   cudaStream_t s, SegGeometry& g) {
    int rc = 0;
    if ((rc = dev_reserve(sc.keys_a, n * 8)) || (rc = dev_reserve(sc.vals_a, n * 4)) ||
        (rc = dev_reserve(sc.small, 256)) || (rc = dev_reserve(sc.seg_starts, n * 4 + 4)) ||
        (rc = dev_reserve(sc.seg_valid, n * 4 + 4)) || (rc = dev_reserve(sc.seg_rank, n * 4 + 4)) ||
        (rc = dev_reserve(sc.seg_rec, n * sizeof(SegRec))))
        return rc;
    size_t tmp = std::max(radix_sort_temp_bytes(n), detect_segments_temp_bytes(n));
    tmp = std::max(tmp, scan_temp_bytes(n));
    if ((rc = dev_reserve(sc.tmp, tmp))) return rc;
    uint32_t* vals = (uint32_t*)sc.vals_a.p;
    int32_t* mm = (int32_t*)sc.small.p;
    uint32_t* nseg = (uint32_t*)((char*)sc.small.p + 64);

    cell_bounds(d_pts, n, cfg.resolution, mm, s);
    int32_t hmm[7];
    cudaMemcpyAsync(hmm, mm, sizeof hmm, cudaMemcpyDeviceToHost, s);
    if ((rc = cuda_fail(cudaStreamSynchronize(s), "map bounds"))) return rc;
    g.nf = (size_t)(uint32_t)hmm[6];
    if (g.nf == 0) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    for (int a = 0; a < 3; ++a) {
        g.mn[a] = hmm[a];
        g.mx[a] = hmm[3 + a];
    }
    uint32_t bits[3];
    if ((rc = box_bits(g.mn, g.mx, bits))) return rc;
    const uint32_t lv = std::max(bits[0], std::max(bits[1], bits[2]));
    const int end_bit = std::min(64, (int)(3 * lv + 1));
    const unsigned gp = (unsigned)((n + BT - 1) / BT);
    if (end_bit <= 32) {
        // the keys fit 32 bits (the non-finite key, all ones, still sorts last)
        uint32_t* keys = (uint32_t*)sc.keys_a.p;
        k_morton<uint32_t><<<gp, BT, 0, s>>>(d_pts, n, cfg.resolution, mm, keys, vals);
        if ((rc = radix_sort_pairs32(keys, vals, n, 0, end_bit, sc.tmp.p, sc.tmp.bytes, s)) ||
            (rc = segment_starts(keys, g.nf, (uint32_t*)sc.seg_starts.p, nseg, sc.tmp.p, s)))
            return rc;
    } else {
        uint64_t* keys = (uint64_t*)sc.keys_a.p;
        k_morton<uint64_t><<<gp, BT, 0, s>>>(d_pts, n, cfg.resolution, mm, keys, vals);
        if ((rc = radix_sort_pairs(keys, vals, n, 0, end_bit, sc.tmp.p, sc.tmp.bytes, s)) ||
            (rc = segment_starts(keys, g.nf, (uint32_t*)sc.seg_starts.p, nseg, sc.tmp.p, s)))
            return rc;
    }
    cudaMemcpyAsync(&g.S, nseg, 4, cudaMemcpyDeviceToHost, s);
    if ((rc = cuda_fail(cudaStreamSynchronize(s), "segments"))) return rc;
    // visit order of the segments, largest first (the keys' buffer is free again: the
    // segments are recorded by their starts)
    uint32_t* skeys = (uint32_t*)sc.keys_a.p;
    uint32_t* order = (uint32_t*)sc.seg_rank.p;
    k_seg_size_keys<<<(g.S + 255) / 256, 256, 0, s>>>((const uint32_t*)sc.seg_starts.p, g.S,
                                                      (uint32_t)g.nf, skeys, order);
    if ((rc = radix_sort_pairs32(skeys, order, g.S, 0, 16, sc.tmp.p, sc.tmp.bytes, s))) return rc;
    // the large segments' sums into the sort's temporary storage (free again): at most
    // nf / WARP_SEG_MIN segments of SegSums, well inside its 12 bytes per point
    SegSums* sums = (SegSums*)sc.tmp.p;
    const uint32_t wmax = (uint32_t)std::min<size_t>(g.S, g.nf / WARP_SEG_MIN + 1);
    const unsigned gs = (unsigned)std::min<uint32_t>((wmax + 3) / 4, 152u * 64u);
    k_segment_sums<<<gs, 128, 0, s>>>(d_pts, vals, (uint32_t*)sc.seg_starts.p, order, skeys,
                                      g.S, (uint32_t)g.nf, cfg.resolution,
                                      cfg.min_points_per_voxel, sums);
    k_voxel_stats<<<(g.S + 127) / 128, 128, 0, s>>>(
        d_pts, vals, (uint32_t*)sc.seg_starts.p, order, skeys, sums, g.S, (uint32_t)g.nf,
        cfg.resolution, cfg.min_points_per_voxel, cfg.eigenvalue_ratio, (SegRec*)sc.seg_rec.p,
        (uint32_t*)sc.seg_valid.p);
    return cuda_fail(cudaStreamSynchronize(s), "voxel statistics");
}

// Stages 6-7: valid voxels of the S records (in Morton order of their cells) compacted into
// the map's voxel arrays, hash insert, dense cell index and neighbourhood masks.
int finish_map(Map& map, BuildScratch& sc, const SegRec* rec, const uint32_t* valid, uint32_t S,
               const SegGeometry& g, const ndt_config& cfg, uint32_t* d_status, cudaStream_t s) {
    int rc;
    if ((rc = dev_reserve(sc.seg_rank, (size_t)S * 4 + 4)) ||
        (rc = dev_reserve(sc.tmp, std::max(sc.tmp.bytes, scan_temp_bytes(S)))) ||
        (rc = dev_reserve(sc.small, 256)))
        return rc;
    uint32_t* mprobe = (uint32_t*)((char*)sc.small.p + 128);
    uint32_t* d_S = (uint32_t*)((char*)sc.small.p + 192);
    uint32_t bits[3];
    if ((rc = box_bits(g.mn, g.mx, bits))) return rc;
    if ((rc = exclusive_scan(valid, (uint32_t*)sc.seg_rank.p, S, sc.tmp.p, s))) return rc;
    uint32_t hs[2];
    cudaMemcpyAsync(&hs[0], (uint32_t*)sc.seg_rank.p + (S - 1), 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&hs[1], valid + (S - 1), 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(d_S, &S, 4, cudaMemcpyHostToDevice, s);
    if ((rc = cuda_fail(cudaStreamSynchronize(s), "voxel compaction"))) return rc;
    const uint32_t V = hs[0] + hs[1];
    if (V == 0) {
        set_error("No voxels created from target points (too sparse?)");
        return NDT_ERR_NO_VOXELS;
    }
    uint64_t factor = (uint64_t)std::max(2, cfg.hash_capacity_factor);
    uint64_t cap = 1;
    while (cap < factor * V) cap *= 2;
    if (cap > (1ull << 31)) {
        set_error("hash capacity exceeds 2^31 slots");
        return NDT_ERR_CAPACITY;
    }
    if ((rc = dev_reserve(map.vox_coord, (size_t)V * 12)) ||
        (rc = dev_reserve(map.vox_mean, (size_t)V * 16)) ||
        (rc = dev_reserve(map.vox_cov, (size_t)V * 36)) ||
        (rc = dev_reserve(map.vox_icov, (size_t)V * 36)) ||
        (rc = dev_reserve(map.vox_count, (size_t)V * 4)) ||
        (rc = dev_reserve(map.slots, cap * 16)) || (rc = dev_reserve(map.slot_icov, cap * 32)) ||
        (rc = dev_reserve(map.slot_vidx, cap * 4)))
        return rc;
    const unsigned blk = (unsigned)((S + 127) / 128);
    k_voxel_compact<<<blk, 128, 0, s>>>(rec, valid, (uint32_t*)sc.seg_rank.p, d_S,
                                        (int32_t*)map.vox_coord.p, (float4*)map.vox_mean.p,
                                        (float*)map.vox_cov.p, (float*)map.vox_icov.p,
                                        (uint32_t*)map.vox_count.p);
    cudaMemsetAsync(map.slots.p, 0xFF, cap * 16, s);
    cudaMemsetAsync(mprobe, 0, 4, s);
    MapView v{};
    v.slots = (const uint4*)map.slots.p;
    v.slot_icov = (const float4*)map.slot_icov.p;
    v.slot_vidx = (const int32_t*)map.slot_vidx.p;
    v.mask = (uint32_t)(cap - 1);
    v.max_probe = 0;
    for (int a = 0; a < 3; ++a) {
        v.min_cell[a] = g.mn[a];
        v.bits[a] = bits[a];
    }
    v.res = cfg.resolution;
    v.inv_res = 1.0f / cfg.resolution;
    v.r2 = cfg.resolution * cfg.resolution;
    v.num_voxels = V;
    {
        int ex = 0;
        float fr = frexpf(v.inv_res, &ex);
        v.exact_inv = (fr == 0.5f) ? 1 : 0;
    }
    k_hash_insert<<<(V + 127) / 128, 128, 0, s>>>(
        (int32_t*)map.vox_coord.p, (float4*)map.vox_mean.p, (float*)map.vox_icov.p, V, v,
        (uint4*)map.slots.p, (float4*)map.slot_icov.p, (int32_t*)map.slot_vidx.p, mprobe,
        d_status);
    // dense cell index over the bounding box of the map's cells, when it fits the budget
    uint64_t cells = 1;
    for (int a = 0; a < 3; ++a) {
        v.ext[a] = (uint32_t)((int64_t)g.mx[a] - (int64_t)g.mn[a] + 1);
        cells *= v.ext[a];
    }
    v.grid = nullptr;
    v.nmask = nullptr;
    v.msh = 0;
    const uint64_t mcells = (uint64_t)(v.ext[0] + 2) * (v.ext[1] + 2) * (v.ext[2] + 2);
    uint64_t mwords = 0;
    if (cfg.cell_index != NDT_CELL_INDEX_HASH && cells * 16 <= DENSE_GRID_MAX_BYTES) {
        // octant masks (eight words per cell of the grown box) while they fit their budget,
        // or (NDT_CELL_INDEX_OCTANT) while grid and masks fit the dense index's
        const bool oct = cfg.cell_index == NDT_CELL_INDEX_OCTANT
                             ? cells * 16 + mcells * 32 <= DENSE_GRID_MAX_BYTES
                             : mcells * 32 <= OCTANT_MASK_MAX_BYTES;
        v.msh = oct ? 3u : 0u;
        mwords = mcells << v.msh;
        if ((rc = dev_reserve(map.grid, (size_t)cells * 16)) ||
            (rc = dev_reserve(map.nmask, (size_t)mwords * 4)))
            return rc;
        cudaMemsetAsync(map.grid.p, 0xFF, (size_t)cells * 16, s);
        cudaMemsetAsync(map.nmask.p, 0, (size_t)mwords * 4, s);
        k_grid_fill<<<(unsigned)((cap + 255) / 256), 256, 0, s>>>(v, (float4*)map.grid.p);
        if (v.msh)
            k_grid_mask<true><<<(unsigned)((cap + 255) / 256), 256, 0, s>>>(v, (uint32_t*)map.nmask.p);
        else
            k_grid_mask<false><<<(unsigned)((cap + 255) / 256), 256, 0, s>>>(v, (uint32_t*)map.nmask.p);
        v.grid = (const float4*)map.grid.p;
        v.nmask = (const uint32_t*)map.nmask.p;
    }
    uint32_t hprobe = 0;
    cudaMemcpyAsync(&hprobe, mprobe, 4, cudaMemcpyDeviceToHost, s);
    if ((rc = cuda_fail(cudaStreamSynchronize(s), "hash insert"))) return rc;
    v.max_probe = hprobe;
    map.view = v;
    ndt_map_info& info = map.info;
    info.num_points = g.nf;
    info.num_segments = S;
    info.num_voxels = V;
    info.hash_capacity = cap;
    info.max_probe = hprobe;
    for (int a = 0; a < 3; ++a) {
        info.key_bits[a] = bits[a];
        info.min_coord[a] = g.mn[a];
        info.max_coord[a] = g.mx[a];
    }
    info.dense_grid_mib =
        v.grid ? (float)(((double)cells * 16.0 + (double)mwords * 4.0) / (1024.0 * 1024.0)) : 0.f;
    info.masks_per_cell = v.grid ? 1u << v.msh : 0u;
    info.reserved = 0u;
    map.valid = true;
    return 0;
}

// ---------------------------------------------------------------------------------------
// Map tiles: segments built once per tile, merged per commit.
// ---------------------------------------------------------------------------------------
// Keys of every tile's segments for the merged map: Morton code of the cell relative to the
// merged box's minimum cell (the key set_target of the concatenated points would give each of
// its points), value = the segment's index in tile order.
__global__ void k_merge_keys(const TileSegRef* __restrict__ tiles, int nt, uint64_t total,
                             int32_t mn0, int32_t mn1, int32_t mn2, uint64_t* __restrict__ keys,
                             uint32_t* __restrict__ vals) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    int t = 0;
    while (t + 1 < nt && i >= tiles[t + 1].seg_off) ++t;
    const int32_t* c = tiles[t].rec[i - tiles[t].seg_off].coord;
    const int32_t mn[3] = {mn0, mn1, mn2};
    uint32_t q[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int64_t d = (int64_t)c[a] - (int64_t)mn[a];
        q[a] = d > 0x1FFFFF ? 0x1FFFFFu : (uint32_t)d;
    }
    keys[i] = morton3(q[0], q[1], q[2]);
    vals[i] = (uint32_t)i;
}

// One thread per cell of the merged map (a group of equal keys: the segments of that cell in
// tile order). A cell held by one tile keeps that tile's record; a cell shared by tiles is
// recomputed from all its points in tile order, then each tile's input order, which is the
// order set_target of the concatenated tiles would visit them in.
__global__ void __launch_bounds__(128) k_merge_groups(
    const TileSegRef* __restrict__ tiles, int nt, const uint32_t* __restrict__ members,
    const uint32_t* __restrict__ gstart, const uint32_t* __restrict__ num_groups,
    uint32_t n_members, int min_points, float ratio, float res, SegRec* __restrict__ grec,
    uint32_t* __restrict__ gvalid) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t G = *num_groups;
    if (g >= G) return;
    const uint32_t m0 = gstart[g], m1 = g + 1 < G ? gstart[g + 1] : n_members;
    auto locate = [&](uint32_t id, int& t, uint32_t& sl) {
        t = 0;
        while (t + 1 < nt && id >= tiles[t + 1].seg_off) ++t;
        sl = id - (uint32_t)tiles[t].seg_off;
    };
    int t;
    uint32_t sl;
    locate(members[m0], t, sl);
    if (m1 - m0 == 1) {
        grec[g] = tiles[t].rec[sl];
        gvalid[g] = tiles[t].valid[sl];
        return;
    }
    SegRec r;
    for (int a = 0; a < 3; ++a) r.coord[a] = tiles[t].rec[sl].coord[a];
    uint32_t cnt = 0;
    for (uint32_t m = m0; m < m1; ++m) {
        locate(members[m], t, sl);
        cnt += tiles[t].rec[sl].count;
    }
    auto each = [&](auto f) {
        for (uint32_t m = m0; m < m1; ++m) {
            int tm;
            uint32_t sm;
            locate(members[m], tm, sm);
            const TileSegRef& T = tiles[tm];
            const uint32_t b = T.starts[sm], e = sm + 1 < T.S ? T.starts[sm + 1] : T.nf;
            for (uint32_t k = b; k < e; ++k) f(T.pts + 3 * (size_t)T.idx[k]);
        }
    };
    locate(members[m0], t, sl);
    const float* first = tiles[t].pts + 3 * (size_t)tiles[t].idx[tiles[t].starts[sl]];
    const bool ok = voxel_stats(each, first, cnt, min_points, ratio, res, r);
    grec[g] = r;
    gvalid[g] = ok ? 1u : 0u;
}

int merge_tiles(Map& map, BuildScratch& sc, const std::vector<TileSegRef>& refs,
                DevBuf& d_refs, const ndt_config& cfg, uint32_t* d_status, cudaStream_t s,
                float* build_ms) {
    SegGeometry g{};
    uint64_t total = 0;
    bool any = false;
    for (const auto& t : refs) {
        if (!t.S) continue;
        for (int a = 0; a < 3; ++a) {
            g.mn[a] = any ? std::min(g.mn[a], t.mn[a]) : t.mn[a];
            g.mx[a] = any ? std::max(g.mx[a], t.mx[a]) : t.mx[a];
        }
        any = true;
        g.nf += t.nf;
        total += t.S;
    }
    if (!any) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    if (total >= 0xFFFFFFF0ull) {
        set_error("too many occupied cells in the tiles");
        return NDT_ERR_CAPACITY;
    }
    uint32_t bits[3];
    int rc = box_bits(g.mn, g.mx, bits);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    std::vector<TileSegRef> used;
    for (const auto& t : refs)
        if (t.S) used.push_back(t);
    const int nt = (int)used.size();
    size_t tmp = std::max(radix_sort_temp_bytes(total), detect_segments_temp_bytes(total));
    if ((rc = dev_reserve(d_refs, used.size() * sizeof(TileSegRef))) ||
        (rc = dev_reserve(sc.keys_a, total * 8)) || (rc = dev_reserve(sc.vals_a, total * 4)) ||
        (rc = dev_reserve(sc.small, 256)) || (rc = dev_reserve(sc.seg_starts, total * 4 + 4)) ||
        (rc = dev_reserve(sc.seg_valid, total * 4 + 4)) ||
        (rc = dev_reserve(sc.seg_rec, total * sizeof(SegRec))) ||
        (rc = dev_reserve(sc.tmp, std::max(tmp, scan_temp_bytes(total)))))
        return rc;
    cudaMemcpyAsync(d_refs.p, used.data(), used.size() * sizeof(TileSegRef),
                    cudaMemcpyHostToDevice, s);
    uint64_t* keys = (uint64_t*)sc.keys_a.p;
    uint32_t* vals = (uint32_t*)sc.vals_a.p;
    uint32_t* ngroups = (uint32_t*)((char*)sc.small.p + 64);
    const TileSegRef* dref = (const TileSegRef*)d_refs.p;
    k_merge_keys<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(dref, nt, total, g.mn[0],
                                                                 g.mn[1], g.mn[2], keys, vals);
    const uint32_t lv = std::max(bits[0], std::max(bits[1], bits[2]));
    const int end_bit = std::min(64, (int)(3 * lv + 1));
    if ((rc = radix_sort_pairs(keys, vals, total, 0, end_bit, sc.tmp.p, sc.tmp.bytes, s)) ||
        (rc = detect_segments(keys, total, nullptr, (uint32_t*)sc.seg_starts.p, ngroups,
                              sc.tmp.p, sc.tmp.bytes, s)))
        return rc;
    k_merge_groups<<<(unsigned)((total + 127) / 128), 128, 0, s>>>(
        dref, nt, vals, (const uint32_t*)sc.seg_starts.p, ngroups, (uint32_t)total,
        cfg.min_points_per_voxel, cfg.eigenvalue_ratio, cfg.resolution, (SegRec*)sc.seg_rec.p,
        (uint32_t*)sc.seg_valid.p);
    cudaMemcpyAsync(&g.S, ngroups, 4, cudaMemcpyDeviceToHost, s);
    if ((rc = cuda_fail(cudaStreamSynchronize(s), "tile merge"))) return rc;
    rc = finish_map(map, sc, (const SegRec*)sc.seg_rec.p, (const uint32_t*)sc.seg_valid.p, g.S,
                    g, cfg, d_status, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (build_ms) *build_ms = ms;
    map.info.build_ms = ms;
    return 0;
}

// A tile's segments, kept with the tile: the outputs of build_segments moved into the tile's
// own buffers (point indices in key order, segment starts, records, validity).
int build_tile_segments(BuildScratch& sc, const float* d_pts, size_t n, const ndt_config& cfg,
                        cudaStream_t s, TileSegs& out, float* ms_out) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    SegGeometry g{};
    int rc = build_segments(sc, d_pts, n, cfg, s, g);
    if (rc == NDT_ERR_EMPTY_INPUT) {  // no finite point: the tile adds no cell
        out.geo = SegGeometry{};
        rc = 0;
    } else if (!rc) {
        out.geo = g;
        if ((rc = dev_reserve(out.idx, g.nf * 4)) || (rc = dev_reserve(out.starts, (size_t)g.S * 4)) ||
            (rc = dev_reserve(out.rec, (size_t)g.S * sizeof(SegRec))) ||
            (rc = dev_reserve(out.valid, (size_t)g.S * 4)))
            return rc;
        cudaMemcpyAsync(out.idx.p, sc.vals_a.p, g.nf * 4, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(out.starts.p, sc.seg_starts.p, (size_t)g.S * 4, cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(out.rec.p, sc.seg_rec.p, (size_t)g.S * sizeof(SegRec),
                        cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(out.valid.p, sc.seg_valid.p, (size_t)g.S * 4, cudaMemcpyDeviceToDevice, s);
    }
    cudaEventRecord(e1, s);
    if (!rc) rc = cuda_fail(cudaEventSynchronize(e1), "tile segments");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms_out) *ms_out = ms;
    return rc;
}

int build_map(Map& map, BuildScratch& sc, const float* d_pts, size_t n, const ndt_config& cfg,
              uint32_t* d_status, cudaStream_t s, float* build_ms) {
    if (n == 0) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    if (n >= 0xFFFFFFF0ull) {
        set_error("target point cloud exceeds 2^32 points");
        return NDT_ERR_CAPACITY;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
    SegGeometry g{};
    int rc = build_segments(sc, d_pts, n, cfg, s, g);
    if (!rc)
        rc = finish_map(map, sc, (const SegRec*)sc.seg_rec.p, (const uint32_t*)sc.seg_valid.p, g.S,
                        g, cfg, d_status, s);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (build_ms) *build_ms = ms;
    map.info.build_ms = ms;
    return 0;
}

}  // namespace ndtgb
