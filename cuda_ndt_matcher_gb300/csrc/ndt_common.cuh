// ndt_common.cuh — device-side definitions shared by the NDT kernels (sm_103a).
//
// Voxel map layout in HBM (built by voxel_build.cu, read by ndt_align.cu / ndt_score.cu):
//   slots[cap]      uint4 {key32, mean.x, mean.y, mean.z}: open-addressing hash, 16 B per
//                   slot, key32 = EMPTY_KEY when free. The stored key is the cell relative
//                   to the map's minimum cell (key_bits per axis, <= 31 bits in total); the
//                   home slot is mix32(key32) masked by the power-of-two capacity (the
//                   reference uses the MurmurHash3 64-bit finaliser of a 63-bit packed key,
//                   src/cuda_ffi/csrc/voxel_hash.cu:33-58). One 16-byte load both tests the
//                   key and yields the centroid for the radius check.
//   slot_icov[cap]  2 x float4 {c00, c01, c02, c11}, {c12, c22, 0, 0}: inverse covariance of
//                   the voxel in that slot (one 32-byte sector per accepted neighbour).
//   slot_vidx[cap]  int32 voxel index (ascending coordinate-Morton order), for the query API.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace ndtgb {

constexpr uint32_t EMPTY_KEY = 0xFFFFFFFFu;
constexpr int MAX_NB_GPU = 8;    // graph-kernel truncation (ndt_graph_common.cuh:21)
constexpr int MAX_NB_ALL = 27;   // one voxel per cell at most

// status word bits written by kernels (atomicOr), mapped to NDT_ERR_* on the host
constexpr uint32_t ST_HASH_FULL = 1u << 0;
constexpr uint32_t ST_PROBE_LIMIT = 1u << 1;
constexpr uint32_t ST_BAD_INPUT = 1u << 2;
constexpr uint32_t ST_QUEUE_STALL = 1u << 3;  // work-queue kernel found no progress for 2 s
constexpr uint32_t ST_STAGE_TIMEOUT = 1u << 4;  // a point-staging bulk copy did not land in 1 s

struct MapView {
    const uint4* slots;
    const float4* slot_icov;
    const int32_t* slot_vidx;
    uint32_t mask;        // capacity - 1
    uint32_t max_probe;   // longest insert displacement; queries scan max_probe + 1 slots
    int32_t min_cell[3];
    uint32_t bits[3];     // local key bits per axis
    float res;
    float inv_res;        // 1.0f / res, as the reference query computes it
    float r2;             // res * res (f32)
    uint32_t num_voxels;
    int32_t exact_inv;    // inv_res is a power of two (q * inv_res is exact in f32)
    // dense cell index (null when the hash serves): grid[(lx * ext[1] + ly) * ext[2] + lz]
    // = {centroid x, y, z, slot as int bits} of the voxel in local cell (lx, ly, lz), or
    // slot -1 for an empty cell
    const float4* grid;
    uint32_t ext[3];
    // neighbourhood masks over the dense index's box grown by one cell on every side, 2^msh
    // of them per cell: msh = 0, one mask per cell; msh = 3, one per octant of the cell
    // (octant o: bit 2 of o set for the upper half along x, bit 1 along y, bit 0 along z).
    // nmask[((((ux + 1) * (ext[1] + 2) + uy + 1) * (ext[2] + 2) + uz + 1) << msh) + o] has bit
    // 9 (dx + 1) + 3 (dy + 1) + (dz + 1) set when local cell (ux + dx, uy + dy, uz + dz) holds
    // a voxel whose centroid a point of that cell (octant) can accept; ascending bits are the
    // reference's 27-cell search order (dx outer, dz inner)
    const uint32_t* nmask;
    uint32_t msh;
};

// Column (ux, uy) of local cells lies inside the dense index. Local coordinates are unsigned
// (cell - min cell, wrapped), so a cell below the box reads as a huge value.
__device__ __forceinline__ bool grid_in(const MapView& m, uint32_t ux, uint32_t uy) {
    return ux < m.ext[0] && uy < m.ext[1];
}

// Occupied neighbours of cell gc (dense index only) that a point in octant `oct` of it
// (cell_oct_of_sum) can accept: the neighbourhood mask (0 when gc lies more than one cell
// outside the box), and in `corner` the dense-index position of cell
// gc - (1, 1, 1), from which nbhd_index finds each neighbour. Positions are computed modulo
// 2^32: the corner of a cell in the outer ring lies outside the box, but every neighbour
// whose bit is set lies inside it, so its position comes out exact.
__device__ __forceinline__ uint32_t nbhd_mask(const MapView& m, const int32_t* gc, uint32_t oct,
                                              uint32_t& corner) {
    const uint32_t mx = (uint32_t)gc[0] - (uint32_t)m.min_cell[0] + 1u;
    const uint32_t my = (uint32_t)gc[1] - (uint32_t)m.min_cell[1] + 1u;
    const uint32_t mz = (uint32_t)gc[2] - (uint32_t)m.min_cell[2] + 1u;
    const uint32_t E1 = m.ext[1] + 2u, E2 = m.ext[2] + 2u;
    corner = ((mx - 2u) * m.ext[1] + (my - 2u)) * m.ext[2] + (mz - 2u);
    if (mx >= m.ext[0] + 2u || my >= E1 || mz >= E2) return 0u;
    const size_t cell = ((size_t)mx * E1 + my) * E2 + mz;
    return __ldg(m.nmask + (cell << m.msh) + (oct & ((1u << m.msh) - 1u)));
}

// Dense-index position of neighbour b (bit b of the mask) of the cell whose corner is given.
__device__ __forceinline__ uint32_t nbhd_index(const MapView& m, uint32_t corner, uint32_t b) {
    return corner + (b / 9u) * (m.ext[1] * m.ext[2]) + (b / 3u % 3u) * m.ext[2] + b % 3u;
}

// The 27 offsets nbhd_index adds to the corner, by mask bit, written once per CTA to a
// 32-entry shared table (entries 27..31 zero, so any 5-bit index reads in bounds): a search
// then finds a neighbour with one shared load and an add. The caller synchronises the block
// before the table is read.
__device__ __forceinline__ void nbhd_offsets(const MapView& m, uint32_t* off32) {
    for (int b = threadIdx.x; b < 32; b += blockDim.x)
        off32[b] = b < 27 ? nbhd_index(m, 0u, (uint32_t)b) : 0u;
}

// local key of a cell, or EMPTY_KEY when the cell lies outside the map's bounding box
__device__ __forceinline__ uint32_t local_key(const MapView& m, int32_t gx, int32_t gy,
                                              int32_t gz) {
    uint32_t lx = (uint32_t)(gx - m.min_cell[0]);
    uint32_t ly = (uint32_t)(gy - m.min_cell[1]);
    uint32_t lz = (uint32_t)(gz - m.min_cell[2]);
    if ((lx >> m.bits[0]) | (ly >> m.bits[1]) | (lz >> m.bits[2])) return EMPTY_KEY;
    return lx | (ly << m.bits[0]) | (lz << (m.bits[0] + m.bits[1]));
}

// Home slot of a cell: a 32-bit avalanche mix ("lowbias32", two multiply-xorshift rounds)
// of its 31-bit local key. The reference addresses its table with the MurmurHash3 64-bit
// finaliser of a 63-bit key; which slot a voxel lands in is invisible to callers (a lookup
// returns the voxel of exactly that cell), and the 32-bit mix costs a fraction of the
// 64-bit multiplies while spreading keys as evenly (no primary clustering).
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// cell -> (local key, home slot); false when the cell lies outside the map's bounding box
__device__ __forceinline__ bool cell_slot(const MapView& m, int32_t gx, int32_t gy, int32_t gz,
                                          uint32_t& key, uint32_t& home) {
    uint32_t lx = (uint32_t)gx - (uint32_t)m.min_cell[0];
    uint32_t ly = (uint32_t)gy - (uint32_t)m.min_cell[1];
    uint32_t lz = (uint32_t)gz - (uint32_t)m.min_cell[2];
    if ((lx >> m.bits[0]) | (ly >> m.bits[1]) | (lz >> m.bits[2])) return false;
    key = lx | (ly << m.bits[0]) | (lz << (m.bits[0] + m.bits[1]));
    home = mix32(key) & m.mask;
    return true;
}

// Bounded linear probe: returns the slot holding `key` or -1. The bound max_probe + 1 is
// exact (no stored key sits further than max_probe from its home), so the loop both matches
// "probe to empty or match" and cannot spin.
__device__ __forceinline__ int32_t probe(const MapView& m, uint32_t key, uint32_t home,
                                         uint4* out) {
    uint32_t s = home;
    for (uint32_t j = 0; j <= m.max_probe; ++j) {
        uint4 v = __ldg(m.slots + s);
        if (v.x == key) {
            *out = v;
            return (int32_t)s;
        }
        if (v.x == EMPTY_KEY) return -1;
        s = (s + 1) & m.mask;
    }
    return -1;
}

// Continues a probe whose home slot held another key: slots home+1 .. home+max_probe.
__device__ __forceinline__ int32_t probe_next(const MapView& m, uint32_t key, uint32_t home,
                                              uint4* out) {
    for (uint32_t j = 1; j <= m.max_probe; ++j) {
        uint32_t s = (home + j) & m.mask;
        uint4 v = __ldg(m.slots + s);
        if (v.x == key) {
            *out = v;
            return (int32_t)s;
        }
        if (v.x == EMPTY_KEY) return -1;
    }
    return -1;
}

// Voxel of cell (gx, gy, gz): its slot (or -1) and centroid, through the dense index when
// the map has one, else through the hash.
__device__ __forceinline__ int32_t find_cell(const MapView& m, int32_t gx, int32_t gy,
                                             int32_t gz, float* cx, float* cy, float* cz) {
    if (m.grid) {
        const uint32_t ux = (uint32_t)gx - (uint32_t)m.min_cell[0];
        const uint32_t uy = (uint32_t)gy - (uint32_t)m.min_cell[1];
        const uint32_t uz = (uint32_t)gz - (uint32_t)m.min_cell[2];
        if (ux >= m.ext[0] || uy >= m.ext[1] || uz >= m.ext[2]) return -1;
        const float4 e = __ldg(m.grid + ((size_t)ux * m.ext[1] + uy) * m.ext[2] + uz);
        *cx = e.x;
        *cy = e.y;
        *cz = e.z;
        return __float_as_int(e.w);
    }
    uint32_t key, home;
    if (!cell_slot(m, gx, gy, gz, key, home)) return -1;
    uint4 sv;
    const int32_t s = probe(m, key, home, &sv);
    *cx = __uint_as_float(sv.y);
    *cy = __uint_as_float(sv.z);
    *cz = __uint_as_float(sv.w);
    return s;
}

// Cell of the unevaluated sum qh + ql (|ql| <= half an ulp of qh): floor(qh * inv_res),
// stepped down when qh * inv_res is exactly an integer and ql is negative. The correction
// is exact when inv_res is a power of two (then qh * inv_res is exact).
__device__ __forceinline__ void cell_of_sum(const MapView& m, const float* qh, const float* ql,
                                            int32_t* gc) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float f = __fmul_rn(qh[i], m.inv_res);
        float fl = floorf(f);
        if (m.exact_inv && f == fl && ql[i] < 0.f) fl -= 1.f;
        gc[i] = (int32_t)fl;
    }
}

// cell_of_sum, and the point's octant in that cell: bit 2 (x), 1 (y), 0 (z) set when the
// point lies in the upper half along that axis (f - floor(f) >= 1/2, exact in f32). A point
// within rounding of a half-cell face may land in either octant; the octant masks are widened
// by more than that rounding, so either octant's mask lists every neighbour the point accepts.
__device__ __forceinline__ uint32_t cell_oct_of_sum(const MapView& m, const float* qh,
                                                    const float* ql, int32_t* gc) {
    uint32_t oct = 0u;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float f = __fmul_rn(qh[i], m.inv_res);
        float fl = floorf(f);
        if (m.exact_inv && f == fl && ql[i] < 0.f) fl -= 1.f;
        gc[i] = (int32_t)fl;
        oct = (oct << 1) | (f - fl >= 0.5f ? 1u : 0u);
    }
    return oct;
}

// Offsets in the reference's fixed order (ndt_graph_kernels.cu:29-39): dx outer, dz inner.
__host__ __device__ __forceinline__ void offset27(int n, int& dx, int& dy, int& dz) {
    dx = n / 9 - 1;
    dy = (n / 3) % 3 - 1;
    dz = n % 3 - 1;
}

// Morton spreading (src/ndt_cuda/src/voxel_grid/gpu/morton.rs:284-305)
__host__ __device__ __forceinline__ uint64_t spread21(uint64_t v) {
    v &= 0x1FFFFFull;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}
__host__ __device__ __forceinline__ uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return (spread21(x) << 2) | (spread21(y) << 1) | spread21(z);
}

__device__ __forceinline__ float dist2_rn(float ax, float ay, float az, float bx, float by,
                                          float bz) {
    // unfused, left to right: the reference's f32 expression dx*dx + dy*dy + dz*dz
    float ex = __fsub_rn(ax, bx), ey = __fsub_rn(ay, by), ez = __fsub_rn(az, bz);
    float d = __fmul_rn(ex, ex);
    d = __fadd_rn(d, __fmul_rn(ey, ey));
    d = __fadd_rn(d, __fmul_rn(ez, ez));
    return d;
}

// f32 -> int32 with Rust `as i32` semantics (saturating, NaN -> 0)
__device__ __forceinline__ int32_t sat_i32(float v) {
    if (v != v) return 0;
    if (v >= 2147483648.0f) return INT32_MAX;
    if (v < -2147483648.0f) return INT32_MIN;
    return (int32_t)v;
}

}  // namespace ndtgb
