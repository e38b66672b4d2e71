// ndt_score.cu — per-pose scoring and the neighbour query on sm_103a.
//
// k_score: for each (scan, pose) job, every point is transformed (compensated f32: the
// transform as hi/lo pairs, so x = q - mean keeps f32 precision), the voxels whose
// centroid lies within one resolution are found through the 27-cell hash probe (all of
// them: kiddo's `within` set, src/ndt_cuda/src/voxel_grid/search.rs:90-99), and the block
// accumulates
//   NVTL terms : max over those voxels of -d1 exp(-d2/2 x^T C x), for points with >= 1
//                voxel (compute_nvtl_simple, src/ndt_cuda/src/scoring/nvtl.rs:211-260);
//   TP terms   : the sum of the scores and the number of pairs
//                (compute_transform_probability, src/ndt_cuda/src/scoring/metrics.rs:58-121).
// The transform is either given (evaluate_*), or built from an alignment's final pose vector
// with nalgebra's from_euler_angles (Rz*Ry*Rx), the isometry the reference evaluates NVTL on
// after an alignment (src/ndt_cuda/src/optimization/types.rs:156-161, solver.rs:386,424).
// Block partials are reduced in a fixed order by a second kernel: results are deterministic.
#include "ndt_internal.h"

namespace ndtgb {

constexpr int ST = 256;          // threads per block
constexpr int SCHUNK = ST * 8;   // points per block

struct ScorePartial {
    double nvtl_sum;
    double score_sum;
    uint64_t nvtl_count;
    uint64_t ncorr;
};

// nalgebra from_euler_angles (Rz*Ry*Rx) transform in FP64
__device__ void zyx_T(const double* pose, double* T) {
    double sr, cr, sp, cp, sy, cy;
    sincos(pose[3], &sr, &cr);
    sincos(pose[4], &sp, &cp);
    sincos(pose[5], &sy, &cy);
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

// q = T p as an unevaluated sum qh + ql: T given as hi/lo f32 pairs, TwoProd/TwoSum
__device__ __forceinline__ void transform_comp(const float* Th, const float* Tl, float px,
                                               float py, float pz, float* qh, float* ql) {
    const float pv[3] = {px, py, pz};
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float hi = Th[4 * i + 3], lo = Tl[4 * i + 3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float r = Th[4 * i + j];
            float ph = r * pv[j];
            float pl = fmaf(r, pv[j], -ph);
            float s = hi + ph;
            float bb = s - hi;
            float e = (hi - (s - bb)) + (ph - bb);
            hi = s;
            lo += e + pl + Tl[4 * i + j] * pv[j];
        }
        float s = hi + lo;
        ql[i] = lo - (s - hi);
        qh[i] = s;
    }
}

__global__ void __launch_bounds__(ST) k_score(MapView m, const float* __restrict__ pts,
                                              const ScoreJob* __restrict__ jobs,
                                              const AlignOut* __restrict__ aout, float d1,
                                              float d2, ScorePartial* __restrict__ part) {
    __shared__ float Th[12], Tl[12];
    __shared__ double red[ST / 32][2];
    __shared__ unsigned long long redc[ST / 32][2];
    __shared__ uint32_t s_off[32];  // neighbour offsets of the dense index
    nbhd_offsets(m, s_off);         // read after the barrier below
    const ScoreJob job = jobs[blockIdx.y];
    const size_t pidx = (size_t)blockIdx.y * gridDim.x + blockIdx.x;
    const uint32_t first = blockIdx.x * SCHUNK;
    if (threadIdx.x == 0) {
        double T[12];
        if (job.pose_src == 1) {
            zyx_T(aout[job.out_index].pose, T);
        } else {
            for (int i = 0; i < 12; ++i) T[i] = job.T[i];
        }
        for (int i = 0; i < 12; ++i) {
            Th[i] = (float)T[i];
            Tl[i] = (float)(T[i] - (double)Th[i]);
        }
    }
    __syncthreads();
    double nv = 0.0, sc = 0.0;
    unsigned long long nvc = 0, nc = 0;
    const float* P = pts + 3 * job.offset;
    uint32_t last = min(job.n, first + SCHUNK);
    for (uint32_t i = first + threadIdx.x; i < last; i += ST) {
        float px = __ldg(P + 3 * (size_t)i), py = __ldg(P + 3 * (size_t)i + 1),
              pz = __ldg(P + 3 * (size_t)i + 2);
        if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;
        float qh[3], ql[3];
        transform_comp(Th, Tl, px, py, pz, qh, ql);
        const float qx = qh[0], qy = qh[1], qz = qh[2];
        int32_t gc[3];
        const uint32_t oct = cell_oct_of_sum(m, qh, ql, gc);
        const int32_t gx = gc[0], gy = gc[1], gz = gc[2];
        float best = -INFINITY, sum = 0.f;
        int cnt = 0;
        // one voxel with centroid (mx, my, mz) in slot s: radius test, then its score term
        auto visit = [&](int32_t s, float mx, float my, float mz) {
            const float x0 = (qx - mx) + ql[0], x1 = (qy - my) + ql[1], x2 = (qz - mz) + ql[2];
            if (fmaf(x0, x0, fmaf(x1, x1, x2 * x2)) > m.r2) return;
            const float4 ca = __ldg(m.slot_icov + 2 * (size_t)s);
            const float4 cb = __ldg(m.slot_icov + 2 * (size_t)s + 1);
            const float c0 = fmaf(ca.x, x0, fmaf(ca.y, x1, ca.z * x2));
            const float c1 = fmaf(ca.y, x0, fmaf(ca.w, x1, cb.x * x2));
            const float c2 = fmaf(ca.z, x0, fmaf(cb.x, x1, cb.y * x2));
            const float md = fmaf(x0, c0, fmaf(x1, c1, x2 * c2));
            const float s0 = -d1 * expf(-d2 * md * 0.5f);
            best = fmaxf(best, s0);
            sum += s0;
            cnt++;
        };
        if (m.grid) {  // occupied neighbours only, in the same order, from the mask
            uint32_t corner;
            uint32_t bits = nbhd_mask(m, gc, oct, corner);
#pragma unroll 1
            while (bits != 0u) {
                const uint32_t b = (uint32_t)(__ffs(bits) - 1);
                bits &= bits - 1u;
                const float4 e = __ldg(m.grid + (corner + s_off[b]));
                visit(__float_as_int(e.w), e.x, e.y, e.z);
            }
        } else {
#pragma unroll 1
            for (int c = 0; c < 27; ++c) {
                int dx, dy, dz;
                offset27(c, dx, dy, dz);
                float mx, my, mz;
                const int32_t s = find_cell(m, (int32_t)((uint32_t)gx + (uint32_t)dx),
                                            (int32_t)((uint32_t)gy + (uint32_t)dy),
                                            (int32_t)((uint32_t)gz + (uint32_t)dz), &mx, &my,
                                            &mz);
                if (s >= 0) visit(s, mx, my, mz);
            }
        }
        if (cnt) {
            nv += (double)best;
            nvc++;
            sc += (double)sum;
            nc += (unsigned long long)cnt;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        nv += __shfl_xor_sync(0xffffffffu, nv, o);
        sc += __shfl_xor_sync(0xffffffffu, sc, o);
        nvc += __shfl_xor_sync(0xffffffffu, nvc, o);
        nc += __shfl_xor_sync(0xffffffffu, nc, o);
    }
    if (lane == 0) {
        red[warp][0] = nv;
        red[warp][1] = sc;
        redc[warp][0] = nvc;
        redc[warp][1] = nc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        ScorePartial p{0.0, 0.0, 0, 0};
        for (int w = 0; w < ST / 32; ++w) {
            p.nvtl_sum += red[w][0];
            p.score_sum += red[w][1];
            p.nvtl_count += redc[w][0];
            p.ncorr += redc[w][1];
        }
        part[pidx] = p;
    }
}

__global__ void k_score_reduce(const ScorePartial* __restrict__ part, uint32_t bx,
                               uint32_t njobs, ScoreOut* __restrict__ out) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    ScoreOut o{0.0, 0.0, 0, 0};
    for (uint32_t b = 0; b < bx; ++b) {
        const ScorePartial& p = part[(size_t)j * bx + b];
        o.nvtl_sum += p.nvtl_sum;
        o.score_sum += p.score_sum;
        o.nvtl_count += p.nvtl_count;
        o.ncorr += p.ncorr;
    }
    out[j] = o;
}

int launch_score(const MapView& map, const float* pts, const ScoreJob* jobs, uint32_t num_jobs,
                  uint32_t max_n, const AlignOut* align_out, void* part, ScoreOut* out, float d1,
                  float d2, cudaStream_t s) {
    if (num_jobs == 0) return 0;
    uint32_t bx = (max_n + SCHUNK - 1) / SCHUNK;
    if (bx == 0) bx = 1;
    k_score<<<dim3(bx, num_jobs), ST, 0, s>>>(map, pts, jobs, align_out, d1, d2,
                                              (ScorePartial*)part);
    k_score_reduce<<<(num_jobs + 127) / 128, 128, 0, s>>>((ScorePartial*)part, bx, num_jobs, out);
    return cuda_fail(cudaGetLastError(), "score launch");
}

size_t score_part_bytes(uint32_t num_jobs, uint32_t max_n) {
    uint32_t bx = (max_n + SCHUNK - 1) / SCHUNK;
    if (bx == 0) bx = 1;
    return (size_t)bx * num_jobs * sizeof(ScorePartial);
}

// Standalone neighbour query with the graph kernel's semantics, f32 arithmetic unfused.
__global__ void k_query(MapView m, const float* __restrict__ q, size_t n, int max_nb,
                        int32_t* __restrict__ idx, int32_t* __restrict__ cnt) {
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float qx = q[3 * i], qy = q[3 * i + 1], qz = q[3 * i + 2];
    int32_t gx = (int32_t)floorf(__fmul_rn(qx, m.inv_res));
    int32_t gy = (int32_t)floorf(__fmul_rn(qy, m.inv_res));
    int32_t gz = (int32_t)floorf(__fmul_rn(qz, m.inv_res));
    int c = 0;
    for (int k = 0; k < 27 && c < max_nb; ++k) {
        int dx, dy, dz;
        offset27(k, dx, dy, dz);
        float mx, my, mz;
        const int32_t s = find_cell(m, (int32_t)((uint32_t)gx + (uint32_t)dx),
                                    (int32_t)((uint32_t)gy + (uint32_t)dy),
                                    (int32_t)((uint32_t)gz + (uint32_t)dz), &mx, &my, &mz);
        if (s < 0) continue;
        if (dist2_rn(qx, qy, qz, mx, my, mz) <= m.r2)
            idx[i * (size_t)max_nb + c++] = m.slot_vidx[s];
    }
    for (int k = c; k < max_nb; ++k) idx[i * (size_t)max_nb + k] = -1;
    cnt[i] = c;
}

int launch_query(const MapView& map, const float* q, size_t n, int max_nb, int32_t* idx,
                 int32_t* cnt, cudaStream_t s) {
    if (n == 0) return 0;
    k_query<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(map, q, n, max_nb, idx, cnt);
    return cuda_fail(cudaGetLastError(), "query launch");
}

}  // namespace ndtgb
