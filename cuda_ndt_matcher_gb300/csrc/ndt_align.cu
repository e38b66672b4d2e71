// ndt_align.cu — persistent Newton kernel for NDT alignment on sm_103a.
//
// One thread-block cluster owns one alignment for all of its iterations (graph kernels
// K1-K5 of src/cuda_ffi/csrc/ndt_graph_kernels.cu fused into one launch; many alignments
// of uneven size share the launch, one cluster each). Per iteration:
//   1. every thread transforms its points with a compensated f32 transform (R and t as
//      hi + lo f32 pairs, TwoProd/TwoSum, so x = (q_hi - mean) + q_lo keeps f32 precision of
//      x itself), finds the voxels of the 27 surrounding cells through the hash
//      (graph_hash_query_inline semantics: fixed offset order, one voxel per cell,
//      dist^2 <= res^2 in f32, at most max_nb), and aggregates per point
//        S = sum -d1 e,  G = sum w c,  M = sum w (C - d2 c c^T)    (w = d1 d2 e, c = C x)
//      (Magnusson eqs. 6.9-6.13: per-pair work is only this aggregation); the point Jacobian
//      J_k = A_k p (A_k = dR/dtheta_k, pose constant) is contracted with M and G once per
//      point into 34 FP32 accumulators: score, G, G p^T, M, M J, J^T M J. The second
//      derivative term G . (d2R/dtheta_k dtheta_l) p is recovered from G p^T at the end;
//   2. warp reduction with two-sum compensation, CTA reduction in FP64, cluster reduction in
//      FP64 over distributed shared memory (fixed order: deterministic);
//   3. rank 0 forms g and H in FP64, solves (Jacobi |lambda| pseudo-inverse of
//      jacobi_svd_6x6.cuh for the graph semantics, negative-definite clamp + SVD solve of
//      src/ndt_cuda/src/optimization/newton.rs:160-176 for the CPU semantics, with an FP64
//      Cholesky fast path when H is definite and well conditioned), applies the reference's
//      step control and convergence test, and broadcasts the next pose through DSMEM.
// Only hardware cluster barriers are used: no global-memory spin waits.
#include <cooperative_groups.h>

#include <cstdio>

#include "ndt_internal.h"

namespace cg = cooperative_groups;

namespace ndtgb {

constexpr int NACC = 34;          // f32 per-thread accumulators
constexpr int NRED = NACC + 1;    // + correspondence count
constexpr int MAX_WARPS = 16;
constexpr int NFR = 52;           // per-iteration frame: R,t hi (12), R,t lo (12), A_k (27)

// accumulator offsets: score, G[3], G p^T [3x3], M[6 sym], (M J_k)[a][k] [3x3], J^T M J [6]
constexpr int A_SC = 0, A_G = 1, A_GP = 4, A_M = 13, A_HTR = 19, A_HRR = 28;

struct SolveScratch {
    double A[36], V[36], cs[6], x[6];
    int ok, path;  // path: 0 Cholesky, 1 eigen
};

struct AlignShared {
    SolveScratch solve;
    unsigned long long cyc[4];  // rank 0: points+CTA reduce, cluster wait, control, broadcast
    int n_eigen;
    double warp_part[MAX_WARPS][NRED];
    double part[NRED];
    double tot[NRED];
    double pose[6];
    double H[36];
    double g[6];
    float fr[NFR];
    int done;
    // rank-0 controller state
    double best_pose[6];
    double best_score;
    double last_H[36];
    double prev[3], prev2[3];
    int last_corr;
    int osc, max_osc;
};

__device__ __forceinline__ int sym3(int a, int b) {
    // (0,0)->0 (0,1)->1 (0,2)->2 (1,1)->3 (1,2)->4 (2,2)->5
    int i = a < b ? a : b, j = a < b ? b : a;
    return i == 0 ? j : (i == 1 ? 2 + j : 5);
}

// Angular derivative matrices (src/ndt_cuda/src/derivatives/angular.rs:37-189):
// A[k] = dR/d(theta_k) for roll, pitch, yaw; B[kl] = d2R/d(theta_k)d(theta_l) for
// kl = rr, rp, ry, pp, py, yy. `small` applies the CPU path's |angle| < 1e-5 rule.
__device__ void angular_mats(const double* pose, bool small, double A[3][9], double B[6][9]) {
    double sx, cx, sy, cy, sz, cz;
    sincos(pose[3], &sx, &cx);
    sincos(pose[4], &sy, &cy);
    sincos(pose[5], &sz, &cz);
    if (small) {
        if (fabs(pose[3]) < 1e-5) sx = 0.0, cx = 1.0;
        if (fabs(pose[4]) < 1e-5) sy = 0.0, cy = 1.0;
        if (fabs(pose[5]) < 1e-5) sz = 0.0, cz = 1.0;
    }
    const double j[8][3] = {
        {-sx * sz + cx * sy * cz, -sx * cz - cx * sy * sz, -cx * cy},
        {cx * sz + sx * sy * cz, cx * cz - sx * sy * sz, -sx * cy},
        {-sy * cz, sy * sz, cy},
        {sx * cy * cz, -sx * cy * sz, sx * sy},
        {-cx * cy * cz, cx * cy * sz, -cx * sy},
        {-cy * sz, -cy * cz, 0.0},
        {cx * cz - sx * sy * sz, -cx * sz - sx * sy * cz, 0.0},
        {sx * cz + cx * sy * sz, cx * sy * cz - sx * sz, 0.0},
    };
    const double h[15][3] = {
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
    for (int q = 0; q < 9; ++q) {
        A[0][q] = 0.0;
        for (int k = 0; k < 6; ++k) B[k][q] = 0.0;
    }
    for (int c = 0; c < 3; ++c) {
        A[0][3 + c] = j[0][c];
        A[0][6 + c] = j[1][c];
        A[1][c] = j[2][c];
        A[1][3 + c] = j[3][c];
        A[1][6 + c] = j[4][c];
        A[2][c] = j[5][c];
        A[2][3 + c] = j[6][c];
        A[2][6 + c] = j[7][c];
        B[0][3 + c] = h[0][c];   // roll-roll   a = [0, a2, a3]
        B[0][6 + c] = h[1][c];
        B[1][3 + c] = h[2][c];   // roll-pitch  b
        B[1][6 + c] = h[3][c];
        B[2][3 + c] = h[4][c];   // roll-yaw    c
        B[2][6 + c] = h[5][c];
        B[3][c] = h[6][c];       // pitch-pitch d
        B[3][3 + c] = h[7][c];
        B[3][6 + c] = h[8][c];
        B[4][c] = h[9][c];       // pitch-yaw   e
        B[4][3 + c] = h[10][c];
        B[4][6 + c] = h[11][c];
        B[5][c] = h[12][c];      // yaw-yaw     f
        B[5][3 + c] = h[13][c];
        B[5][6 + c] = h[14][c];
    }
}

// Per-iteration frame for the per-point work: R = Rx(roll) Ry(pitch) Rz(yaw) and t as
// hi/lo f32 pairs (hi = fl(v), lo = fl(v - hi)), and the angular Jacobian matrices A_k in f32.
__device__ __noinline__ void make_frame(const double* pose, bool small, float* fr) {
    double sr, cr, sp, cp, sy, cy;
    sincos(pose[3], &sr, &cr);
    sincos(pose[4], &sp, &cp);
    sincos(pose[5], &sy, &cy);
    double v[12] = {cp * cy, -cp * sy, sp,
                    sr * sp * cy + cr * sy, cr * cy - sr * sp * sy, -sr * cp,
                    sr * sy - cr * sp * cy, cr * sp * sy + sr * cy, cr * cp,
                    pose[0], pose[1], pose[2]};
    for (int i = 0; i < 12; ++i) {
        float h = (float)v[i];
        fr[i] = h;
        fr[12 + i] = (float)(v[i] - (double)h);
    }
    double A[3][9], B[6][9];
    angular_mats(pose, small, A, B);
    for (int k = 0; k < 3; ++k)
        for (int q = 0; q < 9; ++q) fr[24 + 9 * k + q] = (float)A[k][q];
}

// ------------------------------------------------------------------------------------
// 6x6 solvers (FP64)
// ------------------------------------------------------------------------------------
// Round-robin schedule of the 15 index pairs of a 6x6 matrix in 5 rounds of 3 disjoint
// pairs (circle method), so the three rotations of a round commute and run in parallel.
__constant__ int8_t RR_PAIRS[5][3][2] = {
    {{0, 1}, {2, 5}, {3, 4}}, {{0, 2}, {1, 3}, {4, 5}}, {{0, 3}, {2, 4}, {1, 5}},
    {{0, 4}, {3, 5}, {1, 2}}, {{0, 5}, {1, 4}, {2, 3}}};

// Warp-parallel Jacobi eigen-decomposition of the symmetric 6x6 in `A` (FP64, shared memory):
// A becomes diagonal, V accumulates the rotations. Rotation angles and stopping rules follow
// the reference's jacobi_svd_6x6.cuh:135-210 (tau formula, skip |a_pq| < 1e-15, stop when
// 2 sum(offdiag^2) < 1e-28 sum(diag^2), <= 30 sweeps); the sweep order is parallel
// round-robin instead of cyclic-by-row, which changes results only by FP64 rounding. Every
// FP64 instruction does the work of up to 32 lanes (the FP64 pipe is narrow on this GPU).
__device__ __noinline__ int jacobi6_warp(double* A, double* V, double* cs, int lane) {
    if (lane < 36 - 32) V[32 + lane] = ((32 + lane) % 7 == 0) ? 1.0 : 0.0;
    V[lane] = (lane % 7 == 0) ? 1.0 : 0.0;
    __syncwarp();
    int sweeps = 0;
    for (int sweep = 0; sweep < 30; ++sweep) {
        // convergence test (lane i < 6 owns diagonal i; lanes < 15 own one off-diagonal pair)
        double dg = lane < 6 ? A[lane * 7] * A[lane * 7] : 0.0;
        double off = 0.0;
        if (lane < 15) {
            int p = RR_PAIRS[lane / 3][lane % 3][0], q = RR_PAIRS[lane / 3][lane % 3][1];
            off = A[p * 6 + q] * A[p * 6 + q];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dg += __shfl_xor_sync(0xffffffffu, dg, o);
            off += __shfl_xor_sync(0xffffffffu, off, o);
        }
        if (2.0 * off < 1e-28 * dg) break;
        sweeps++;
        for (int r = 0; r < 5; ++r) {
            if (lane < 3) {
                int p = RR_PAIRS[r][lane][0], q = RR_PAIRS[r][lane][1];
                double apq = A[p * 6 + q];
                double c = 1.0, sn = 0.0;
                if (fabs(apq) >= 1e-15) {
                    double tau = (A[q * 6 + q] - A[p * 6 + p]) / (2.0 * apq);
                    double t = tau >= 0.0 ? 1.0 / (tau + sqrt(tau * tau + 1.0))
                                          : -1.0 / (-tau + sqrt(tau * tau + 1.0));
                    c = 1.0 / sqrt(t * t + 1.0);
                    sn = t * c;
                }
                cs[2 * lane] = c;
                cs[2 * lane + 1] = sn;
            }
            __syncwarp();
            // rotation of index i: partner j and coefficients (own, partner) of row i of J^T
            // (p: c, -s; q: s, c)
            double nA0 = 0.0, nV0 = 0.0, nV1 = 0.0;
            int ai = 0, aj = 0;
            if (lane < 21) {  // upper-triangle entry (ai <= aj)
                int t = lane;
                ai = 0;
                while (t >= 6 - ai) {
                    t -= 6 - ai;
                    ++ai;
                }
                aj = ai + t;
            }
            auto coef = [&](int i, int& partner, double& cown, double& cpart) {
                for (int k = 0; k < 3; ++k) {
                    int p = RR_PAIRS[r][k][0], q = RR_PAIRS[r][k][1];
                    if (i == p) {
                        partner = q;
                        cown = cs[2 * k];
                        cpart = -cs[2 * k + 1];
                    } else if (i == q) {
                        partner = p;
                        cown = cs[2 * k];
                        cpart = cs[2 * k + 1];
                    }
                }
            };
            if (lane < 21) {
                int pi, pj;
                double ci, si, cj, sj;
                coef(ai, pi, ci, si);
                coef(aj, pj, cj, sj);
                if (pi == aj) {  // rotated pair itself: zeroed by construction
                    nA0 = 0.0;
                } else {
                    double a_ij = A[ai * 6 + aj], a_ipj = A[pi * 6 + aj];
                    double a_ijp = A[ai * 6 + pj], a_ipjp = A[pi * 6 + pj];
                    nA0 = ci * (cj * a_ij + sj * a_ijp) + si * (cj * a_ipj + sj * a_ipjp);
                }
            }
            // V' = V J: column j mixes with its partner
            {
                int vi = lane / 6, vj = lane % 6, pj;
                double cj, sj;
                coef(vj, pj, cj, sj);
                nV0 = cj * V[vi * 6 + vj] + sj * V[vi * 6 + pj];
                if (lane < 4) {
                    int e = 32 + lane;
                    int wi = e / 6, wj = e % 6, pw;
                    double cw, sw;
                    coef(wj, pw, cw, sw);
                    nV1 = cw * V[wi * 6 + wj] + sw * V[wi * 6 + pw];
                }
            }
            __syncwarp();
            if (lane < 21) {
                A[ai * 6 + aj] = nA0;
                A[aj * 6 + ai] = nA0;
            }
            V[lane] = nV0;
            if (lane < 4) V[32 + lane] = nV1;
            __syncwarp();
        }
    }
    return sweeps;
}

// Cholesky of a symmetric matrix (one lane); false if a pivot is not positive or the pivot
// ratio falls below 1e-6 (then the caller takes the eigen path).
__device__ __noinline__ bool chol6(const double* M, double* L) {
    double dmin = 1e300, dmax = 0.0;
    for (int i = 0; i < 6; ++i) {
        for (int j = 0; j <= i; ++j) {
            double s = M[i * 6 + j];
            for (int k = 0; k < j; ++k) s -= L[i * 6 + k] * L[j * 6 + k];
            if (i == j) {
                if (!(s > 0.0)) return false;
                dmin = fmin(dmin, s);
                dmax = fmax(dmax, s);
                L[i * 6 + i] = sqrt(s);
            } else {
                L[i * 6 + j] = s / L[j * 6 + j];
            }
        }
    }
    return dmin > 1e-6 * dmax;
}

__device__ void chol6_solve(const double* L, const double* b, double* x) {
    double y[6];
    for (int i = 0; i < 6; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[i * 6 + k] * y[k];
        y[i] = s / L[i * 6 + i];
    }
    for (int i = 5; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < 6; ++k) s -= L[k * 6 + i] * x[k];
        x[i] = s / L[i * 6 + i];
    }
}

// Newton step for both semantics; all 32 lanes of one warp call it, result in S.x / S.ok.
//  graph (K3): x = V diag(1/|lambda|) V^T (-g), |lambda| > max(1e-10 max|lambda|, 1e-15)
//              (jacobi_svd_solve_6x6_f64); definite H: x = (sH)^-1 (-g), s = sign
//  cpu       : newton_step_negative_definite(g, H, -1e-3, 1e-10) (newton.rs:160-176)
template <bool CPU_SEM>
__device__ __noinline__ void solve_warp(const double* H, const double* g, SolveScratch& S,
                                        int lane) {
    if (lane == 0) {
        double M[36], L[36];
        S.ok = 0;
        S.path = 1;
        for (int sgn = 1; sgn >= -1; sgn -= 2) {
            if (CPU_SEM && sgn == 1) continue;  // only the negative-definite fast path
            for (int i = 0; i < 36; ++i) M[i] = sgn * H[i];
            if (chol6(M, L)) {
                double b[6];
                for (int i = 0; i < 6; ++i) b[i] = CPU_SEM ? g[i] : -g[i];
                chol6_solve(L, b, S.x);
                S.ok = 1;
                S.path = 0;
                break;
            }
        }
    }
    __syncwarp();
    if (S.path == 0) return;
    S.A[lane] = H[lane];
    if (lane < 4) S.A[32 + lane] = H[32 + lane];
    __syncwarp();
    jacobi6_warp(S.A, S.V, S.cs, lane);
    if (lane == 0) {
        double lam[6];
        for (int i = 0; i < 6; ++i) lam[i] = S.A[i * 7];
        double thr;
        bool use_abs;
        if (!CPU_SEM) {
            double mx = 0.0;
            for (int i = 0; i < 6; ++i) mx = fmax(mx, fabs(lam[i]));
            thr = fmax(1e-10 * mx, 1e-15);
            use_abs = true;
        } else {
            bool nd = true;
            for (int i = 0; i < 6; ++i)
                if (!(lam[i] < 0.0)) nd = false;
            if (!nd)
                for (int i = 0; i < 6; ++i)
                    if (lam[i] > -1e-3) lam[i] = -1e-3;
            double mx = 0.0;
            for (int i = 0; i < 6; ++i) mx = fmax(mx, fabs(lam[i]));
            thr = 1e-10;
            use_abs = false;
            if (mx < 1e-10) {
                S.ok = 0;
                return;
            }
        }
        double z[6];
        int nz = 0;
        for (int i = 0; i < 6; ++i) {
            double y = 0.0;
            for (int j = 0; j < 6; ++j) y += S.V[j * 6 + i] * (-g[j]);
            double al = fabs(lam[i]);
            if (al > thr) {
                z[i] = y / (use_abs ? al : lam[i]);
                nz++;
            } else {
                z[i] = 0.0;
            }
        }
        for (int i = 0; i < 6; ++i) {
            double s = 0.0;
            for (int j = 0; j < 6; ++j) s += S.V[i * 6 + j] * z[j];
            S.x[i] = s;
        }
        S.ok = CPU_SEM ? 1 : (nz > 0);
    }
    __syncwarp();
}

// ------------------------------------------------------------------------------------
// Per-point work
// ------------------------------------------------------------------------------------
template <bool CPU_SEM>
__device__ __forceinline__ void point_terms(const MapView& m, float px, float py, float pz,
                                            const float* fr, int max_nb, float d1f, float d2f,
                                            float* acc, int& ncorr, uint32_t* nbl,
                                            int nbl_stride) {
    const float pv[3] = {px, py, pz};
    float qh[3], ql[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        float hi = fr[9 + i], lo = fr[21 + i];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float r = fr[3 * i + j];
            float ph = r * pv[j];
            float pl = fmaf(r, pv[j], -ph);      // exact product error
            float s = hi + ph;                   // TwoSum(hi, ph)
            float bb = s - hi;
            float e = (hi - (s - bb)) + (ph - bb);
            hi = s;
            lo += e + pl + fr[12 + 3 * i + j] * pv[j];
        }
        float s = hi + lo;                       // FastTwoSum renormalisation
        ql[i] = lo - (s - hi);
        qh[i] = s;
    }
    int32_t gc[3];
    cell_of_sum(m, qh, ql, gc);
    // ---- search: the 27 cells in the reference's order (dx outer, dy, dz inner); the slots
    // of the accepted voxels (centroid within one resolution, at most max_nb) are listed in
    // shared memory, so the search runs with all lanes busy and the pair work below runs once
    // per listed voxel rather than once per cell
    int cnt = 0;
    const uint32_t bxy = m.bits[0] + m.bits[1];
    const uint32_t lz0 = (uint32_t)(gc[2] - m.min_cell[2]);
#pragma unroll 1
    for (int c9 = 0; c9 < 9; ++c9) {
        if (cnt >= max_nb) break;
        const int dx = c9 / 3 - 1, dy = c9 % 3 - 1;
        const uint32_t lx = (uint32_t)(gc[0] + dx - m.min_cell[0]);
        const uint32_t ly = (uint32_t)(gc[1] + dy - m.min_cell[1]);
        if ((lx >> m.bits[0]) | (ly >> m.bits[1])) continue;
        const uint32_t kxy = lx | (ly << m.bits[0]);
        uint4 sv[3];
        uint32_t key[3], home[3];
        bool inb[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {  // the column's three home slots, loaded together
            const uint32_t lz = lz0 + (uint32_t)(k - 1);
            inb[k] = (lz >> m.bits[2]) == 0u;
            key[k] = kxy | (lz << bxy);
            home[k] = mix32(key[k]) & m.mask;
            sv[k] = inb[k] ? __ldg(m.slots + home[k]) : make_uint4(EMPTY_KEY, 0u, 0u, 0u);
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (cnt >= max_nb) break;
            if (!inb[k]) continue;
            uint4 v = sv[k];
            int32_t s = (int32_t)home[k];
            if (v.x != key[k]) {
                if (v.x == EMPTY_KEY) continue;
                s = probe_next(m, key[k], home[k], &v);
                if (s < 0) continue;
            }
            const float e0 = (qh[0] - __uint_as_float(v.y)) + ql[0];
            const float e1 = (qh[1] - __uint_as_float(v.z)) + ql[1];
            const float e2 = (qh[2] - __uint_as_float(v.w)) + ql[2];
            if (fmaf(e0, e0, fmaf(e1, e1, e2 * e2)) > m.r2) continue;
            nbl[cnt * nbl_stride] = (uint32_t)s;
            cnt++;
        }
    }
    if (cnt == 0) return;
    // ---- pairs: S, G, M aggregated over the listed voxels
    float S = 0.f, G0 = 0.f, G1 = 0.f, G2 = 0.f;
    float M0 = 0.f, M1 = 0.f, M2 = 0.f, M3 = 0.f, M4 = 0.f, M5 = 0.f;
    const float d1d2 = d1f * d2f;
#pragma unroll 1
    for (int j = 0; j < cnt; ++j) {
        const uint32_t s = nbl[j * nbl_stride];
        const uint4 v = __ldg(m.slots + s);
        const float4 ca = __ldg(m.slot_icov + 2 * (size_t)s);
        const float4 cb = __ldg(m.slot_icov + 2 * (size_t)s + 1);
        const float x0 = (qh[0] - __uint_as_float(v.y)) + ql[0];
        const float x1 = (qh[1] - __uint_as_float(v.z)) + ql[1];
        const float x2 = (qh[2] - __uint_as_float(v.w)) + ql[2];
        // C = [[ca.x ca.y ca.z] [ca.y ca.w cb.x] [ca.z cb.x cb.y]]
        const float c0 = fmaf(ca.x, x0, fmaf(ca.y, x1, ca.z * x2));
        const float c1 = fmaf(ca.y, x0, fmaf(ca.w, x1, cb.x * x2));
        const float c2 = fmaf(ca.z, x0, fmaf(cb.x, x1, cb.y * x2));
        const float sq = fmaf(x0, c0, fmaf(x1, c1, x2 * c2));
        const float e = expf(-0.5f * d2f * sq);
        if (CPU_SEM) {
            const float wn = d2f * e;  // compute_derivative_single: zero unless d2*e in [0,1]
            if (!(wn >= 0.f && wn <= 1.f)) continue;
        }
        const float w = d1d2 * e;
        const float wd = w * d2f;
        S = fmaf(-d1f, e, S);
        G0 = fmaf(w, c0, G0);
        G1 = fmaf(w, c1, G1);
        G2 = fmaf(w, c2, G2);
        M0 += fmaf(w, ca.x, -wd * c0 * c0);
        M1 += fmaf(w, ca.y, -wd * c0 * c1);
        M2 += fmaf(w, ca.z, -wd * c0 * c2);
        M3 += fmaf(w, ca.w, -wd * c1 * c1);
        M4 += fmaf(w, cb.x, -wd * c1 * c2);
        M5 += fmaf(w, cb.y, -wd * c2 * c2);
    }
    if (cnt == 0) return;
    ncorr += cnt;
    const float G[3] = {G0, G1, G2};
    const float Ms[3][3] = {{M0, M1, M2}, {M1, M3, M4}, {M2, M4, M5}};
    acc[A_SC] += S;
    // J_k = A_k p, MJ_k = M J_k
    float J[3][3], MJ[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a)
            J[k][a] = fmaf(fr[24 + 9 * k + 3 * a], pv[0],
                           fmaf(fr[25 + 9 * k + 3 * a], pv[1], fr[26 + 9 * k + 3 * a] * pv[2]));
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int a = 0; a < 3; ++a)
            MJ[k][a] = fmaf(Ms[a][0], J[k][0], fmaf(Ms[a][1], J[k][1], Ms[a][2] * J[k][2]));
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        acc[A_G + a] += G[a];
#pragma unroll
        for (int b = 0; b < 3; ++b) acc[A_GP + 3 * a + b] = fmaf(G[a], pv[b], acc[A_GP + 3 * a + b]);
#pragma unroll
        for (int k = 0; k < 3; ++k) acc[A_HTR + 3 * a + k] += MJ[k][a];
    }
    acc[A_M + 0] += M0;
    acc[A_M + 1] += M1;
    acc[A_M + 2] += M2;
    acc[A_M + 3] += M3;
    acc[A_M + 4] += M4;
    acc[A_M + 5] += M5;
    int kl = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = k; l < 3; ++l, ++kl)
            acc[A_HRR + kl] = fmaf(J[k][0], MJ[l][0],
                                   fmaf(J[k][1], MJ[l][1], fmaf(J[k][2], MJ[l][2], acc[A_HRR + kl])));
}

// g (6) and H (6x6) in FP64 from the reduced accumulators; lanes of one warp share the work.
__device__ __noinline__ void finalize_gH(const double* tot, const double* pose, bool small, double* g,
                            double* H, int lane) {
    double A[3][9], B[6][9];
    angular_mats(pose, small, A, B);
    const double* GP = tot + A_GP;
    if (lane < 6) {
        double v;
        if (lane < 3) {
            v = tot[A_G + lane];
        } else {
            v = 0.0;
            for (int q = 0; q < 9; ++q) v += A[lane - 3][q] * GP[q];
        }
        g[lane] = v;
    }
    if (lane < 21) {
        int i = 0, j = lane;
        while (j >= 6 - i) {
            j -= 6 - i;
            ++i;
        }
        j += i;
        double v;
        if (j < 3) {
            v = tot[A_M + sym3(i, j)];
        } else if (i < 3) {
            v = tot[A_HTR + 3 * i + (j - 3)];
        } else {
            int k = i - 3, l = j - 3;
            int kl = (k == 0) ? l : (k == 1 ? 2 + l : 5);  // rr rp ry pp py yy
            v = tot[A_HRR + kl];
            for (int q = 0; q < 9; ++q) v += B[kl][q] * GP[q];
        }
        H[i * 6 + j] = v;
        H[j * 6 + i] = v;
    }
}

__device__ __forceinline__ void osc_update(AlignShared& sh, const double* pose, int it) {
    if (it >= 1) {
        double cv[3], pv[3];
        for (int a = 0; a < 3; ++a) {
            cv[a] = pose[a] - sh.prev[a];
            pv[a] = sh.prev[a] - sh.prev2[a];
        }
        double cn = sqrt(cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2]);
        double pn = sqrt(pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2]);
        if (cn > 1e-10 && pn > 1e-10) {
            double cosv = (cv[0] * pv[0] + cv[1] * pv[1] + cv[2] * pv[2]) / (cn * pn);
            sh.osc = cosv < -0.9 ? sh.osc + 1 : 0;
            if (sh.osc > sh.max_osc) sh.max_osc = sh.osc;
        } else {
            sh.osc = 0;
        }
    }
    for (int a = 0; a < 3; ++a) {
        sh.prev2[a] = sh.prev[a];
        sh.prev[a] = pose[a];
    }
}

__device__ void write_out(AlignOut& o, const double* pose, double score, const double* H,
                          int iters, int conv, int ncorr, int osc, int status) {
    for (int i = 0; i < 6; ++i) o.pose[i] = pose[i];
    o.score = score;
    for (int i = 0; i < 36; ++i) o.hessian[i] = H ? H[i] : 0.0;
    o.iterations = iters;
    o.converged = conv;
    o.ncorr = ncorr;
    o.osc = osc;
    o.status = status;
}

// One step of the controller (rank 0, lane 0). Returns 1 when the alignment is finished.
template <bool CPU_SEM>
__device__ __noinline__ int control_step(const AlignParams& P, AlignShared& sh, const AlignJob& job,
                            AlignOut& o, int it, double score, int ncorr) {
    double* pose = sh.pose;
    const double* g = sh.g;
    const double* H = sh.H;
    if (!CPU_SEM) {
        double x[6];
        for (int i = 0; i < 6; ++i) x[i] = sh.solve.x[i];
        if (!sh.solve.ok)
            for (int i = 0; i < 6; ++i) x[i] = -g[i] * 1e-4;
        double dphi = 0.0;
        for (int i = 0; i < 6; ++i) dphi += g[i] * x[i];
        if (dphi <= 0.0)
            for (int i = 0; i < 6; ++i) x[i] = -x[i];
        double dn = 0.0;
        for (int i = 0; i < 6; ++i) dn += x[i] * x[i];
        dn = sqrt(dn);
        double step = dn > P.step_size ? P.step_size : dn;
        double scale = dn > 1e-10 ? step / dn : 0.0;
        for (int i = 0; i < 6; ++i) pose[i] += scale * x[i];
        osc_update(sh, pose, it);
        int conv = step < P.eps;
        if (conv || it + 1 >= P.max_iter) {
            int status = ncorr == 0 ? NDT_STATUS_NO_CORRESPONDENCES
                                    : (conv ? NDT_STATUS_CONVERGED : NDT_STATUS_MAX_ITERATIONS);
            write_out(o, pose, score, H, it + 1, conv && ncorr > 0, ncorr, sh.max_osc, status);
            return 1;
        }
        return 0;
    }
    // CPU semantics: NdtOptimizer::align (solver.rs:135-305)
    if (ncorr < P.min_corr) {
        if (it == 0) {
            write_out(o, job.pose, 0.0, nullptr, 0, 0, 0, 0, NDT_STATUS_NO_CORRESPONDENCES);
        } else {
            write_out(o, sh.best_pose, sh.best_score, sh.last_H, P.max_iter, 0, sh.last_corr,
                      sh.max_osc, NDT_STATUS_MAX_ITERATIONS);
        }
        return 1;
    }
    sh.last_corr = ncorr;
    for (int i = 0; i < 36; ++i) sh.last_H[i] = H[i];
    if (score > sh.best_score) {
        sh.best_score = score;
        for (int i = 0; i < 6; ++i) sh.best_pose[i] = pose[i];
    }
    double x[6];
    for (int i = 0; i < 6; ++i) x[i] = sh.solve.x[i];
    if (!sh.solve.ok) {
        write_out(o, sh.best_pose, sh.best_score, sh.last_H, it, 0, sh.last_corr, sh.max_osc,
                  NDT_STATUS_SINGULAR_HESSIAN);
        return 1;
    }
    double dn = 0.0;
    for (int i = 0; i < 6; ++i) dn += x[i] * x[i];
    dn = sqrt(dn);
    if (dn < P.eps) {
        write_out(o, pose, score, H, it + 1, 1, ncorr, sh.max_osc, NDT_STATUS_CONVERGED);
        return 1;
    }
    double gd = 0.0;
    for (int i = 0; i < 6; ++i) {
        x[i] /= dn;
        gd += g[i] * x[i];
    }
    if (gd <= 0.0)
        for (int i = 0; i < 6; ++i) x[i] = -x[i];
    double step = dn < P.step_size ? dn : P.step_size;
    for (int i = 0; i < 6; ++i) pose[i] += x[i] * step;
    osc_update(sh, pose, it);
    if (it + 1 >= P.max_iter) {
        write_out(o, sh.best_pose, sh.best_score, sh.last_H, P.max_iter, 0, sh.last_corr,
                  sh.max_osc, NDT_STATUS_MAX_ITERATIONS);
        return 1;
    }
    return 0;
}

// REGCAP: registers per thread the launch bounds allow (128: the default; 80: more resident
// CTAs per SM at the price of a few spills; the autotuner picks)
template <int THREADS, bool CPU_SEM, int REGCAP>
__global__ void __launch_bounds__(THREADS, 65536 / (THREADS * REGCAP))
    k_ndt_align(const AlignParams P) {
    constexpr int NW = THREADS / 32;
    __shared__ AlignShared sh;
    extern __shared__ uint32_t nbl_smem[];  // [max_nb][THREADS] accepted slots per thread
    cg::cluster_group cluster = cg::this_cluster();
    const int K = P.cluster;
    const int rank = (int)cluster.block_rank();
    const uint32_t jid = blockIdx.x / K;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (jid >= P.num_jobs) return;  // whole clusters exit together (grid = jobs * K)
    const AlignJob job = P.jobs[jid];
    const MapView& m = P.map;
    const float* pts = P.pts + 3 * job.offset;
    const uint32_t n = job.n;

    if (tid == 0) {
        for (int i = 0; i < 6; ++i) {
            sh.pose[i] = job.pose[i];
            sh.best_pose[i] = job.pose[i];
        }
        for (int a = 0; a < 3; ++a) sh.prev[a] = sh.prev2[a] = job.pose[a];
        sh.best_score = -INFINITY;
        sh.last_corr = 0;
        sh.osc = sh.max_osc = 0;
        for (int i = 0; i < 36; ++i) sh.last_H[i] = 0.0;
        sh.done = 0;
        make_frame(sh.pose, CPU_SEM, sh.fr);
    }
    __syncthreads();

    uint64_t point_iters = 0, corr_total = 0;
    if (tid == 0) {
        sh.cyc[0] = sh.cyc[1] = sh.cyc[2] = sh.cyc[3] = 0ull;
        sh.n_eigen = 0;
    }
    unsigned long long t0 = clock64();
    for (int it = 0;; ++it) {
        const float* fr = sh.fr;
        float acc[NACC];
#pragma unroll
        for (int i = 0; i < NACC; ++i) acc[i] = 0.f;
        int nc = 0;
        for (uint32_t i = (uint32_t)rank * THREADS + tid; i < n; i += (uint32_t)K * THREADS) {
            float px = __ldg(pts + 3 * (size_t)i), py = __ldg(pts + 3 * (size_t)i + 1),
                  pz = __ldg(pts + 3 * (size_t)i + 2);
            if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;
            point_terms<CPU_SEM>(m, px, py, pz, fr, P.max_nb, P.d1f, P.d2f, acc, nc,
                                 nbl_smem + tid, THREADS);
        }
        // warp: two-sum compensated butterfly, then FP64 (fully unrolled: acc[] stays in
        // registers)
#pragma unroll
        for (int k = 0; k < NACC; ++k) {
            float s = acc[k], c = 0.f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                float so = __shfl_xor_sync(0xffffffffu, s, o);
                float co = __shfl_xor_sync(0xffffffffu, c, o);
                float t = s + so;
                float bp = t - s;
                float err = (s - (t - bp)) + (so - bp);
                s = t;
                c = c + co + err;
            }
            if (lane == 0) sh.warp_part[warp][k] = (double)s + (double)c;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nc += __shfl_xor_sync(0xffffffffu, nc, o);
        if (lane == 0) sh.warp_part[warp][NACC] = (double)nc;
        __syncthreads();
        for (int k = tid; k < NRED; k += THREADS) {
            double s = 0.0;
            for (int w = 0; w < NW; ++w) s += sh.warp_part[w][k];
            sh.part[k] = s;
        }
        unsigned long long t1 = clock64();
        cluster.sync();  // partials of every CTA of the cluster are ready
        unsigned long long t2 = clock64();
        if (rank == 0) {
            for (int k = tid; k < NRED; k += THREADS) {
                double s = 0.0;
                for (int r = 0; r < K; ++r) {
                    const double* rp = cluster.map_shared_rank(sh.part, r);
                    s += rp[k];
                }
                sh.tot[k] = s;
            }
            __syncthreads();
            if (warp == 0) {
                finalize_gH(sh.tot, sh.pose, CPU_SEM, sh.g, sh.H, lane);
                __syncwarp();
                solve_warp<CPU_SEM>(sh.H, sh.g, sh.solve, lane);
                if (lane == 0) {
                    sh.n_eigen += sh.solve.path;
                    if (P.trace && it < P.max_iter) {  // per-iteration record (opt-in)
                        double* t = P.trace + ((size_t)jid * P.max_iter + it) * TRACE_REC;
                        t[0] = it;
                        t[1] = sh.tot[A_SC];
                        t[2] = sh.tot[NACC];
                        for (int i = 0; i < 6; ++i) {
                            t[3 + i] = sh.pose[i];
                            t[9 + i] = sh.g[i];
                            t[36 + i] = sh.solve.x[i];
                        }
                        int u = 0;
                        for (int i = 0; i < 6; ++i)
                            for (int j = i; j < 6; ++j) t[15 + u++] = sh.H[i * 6 + j];
                        t[42] = sh.solve.path;
                        t[43] = sh.solve.ok;
                    }
                    int ncorr = (int)sh.tot[NACC];
                    point_iters += n;
                    corr_total += (uint64_t)ncorr;
                    AlignOut& o = P.out[jid];
                    int done = control_step<CPU_SEM>(P, sh, job, o, it, sh.tot[A_SC], ncorr);
                    if (done) {
                        o.point_iters = point_iters;
                        o.corr_total = corr_total;
                    }
                    make_frame(sh.pose, CPU_SEM, sh.fr);
                    sh.done = done;
                }
                __syncwarp();
                if (lane > 0 && lane < K) {
                    AlignShared* rs = cluster.map_shared_rank(&sh, lane);
                    for (int i = 0; i < 6; ++i) rs->pose[i] = sh.pose[i];
                    for (int i = 0; i < NFR; ++i) rs->fr[i] = sh.fr[i];
                    rs->done = sh.done;
                }
            }
        }
        unsigned long long t3 = clock64();
        cluster.sync();  // next pose (or done) visible in every CTA
        unsigned long long t4 = clock64();
        if (rank == 0 && tid == 0) {
            sh.cyc[0] += t1 - t0;
            sh.cyc[1] += t2 - t1;
            sh.cyc[2] += t3 - t2;
            sh.cyc[3] += t4 - t3;
        }
        t0 = t4;
        if (sh.done) break;
    }
    if (rank == 0 && tid == 0) {
        AlignOut& o = P.out[jid];
        for (int i = 0; i < 4; ++i) o.cycles[i] = sh.cyc[i];
        o.n_eigen = sh.n_eigen;
    }
}

template <int T, bool SEM, int CAP>
static cudaError_t launch_k(cudaLaunchConfig_t& cfg, const AlignParams& p, int K) {
    cudaFuncSetAttribute(k_ndt_align<T, SEM, CAP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cfg.dynamicSmemBytes);
    if (K > 8)
        cudaFuncSetAttribute(k_ndt_align<T, SEM, CAP>,
                             cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return cudaLaunchKernelEx(&cfg, k_ndt_align<T, SEM, CAP>, p);
}

template <int T, int CAP>
static int launch_t(const AlignParams& p, int K, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.num_jobs * K, 1, 1);
    cfg.blockDim = dim3(T, 1, 1);
    cfg.dynamicSmemBytes = (size_t)T * p.max_nb * sizeof(uint32_t);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = p.semantics == NDT_SEMANTICS_CPU ? launch_k<T, true, CAP>(cfg, p, K)
                                                     : launch_k<T, false, CAP>(cfg, p, K);
    return cuda_fail(e, "ndt align launch");
}

int launch_align(const AlignParams& p, LaunchShape shape, cudaStream_t s) {
    if (p.num_jobs == 0) return 0;
    int K = shape.cluster;
    if (K < 1 || K > 16 || (K & (K - 1))) {
        set_error("cluster size must be a power of two in [1, 16]");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    AlignParams q = p;
    q.cluster = K;
    const bool dense = shape.regcap == 80;
    switch (shape.threads) {
        case 128: return dense ? launch_t<128, 80>(q, K, s) : launch_t<128, 128>(q, K, s);
        case 256: return dense ? launch_t<256, 80>(q, K, s) : launch_t<256, 128>(q, K, s);
        case 512: return launch_t<512, 128>(q, K, s);
        default:
            set_error("threads per CTA must be 128, 256 or 512");
            return NDT_ERR_INVALID_ARGUMENT;
    }
}

}  // namespace ndtgb
