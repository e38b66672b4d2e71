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
// k_ndt_align uses only hardware cluster barriers: no global-memory spin waits. The
// work-queue variant k_ndt_queue (below) splits iterations into chunks claimed by a
// persistent grid; its only waits are bounded polls for work.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdio>
#include <map>
#include <mutex>

#include "ndt_internal.h"

namespace cg = cooperative_groups;

namespace ndtgb {

constexpr int MAX_WARPS = 16;
constexpr int NFR = 52;           // per-iteration frame: R,t hi (12), R,t lo (12), A_k (27)
// line-search candidate sums: score, G[3], G p^T [3x3], correspondence count (14 used)
constexpr int LS_VALS = 16, LS_USED = 14;

// accumulator offsets: score, G[3], G p^T [3x3], M[6 sym], (M J_k)[a][k] [3x3], J^T M J [6]
constexpr int A_SC = 0, A_G = 1, A_GP = 4, A_M = 13, A_HTR = 19, A_HRR = 28;

struct SolveScratch {
    double A[36], V[36], T[36], cs[6], x[6];
    double W[36];  // eigenvectors of the alignment's last eigen solve (warm start)
    float A32[36], V32[36], cs32[6];
    int ok, path;  // path: 0 Cholesky, 1 eigen
    int sweeps;    // FP64 Jacobi sweeps of the eigen path
    int have_w;    // W is set
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
    double trig[16];            // sin/cos of roll, pitch, yaw, 1 (exact; then small-angle rule)
    double Ad[27], Bd[54];      // dR/dtheta_k and d2R/dtheta_k dtheta_l at `pose` (FP64)
    float fr[NFR];
    int done;
    // rank-0 controller state
    double best_pose[6];
    double best_score;
    double last_H[36];
    double prev[3], prev2[3];
    int last_corr;
    int osc, max_osc;
    // line search: direction, start pose, phi(0), phi'(0), candidate step lengths, poses,
    // frames (every rank), A_k at each candidate pose, per-candidate sums. The graph path
    // scores up to 8 candidates; the CPU path's More-Thuente search one trial per round.
    double ls_delta[6], ls_orig[6], ls_phi0, ls_dphi0, ls_best, ls_best_alpha;
    int ls_more;    // the selection needs another round of candidates
    int ls_active;  // this iteration scores line-search candidates (every rank)
    // More-Thuente state (rank 0): interval ends and their values (on psi while mt_open),
    // the trial step, iterations after the first trial, the first trial pending
    double mt_al, mt_fl, mt_gl, mt_au, mt_fu, mt_gu, mt_at;
    int mt_open, mt_iter, mt_first;
    double ls_alpha[LS_MAX], ls_pose[LS_MAX][6], ls_phi[LS_MAX], ls_dphi[LS_MAX];
    double ls_Ad[LS_MAX][27], ls_trig[LS_MAX][16];
    float ls_fr[LS_MAX][NFR];
    double ls_part[LS_MAX][LS_VALS], ls_tot[LS_MAX][LS_VALS];
};

__device__ __forceinline__ int sym3(int a, int b) {
    // (0,0)->0 (0,1)->1 (0,2)->2 (1,1)->3 (1,2)->4 (2,2)->5
    int i = a < b ? a : b, j = a < b ? b : a;
    return i == 0 ? j : (i == 1 ? 2 + j : 5);
}

// Entries of R = Rx(roll) Ry(pitch) Rz(yaw), of A_k = dR/dtheta_k and of
// B_kl = d2R/dtheta_k dtheta_l (kl = rr, rp, ry, pp, py, yy) — ten row-major 3x3 matrices,
// 90 entries, in the order R, A_r, A_p, A_y, B_rr, B_rp, B_ry, B_pp, B_py, B_yy — written
// as polynomials in f = {sin r, cos r, sin p, cos p, sin y, cos y, 1}: every entry is
// c0 f[i0] f[i1] f[i2] + c1 f[j0] f[j1] f[j2] with c0, c1 in {0, +1, -1}. These are the
// entries of the reference's angular tables (src/ndt_cuda/src/derivatives/angular.rs:37-189,
// src/cuda_ffi/csrc/persistent_ndt_device.cuh:38-242): the derivatives of R, except that
// B_pp[0][2] is +sin p where d2R/dpitch2 has -sin p — the reference's point-Hessian term
// h_ang[(6, 2)] = sy (angular.rs:136-139, the PCL convention it follows), kept for parity.
// Word layout: bits 0-8 hold the three 3-bit factor indices of term 0 (6 = the constant 1),
// bits 9-17 those of term 1, bits 18-19 / 20-21 the coefficient codes of terms 0 / 1
// (0: 0, 1: +1, 2: -1).
__device__ const uint32_t FRAME_TERMS[90] = {
    0x076dabu, 0x0b6da3u, 0x076db2u, 0x150ba1u, 0x2621a9u, 0x0b6d83u,
    0x2553a0u, 0x162385u, 0x076d99u, 0x036db6u, 0x036db6u, 0x036db6u,
    0x1953a0u, 0x2a2385u, 0x0b6d99u, 0x150ba1u, 0x2621a9u, 0x0b6d83u,
    0x0b6d95u, 0x076da2u, 0x076db3u, 0x076c2bu, 0x0b6d03u, 0x076d90u,
    0x0b6d59u, 0x076d19u, 0x0b6d91u, 0x0b6da3u, 0x0b6dabu, 0x036db6u,
    0x2621a9u, 0x290ba1u, 0x036db6u, 0x162385u, 0x1953a0u, 0x036db6u,
    0x036db6u, 0x036db6u, 0x036db6u, 0x290ba1u, 0x1a21a9u, 0x076d83u,
    0x1953a0u, 0x2a2385u, 0x0b6d99u, 0x036db6u, 0x036db6u, 0x036db6u,
    0x076d59u, 0x0b6d19u, 0x076d91u, 0x076c2bu, 0x0b6d03u, 0x076d90u,
    0x036db6u, 0x036db6u, 0x036db6u, 0x2a2385u, 0x2553a0u, 0x036db6u,
    0x2621a9u, 0x290ba1u, 0x036db6u, 0x0b6dabu, 0x076da3u, 0x076db2u,
    0x0b6c85u, 0x076d10u, 0x076d83u, 0x076ca9u, 0x0b6d11u, 0x0b6d99u,
    0x076da2u, 0x076d95u, 0x036db6u, 0x0b6d03u, 0x0b6c2bu, 0x036db6u,
    0x076d19u, 0x076d59u, 0x036db6u, 0x0b6dabu, 0x076da3u, 0x036db6u,
    0x290ba1u, 0x1a21a9u, 0x036db6u, 0x1953a0u, 0x2a2385u, 0x036db6u,
};

// Per-pose frame, computed by the 32 lanes of one warp (FP64 work is spread over the lanes:
// one FP64 warp instruction costs the same with one lane active or 32). Lanes 0-2 evaluate
// sin/cos of roll, pitch, yaw; every lane then evaluates up to three of the 90 table
// entries. Outputs: the f32 frame of the point work (R and t as hi/lo pairs, A_k in f32) and
// A_k, B_kl in FP64 for assembling g and H at this pose. `small` applies the CPU path's
// |angle| < 1e-5 rule (sin = 0, cos = 1) to A_k and B_kl (angular.rs), not to R. With Bd
// null the B_kl entries are skipped (a line-search candidate needs the gradient only).
__device__ __noinline__ void make_frame_warp(const double* pose, bool small, float* fr,
                                             double* trig, double* Ad, double* Bd, int lane) {
    // each lane's term words first: their loads overlap the sines and cosines
    const int nterms = Bd ? 90 : 36;
    uint32_t words[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int e = lane + 32 * k;
        words[k] = e < nterms ? __ldg(FRAME_TERMS + e) : 0u;
    }
    if (lane < 3) {
        double s, c;
        sincos(pose[3 + lane], &s, &c);
        trig[2 * lane] = s;
        trig[2 * lane + 1] = c;
        const bool tiny = small && fabs(pose[3 + lane]) < 1e-5;
        trig[8 + 2 * lane] = tiny ? 0.0 : s;
        trig[9 + 2 * lane] = tiny ? 1.0 : c;
        const double t = pose[lane];
        const float h = (float)t;
        fr[9 + lane] = h;
        fr[21 + lane] = (float)(t - (double)h);
    }
    if (lane == 3) {
        trig[6] = 1.0;
        trig[14] = 1.0;
    }
    __syncwarp();
    // a lane's (up to) three terms are independent: unrolled, their FP64 chains overlap
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int e = lane + 32 * k;
        if (e >= nterms) break;
        const uint32_t w = words[k];
        const double* f = e < 9 ? trig : trig + 8;
        const double t0 = f[w & 7u] * f[(w >> 3) & 7u] * f[(w >> 6) & 7u];
        const double t1 = f[(w >> 9) & 7u] * f[(w >> 12) & 7u] * f[(w >> 15) & 7u];
        const uint32_t c0 = (w >> 18) & 3u, c1 = (w >> 20) & 3u;
        const double v = (c0 == 0u ? 0.0 : (c0 == 1u ? t0 : -t0)) +
                         (c1 == 0u ? 0.0 : (c1 == 1u ? t1 : -t1));
        if (e < 9) {
            const float h = (float)v;
            fr[e] = h;
            fr[12 + e] = (float)(v - (double)h);
        } else if (e < 36) {
            fr[24 + (e - 9)] = (float)v;
            Ad[e - 9] = v;
        } else {
            Bd[e - 36] = v;
        }
    }
    __syncwarp();
}

// ------------------------------------------------------------------------------------
// 6x6 solvers (FP64)
// ------------------------------------------------------------------------------------
// Round-robin schedule of the 15 index pairs of a 6x6 matrix in 5 rounds of 3 disjoint
// pairs (circle method), so the three rotations of a round commute and run in parallel.
__constant__ int8_t RR_PAIRS[5][3][2] = {
    {{0, 1}, {2, 5}, {3, 4}}, {{0, 2}, {1, 3}, {4, 5}}, {{0, 3}, {2, 4}, {1, 5}},
    {{0, 4}, {3, 5}, {1, 2}}, {{0, 5}, {1, 4}, {2, 3}}};

__device__ __forceinline__ float rsq(float v) { return rsqrtf(v); }
__device__ __forceinline__ double rsq(double v) { return rsqrt(v); }

// Role of index i in round r of the round-robin schedule: partner index (bits 0-2), slot of
// the round's rotation (bits 3-4), and bit 5 set when i is the q of its pair (p < q).
__device__ __forceinline__ int rr_role(int r, int i) {
    int role = 0;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int p = RR_PAIRS[r][k][0], q = RR_PAIRS[r][k][1];
        if (i == p) role = q | (k << 3);
        if (i == q) role = p | (k << 3) | 32;
    }
    return role;
}

// Warp-parallel Jacobi eigen-decomposition of the symmetric 6x6 in `A` (shared memory, type
// T): A becomes diagonal and V accumulates the rotations, V <- V J, from the identity or,
// when init_v is false, from the orthogonal V the caller left there. Rotation angles and
// stopping rules follow the reference's jacobi_svd_6x6.cuh:135-210 (no rotation when
// |a_pq| < skip; stop when 2 sum(offdiag^2) < stop * sum(diag^2); at most max_sweeps); the
// sweep order is parallel round-robin instead of cyclic-by-row, which changes results only
// by rounding. The tangent t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)) with
// theta = (a_qq - a_pp) / (2 a_pq) is evaluated as
// sgn(theta) |2 a_pq| / (|a_qq - a_pp| + sqrt((a_qq - a_pp)^2 + (2 a_pq)^2)) (one division),
// and c = 1 / sqrt(t^2 + 1) as a reciprocal square root. Lanes 0-20 own one upper-triangle
// entry of A, every lane one entry of V (lanes 0-3 a second); each lane's partners in the
// five rounds are resolved once, before the sweeps. Returns the sweeps that rotated.
template <typename T>
__device__ __noinline__ int jacobi6_warp(T* A, T* V, T* cs, int lane, bool init_v, T skip,
                                         T stop, int max_sweeps) {
    if (init_v) {
        if (lane < 36 - 32) V[32 + lane] = ((32 + lane) % 7 == 0) ? T(1) : T(0);
        V[lane] = (lane % 7 == 0) ? T(1) : T(0);
    }
    int ai = 0, aj = 0;  // upper-triangle entry (ai <= aj) of lanes < 21
    if (lane < 21) {
        int t = lane;
        while (t >= 6 - ai) {
            t -= 6 - ai;
            ++ai;
        }
        aj = ai + t;
    }
    const int vi = lane / 6, vj = lane % 6, wi = (32 + lane) / 6, wj = (32 + lane) % 6;
    int ra[5], rb[5], rv[5], rw[5], rp[5], rq[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
        ra[r] = rr_role(r, ai);
        rb[r] = rr_role(r, aj);
        rv[r] = rr_role(r, vj);
        rw[r] = rr_role(r, wj);
        const int l3 = lane < 3 ? lane : 0;
        rp[r] = RR_PAIRS[r][l3][0];
        rq[r] = RR_PAIRS[r][l3][1];
    }
    int op = 0, oq = 0;  // off-diagonal pair of lanes < 15 for the convergence test
    if (lane < 15) {
        op = RR_PAIRS[lane / 3][lane % 3][0];
        oq = RR_PAIRS[lane / 3][lane % 3][1];
    }
    __syncwarp();
    int sweeps = 0;
    for (int sweep = 0; sweep < max_sweeps; ++sweep) {
        T dg = lane < 6 ? A[lane * 7] * A[lane * 7] : T(0);
        T off = lane < 15 ? A[op * 6 + oq] * A[op * 6 + oq] : T(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            dg += __shfl_xor_sync(0xffffffffu, dg, o);
            off += __shfl_xor_sync(0xffffffffu, off, o);
        }
        if (T(2) * off < stop * dg) break;
        sweeps++;
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            if (lane < 3) {
                const int p = rp[r], q = rq[r];
                const T apq = A[p * 6 + q];
                T c = T(1), sn = T(0);
                if (fabs(apq) >= skip) {
                    const T d = A[q * 6 + q] - A[p * 6 + p], a = T(2) * apq;
                    T t = fabs(a) / (fabs(d) + sqrt(d * d + a * a));
                    if (d * a < T(0)) t = -t;  // theta = d / a < 0; theta = 0 counts as +
                    c = rsq(t * t + T(1));
                    sn = t * c;
                }
                cs[2 * lane] = c;
                cs[2 * lane + 1] = sn;
            }
            __syncwarp();
            // row i of J^T: own coefficient c, partner coefficient -s (i = p) or s (i = q)
            auto own = [&](int role) { return cs[2 * ((role >> 3) & 3)]; };
            auto part = [&](int role) {
                const T s = cs[2 * ((role >> 3) & 3) + 1];
                return (role & 32) ? s : -s;
            };
            T nA = T(0), nV0, nV1 = T(0);
            if (lane < 21) {
                const int pi = ra[r] & 7, pj = rb[r] & 7;
                if (pi != aj) {  // the rotated pair itself becomes zero
                    const T ci = own(ra[r]), si = part(ra[r]);
                    const T cj = own(rb[r]), sj = part(rb[r]);
                    const T a_ij = A[ai * 6 + aj], a_ipj = A[pi * 6 + aj];
                    const T a_ijp = A[ai * 6 + pj], a_ipjp = A[pi * 6 + pj];
                    nA = ci * (cj * a_ij + sj * a_ijp) + si * (cj * a_ipj + sj * a_ipjp);
                }
            }
            {  // V' = V J: column j mixes with its partner
                const int pj = rv[r] & 7;
                nV0 = own(rv[r]) * V[vi * 6 + vj] + part(rv[r]) * V[vi * 6 + pj];
                if (lane < 4) {
                    const int pw = rw[r] & 7;
                    nV1 = own(rw[r]) * V[wi * 6 + wj] + part(rw[r]) * V[wi * 6 + pw];
                }
            }
            __syncwarp();
            if (lane < 21) {
                A[ai * 6 + aj] = nA;
                A[aj * 6 + ai] = nA;
            }
            V[lane] = nV0;
            if (lane < 4) V[32 + lane] = nV1;
            __syncwarp();
        }
    }
    return sweeps;
}

// f32 Cholesky of s*H (s = +1 or -1; H symmetric FP64) by one lane. Every index is a
// compile-time constant, so the factor stays in registers: L lower triangular, packed by
// rows, and rinv[j] = 1 / L_jj. False if a pivot is not positive or the pivot ratio falls
// below 1e-6 (the caller then takes the eigen path).
struct Chol32 {
    float L[21];
    float rinv[6];
};

__device__ __forceinline__ constexpr int tri(int i, int j) { return i * (i + 1) / 2 + j; }

__device__ __forceinline__ bool chol6f(const double* H, float sgn, Chol32& C) {
    float dmin = 3.0e38f, dmax = 0.f;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        float s = sgn * (float)H[j * 6 + j];
#pragma unroll
        for (int k = 0; k < j; ++k) s = fmaf(-C.L[tri(j, k)], C.L[tri(j, k)], s);
        if (!(s > 0.f)) return false;
        dmin = fminf(dmin, s);
        dmax = fmaxf(dmax, s);
        const float r = rsqrtf(s);
        C.rinv[j] = r;
        C.L[tri(j, j)] = s * r;
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            float t = sgn * (float)H[i * 6 + j];
#pragma unroll
            for (int k = 0; k < j; ++k) t = fmaf(-C.L[tri(i, k)], C.L[tri(j, k)], t);
            C.L[tri(i, j)] = t * r;
        }
    }
    return dmin > 1e-6f * dmax;
}

// x = (L L^T)^-1 b in f32
__device__ __forceinline__ void chol6f_solve(const Chol32& C, const float* b, float* x) {
    float y[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        float s = b[i];
#pragma unroll
        for (int k = 0; k < i; ++k) s = fmaf(-C.L[tri(i, k)], y[k], s);
        y[i] = s * C.rinv[i];
    }
#pragma unroll
    for (int i = 5; i >= 0; --i) {
        float s = y[i];
#pragma unroll
        for (int k = i + 1; k < 6; ++k) s = fmaf(-C.L[tri(k, i)], x[k], s);
        x[i] = s * C.rinv[i];
    }
}

// Z = op(X) Y for 6x6 FP64 matrices in shared memory (op(X) = X, or X^T when xt); each lane
// owns entries of Z, each a 6-term dot product split in two chains of three FMAs.
__device__ __forceinline__ void mm6(const double* X, bool xt, const double* Y, double* Z,
                                    int lane) {
    for (int e = lane; e < 36; e += 32) {
        const int i = e / 6, j = e % 6;
        double s0 = 0.0, s1 = 0.0;
#pragma unroll
        for (int k = 0; k < 6; k += 2) {
            s0 = fma(xt ? X[k * 6 + i] : X[i * 6 + k], Y[k * 6 + j], s0);
            s1 = fma(xt ? X[(k + 1) * 6 + i] : X[i * 6 + k + 1], Y[(k + 1) * 6 + j], s1);
        }
        Z[e] = s0 + s1;
    }
    __syncwarp();
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Newton step for both semantics; all 32 lanes of one warp call it, result in S.x / S.ok.
//  graph (K3): x = V diag(1/|lambda|) V^T (-g), |lambda| > max(1e-10 max|lambda|, 1e-15)
//              (jacobi_svd_solve_6x6_f64); definite H: x = (sH)^-1 (-g), s = sign
//  cpu       : newton_step_negative_definite(g, H, -1e-3, 1e-10) (newton.rs:160-176)
// Definite, well-conditioned H takes the Cholesky path (the negative-definite case, a
// maximum of the score, is tried first). Otherwise the eigen path runs Jacobi in f32 to
// convergence, makes the f32 eigenvectors orthogonal to FP64 rounding (two Newton-Schulz
// steps V <- V (3I - V^T V) / 2), and finishes with FP64 Jacobi sweeps on V^T H V under the
// reference's FP64 stopping rule: FP64 eigenpairs at a fraction of the FP64 sweeps.
template <bool CPU_SEM>
__device__ __noinline__ void solve_warp(const double* H, const double* g, SolveScratch& S,
                                        int lane) {
    // Definite fast path: f32 Cholesky factor of (s H), then mixed-precision iterative
    // refinement — the residual r = b - (s H) x in FP64 (lane i owns row i), the correction
    // solved with the f32 factor — until the last correction is below 1e-13 of x (four f32
    // solves reach FP64 accuracy while cond(H) stays below about 1e4; worse-conditioned
    // definite Hessians take the eigen path).
    Chol32 C;
    int sgn = 0;
    if (lane == 0) {
        S.ok = 0;
        S.path = 1;
        S.sweeps = 0;
        for (int s = -1; s <= 1; s += 2) {
            if (CPU_SEM && s == 1) continue;  // only the negative-definite fast path
            if (chol6f(H, (float)s, C)) {
                sgn = s;
                break;
            }
        }
    }
    sgn = __shfl_sync(0xffffffffu, sgn, 0);
    if (sgn != 0) {
        const double b = lane < 6 ? (CPU_SEM ? g[lane] : -g[lane]) : 0.0;
        double x = 0.0, r = b;
        bool conv = false;
        for (int ref = 0; ref < 4; ++ref) {
            if (lane < 6) S.cs[lane] = r;
            __syncwarp();
            if (lane == 0) {
                float rf[6], dx[6];
#pragma unroll
                for (int i = 0; i < 6; ++i) rf[i] = (float)S.cs[i];
                chol6f_solve(C, rf, dx);
#pragma unroll
                for (int i = 0; i < 6; ++i) S.T[i] = (double)dx[i];
            }
            __syncwarp();
            float adx = 0.f, ax = 0.f;
            if (lane < 6) {
                const double d = S.T[lane];
                x += d;
                S.x[lane] = x;
                adx = fabsf((float)d);
                ax = fabsf((float)x);
            }
#pragma unroll
            for (int o = 4; o > 0; o >>= 1) ax = fmaxf(ax, __shfl_xor_sync(0xffffffffu, ax, o));
            ax = __shfl_sync(0xffffffffu, ax, 0);
            conv = __all_sync(0xffffffffu, adx <= 1e-13f * ax);
            if (conv) break;
            __syncwarp();
            if (lane < 6) {
                double t = b;
                for (int j = 0; j < 6; ++j) t = fma(-(double)sgn * H[lane * 6 + j], S.x[j], t);
                r = t;
            }
        }
        if (conv) {
            if (lane == 0) {
                S.ok = 1;
                S.path = 0;
            }
            __syncwarp();
            return;
        }
    }
    __syncwarp();
    // eigen path. f32 Jacobi on W^T H W, where W holds the eigenvectors of this alignment's
    // previous eigen solve (H changes little between iterations, so few sweeps remain) or
    // the identity; then V = W V32 made orthogonal to FP64 rounding (two Newton-Schulz steps
    // V <- V (3I - V^T V) / 2) and FP64 Jacobi sweeps on V^T H V under the reference's FP64
    // stopping rule.
    const bool warm = S.have_w != 0;
    if (warm) {
        mm6(H, false, S.W, S.T, lane);    // T = H W
        mm6(S.W, true, S.T, S.A, lane);   // A = W^T H W
        S.A32[lane] = (float)S.A[lane];
        if (lane < 4) S.A32[32 + lane] = (float)S.A[32 + lane];
    } else {
        S.A32[lane] = (float)H[lane];
        if (lane < 4) S.A32[32 + lane] = (float)H[32 + lane];
    }
    __syncwarp();
    jacobi6_warp<float>(S.A32, S.V32, S.cs32, lane, true, 1e-30f, 1e-12f, 20);
    if (warm) {
        S.T[lane] = (double)S.V32[lane];
        if (lane < 4) S.T[32 + lane] = (double)S.V32[32 + lane];
        __syncwarp();
        mm6(S.W, false, S.T, S.V, lane);  // V = W V32
    } else {
        S.V[lane] = (double)S.V32[lane];
        if (lane < 4) S.V[32 + lane] = (double)S.V32[32 + lane];
        __syncwarp();
    }
    for (int ns = 0; ns < 2; ++ns) {
        mm6(S.V, true, S.V, S.T, lane);   // T = V^T V
        S.T[lane] = ((lane % 7) == 0 ? 3.0 : 0.0) - S.T[lane];
        if (lane < 4) S.T[32 + lane] = ((32 + lane) % 7 == 0 ? 3.0 : 0.0) - S.T[32 + lane];
        __syncwarp();
        mm6(S.V, false, S.T, S.A, lane);  // A = V (3I - V^T V)
        S.V[lane] = 0.5 * S.A[lane];
        if (lane < 4) S.V[32 + lane] = 0.5 * S.A[32 + lane];
        __syncwarp();
    }
    mm6(H, false, S.V, S.T, lane);        // T = H V
    mm6(S.V, true, S.T, S.A, lane);       // A = V^T H V
    {
        double v = 0.0;
        int ai = 0, aj = 0;
        if (lane < 21) {
            int t = lane;
            while (t >= 6 - ai) {
                t -= 6 - ai;
                ++ai;
            }
            aj = ai + t;
            v = 0.5 * (S.A[ai * 6 + aj] + S.A[aj * 6 + ai]);
        }
        __syncwarp();
        if (lane < 21) {
            S.A[ai * 6 + aj] = v;
            S.A[aj * 6 + ai] = v;
        }
        __syncwarp();
    }
    const int sw = jacobi6_warp<double>(S.A, S.V, S.cs, lane, false, 1e-15, 1e-28, 30);
    S.W[lane] = S.V[lane];
    if (lane < 4) S.W[32 + lane] = S.V[32 + lane];
    if (lane == 0) S.have_w = 1;
    // pseudo-inverse step from the eigenpairs, lane i < 6 owning eigenpair i
    double lam = lane < 6 ? S.A[lane * 7] : 0.0;
    double thr;
    bool use_abs;
    if (!CPU_SEM) {
        const double mx = warp_max(lane < 6 ? fabs(lam) : 0.0);
        thr = fmax(1e-10 * mx, 1e-15);
        use_abs = true;
    } else {
        const bool nd = __all_sync(0xffffffffu, lane >= 6 || lam < 0.0);
        if (!nd && lane < 6 && lam > -1e-3) lam = -1e-3;
        const double mx = warp_max(lane < 6 ? fabs(lam) : 0.0);
        thr = 1e-10;
        use_abs = false;
        if (mx < 1e-10) {
            if (lane == 0) {
                S.ok = 0;
                S.sweeps = sw;
            }
            __syncwarp();
            return;
        }
    }
    bool keep = false;
    if (lane < 6) {
        double y = 0.0;
        for (int j = 0; j < 6; ++j) y += S.V[j * 6 + lane] * (-g[j]);
        const double al = fabs(lam);
        double z = 0.0;
        if (al > thr) {
            z = y / (use_abs ? al : lam);
            keep = true;
        }
        S.cs[lane] = z;
    }
    const int nz = __popc(__ballot_sync(0xffffffffu, keep));
    __syncwarp();
    if (lane < 6) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s += S.V[lane * 6 + j] * S.cs[j];
        S.x[lane] = s;
    }
    if (lane == 0) {
        S.ok = CPU_SEM ? 1 : (nz > 0);
        S.sweeps = sw;
    }
    __syncwarp();
}

// ------------------------------------------------------------------------------------
// Per-point work
// ------------------------------------------------------------------------------------
// q = R p + t as an unevaluated sum qh + ql, from the frame's hi/lo R and t (TwoProd and
// TwoSum), so q - mean keeps f32 precision however far the map lies from the origin
__device__ __forceinline__ void transform_point(const float* fr, const float* pv, float* qh,
                                                float* ql) {
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
}

// Neighbour search of the point q = qh + ql: the 27 cells in the reference's order (dx outer,
// dy, dz inner); the slots of the accepted voxels (centroid within one resolution, at most
// max_nb) are listed in shared memory (nbl[k * nbl_stride]), so the search runs with all
// lanes busy and the pair work runs once per listed voxel rather than once per cell.
// Returns the number listed. off27: the CTA's table of neighbour offsets (nbhd_offsets).
__device__ __forceinline__ int search_point(const MapView& m, const uint32_t* off27,
                                            const float* qh, const float* ql, int max_nb,
                                            uint32_t* nbl, int nbl_stride) {
    int32_t gc[3];
    const uint32_t oct = cell_oct_of_sum(m, qh, ql, gc);
    int cnt = 0;
    if (m.grid) {
        // dense cell index: the neighbourhood mask of the point's cell (octant) names the
        // occupied cells among the 27 that it can accept, in search order; their
        // {centroid, slot} entries are loaded NB_BATCH at a time (independent loads in flight
        // together), then tested in order
        constexpr int NB_BATCH = 4;
        uint32_t corner;
        uint32_t bits = nbhd_mask(m, gc, oct, corner);
#pragma unroll 1
        while (bits != 0u && cnt < max_nb) {
            float4 e[NB_BATCH];
#pragma unroll
            for (int k = 0; k < NB_BATCH; ++k) {
                const uint32_t b = (uint32_t)(__ffs(bits) - 1) & 31u;  // 31 when empty
                e[k] = bits != 0u ? __ldg(m.grid + (corner + off27[b]))
                                  : make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
                bits &= bits - 1u;
            }
#pragma unroll
            for (int k = 0; k < NB_BATCH; ++k) {
                const int32_t s = __float_as_int(e[k].w);
                if (s < 0 || cnt >= max_nb) break;
                const float e0 = (qh[0] - e[k].x) + ql[0];
                const float e1 = (qh[1] - e[k].y) + ql[1];
                const float e2 = (qh[2] - e[k].z) + ql[2];
                if (fmaf(e0, e0, fmaf(e1, e1, e2 * e2)) > m.r2) continue;
                nbl[cnt * nbl_stride] = (uint32_t)s;
                cnt++;
            }
        }
    } else {
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
    }
    return cnt;
}

// Per-point terms into the accumulators: acc[0 .. A_HTR) in registers, the 15 trailing ones
// (J^T M J blocks A_HTR.., A_HRR..) in the thread's shared-memory column sacc[k * nbl_stride]
// (they change once per point; keeping them out of registers leaves the search and pair
// work room without spilling to local memory)
template <bool CPU_SEM>
__device__ __forceinline__ void point_pairs(const MapView& m, const float* pv, const float* qh,
                                            const float* ql, int cnt, const float* fr,
                                            float d1f, float d2f, float* acc, float* sacc,
                                            int& ncorr, const uint32_t* nbl, int nbl_stride);

template <bool CPU_SEM>
__device__ __forceinline__ void point_terms(const MapView& m, const uint32_t* off27,
                                            float px, float py, float pz,
                                            const float* fr, int max_nb, float d1f, float d2f,
                                            float* acc, float* sacc, int& ncorr, uint32_t* nbl,
                                            int nbl_stride) {
    const float pv[3] = {px, py, pz};
    float qh[3], ql[3];
    transform_point(fr, pv, qh, ql);
    const int cnt = search_point(m, off27, qh, ql, max_nb, nbl, nbl_stride);
    if (cnt == 0) return;
    point_pairs<CPU_SEM>(m, pv, qh, ql, cnt, fr, d1f, d2f, acc, sacc, ncorr, nbl, nbl_stride);
}

// Neighbour search of the points of a group of NPW lanes, the lanes sharing each point's
// candidates (the dense index's occupied neighbour cells): for the group's points one after
// another, lane j of the group tests the point's candidates of rank j, j + NPW, ... among
// the mask's set bits, the group ORs the accepted bits, and the point's lane lists the first
// max_nb accepted in ascending bit order (the reference's search order), so every list is
// the one search_point gives. Each lane passes its own point (bits = 0 when it has none);
// every lane of the warp takes part. Returns this lane's count.
template <int NPW>
__device__ __forceinline__ int search_group(const MapView& m, const uint32_t* off27,
                                            const float* qh, const float* ql, uint32_t bits,
                                            uint32_t corner, int max_nb, uint32_t* nbl,
                                            int nbl_stride, int lane) {
    const int g0 = lane & ~(NPW - 1), j = lane & (NPW - 1);
    int my_cnt = 0;
#pragma unroll 1
    for (int k = 0; k < NPW; ++k) {
        const int src = g0 + k;
        const uint32_t bq = __shfl_sync(0xffffffffu, bits, src);
        const uint32_t cq = __shfl_sync(0xffffffffu, corner, src);
        float h[3], l[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            h[a] = __shfl_sync(0xffffffffu, qh[a], src);
            l[a] = __shfl_sync(0xffffffffu, ql[a], src);
        }
        uint32_t rem = bq;
#pragma unroll
        for (int t = 0; t < NPW - 1; ++t)
            if (t < j) rem &= rem - 1u;  // this lane starts at the set bit of rank j
        uint32_t accm = 0u;
#pragma unroll 1
        while (rem != 0u) {
            const uint32_t b = (uint32_t)(__ffs(rem) - 1);
            const float4 e = __ldg(m.grid + (cq + off27[b]));
            const float e0 = (h[0] - e.x) + l[0];
            const float e1 = (h[1] - e.y) + l[1];
            const float e2 = (h[2] - e.z) + l[2];
            if (__float_as_int(e.w) >= 0 && !(fmaf(e0, e0, fmaf(e1, e1, e2 * e2)) > m.r2))
                accm |= 1u << b;
#pragma unroll
            for (int t = 0; t < NPW; ++t) rem &= rem - 1u;  // the next candidate of this lane
        }
#pragma unroll
        for (int o = 1; o < NPW; o <<= 1) accm |= __shfl_xor_sync(0xffffffffu, accm, o);
        if (lane == src) {
            // the point's lane lists its accepted voxels in order (slots re-read: L1 hits)
            int c = 0;
            uint32_t mm = accm;
            while (mm != 0u && c < max_nb) {
                const uint32_t b = (uint32_t)(__ffs(mm) - 1);
                nbl[c * nbl_stride] = (uint32_t)__float_as_int(
                    __ldg(reinterpret_cast<const float*>(m.grid + (cq + off27[b])) + 3));
                mm &= mm - 1u;
                ++c;
            }
            my_cnt = c;
        }
    }
    return my_cnt;
}

template <bool CPU_SEM>
__device__ __forceinline__ void point_pairs(const MapView& m, const float* pv, const float* qh,
                                            const float* ql, int cnt, const float* fr,
                                            float d1f, float d2f, float* acc, float* sacc,
                                            int& ncorr, const uint32_t* nbl, int nbl_stride) {
    // ---- pairs: S, G, M aggregated over the listed voxels
    float S = 0.f, G0 = 0.f, G1 = 0.f, G2 = 0.f;
    float M0 = 0.f, M1 = 0.f, M2 = 0.f, M3 = 0.f, M4 = 0.f, M5 = 0.f;
    const float d1d2 = d1f * d2f;
    // e = exp(-d2 sq / 2) as 2^(k2 sq) with k2 = -d2 log2(e) / 2 carried as two floats (the
    // constant -log2(e) / 2 split into two floats, then an exact product split: k2h + k2l), so the
    // argument is as accurate as the product d2 sq itself: two operations and the base-2
    // exponential per pair
    const float k2h = d2f * -0.72134751081466674805f;
    const float k2l = fmaf(d2f, -0.72134751081466674805f, -k2h) + d2f * -9.6298151675000554e-09f;
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
        const float e = exp2f(fmaf(k2h, sq, k2l * sq));
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
        // M += w C - wd c c^T, as two multiply-adds per entry
        const float u0 = wd * c0, u1 = wd * c1, u2 = wd * c2;
        M0 = fmaf(-u0, c0, fmaf(w, ca.x, M0));
        M1 = fmaf(-u0, c1, fmaf(w, ca.y, M1));
        M2 = fmaf(-u0, c2, fmaf(w, ca.z, M2));
        M3 = fmaf(-u1, c1, fmaf(w, ca.w, M3));
        M4 = fmaf(-u1, c2, fmaf(w, cb.x, M4));
        M5 = fmaf(-u2, c2, fmaf(w, cb.y, M5));
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
        for (int k = 0; k < 3; ++k) sacc[(3 * a + k) * nbl_stride] += MJ[k][a];
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
        for (int l = k; l < 3; ++l, ++kl) {
            float& h = sacc[(A_HRR - A_HTR + kl) * nbl_stride];
            h = fmaf(J[k][0], MJ[l][0], fmaf(J[k][1], MJ[l][1], fmaf(J[k][2], MJ[l][2], h)));
        }
}

// Line-search terms of one point at a candidate pose: score and gradient only, as the
// accumulators S (a[0]), G (a[1..3]) and G p^T (a[4..12]) of point_terms, same arithmetic.
// Graph semantics: the candidate pass of ndt_graph_linesearch_kernel
// (ndt_graph_kernels.cu:473-570); CPU semantics: a More-Thuente trial, the score and gradient
// of compute_derivatives_cpu_with_metric without the Hessian (solver.rs:663-673).
template <bool CPU_SEM>
__device__ __forceinline__ void point_terms_ls(const MapView& m, const uint32_t* off27,
                                               float px, float py, float pz,
                                               const float* fr, int max_nb, float d1f, float d2f,
                                               float* a, int& ncorr, uint32_t* nbl,
                                               int nbl_stride) {
    const float pv[3] = {px, py, pz};
    float qh[3], ql[3];
    transform_point(fr, pv, qh, ql);
    const int cnt = search_point(m, off27, qh, ql, max_nb, nbl, nbl_stride);
    if (cnt == 0) return;
    float S = 0.f, G[3] = {0.f, 0.f, 0.f};
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
        S = fmaf(-d1f, e, S);
        G[0] = fmaf(w, c0, G[0]);
        G[1] = fmaf(w, c1, G[1]);
        G[2] = fmaf(w, c2, G[2]);
    }
    ncorr += cnt;
    a[0] += S;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        a[1 + i] += G[i];
#pragma unroll
        for (int b = 0; b < 3; ++b) a[4 + 3 * i + b] = fmaf(G[i], pv[b], a[4 + 3 * i + b]);
    }
}

// g (6) and H (6x6) in FP64 from the reduced accumulators; lanes of one warp share the work.
// Ad / Bd: A_k and B_kl at the pose the accumulators were taken at (make_frame_warp).
__device__ __noinline__ void finalize_gH(const double* tot, const double* Ad, const double* Bd,
                                         double* g, double* H, int lane) {
    const double(*A)[9] = reinterpret_cast<const double(*)[9]>(Ad);
    const double(*B)[9] = reinterpret_cast<const double(*)[9]>(Bd);
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
        // |c| > 1e-10, |p| > 1e-10 and cos(c, p) < -0.9, compared on squares (no square roots
        // or division on the controller's FP64 path)
        const double cn2 = cv[0] * cv[0] + cv[1] * cv[1] + cv[2] * cv[2];
        const double pn2 = pv[0] * pv[0] + pv[1] * pv[1] + pv[2] * pv[2];
        if (cn2 > 1e-20 && pn2 > 1e-20) {
            const double dot = cv[0] * pv[0] + cv[1] * pv[1] + cv[2] * pv[2];
            const bool rev = dot < 0.0 && dot * dot > 0.81 * (cn2 * pn2);
            sh.osc = rev ? sh.osc + 1 : 0;
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

// 6-term FP64 dot product summed as a tree (dependency depth 4 instead of 6)
__device__ __forceinline__ double dot6(const double* a, const double* b) {
    const double p0 = fma(a[1], b[1], a[0] * b[0]);
    const double p1 = fma(a[3], b[3], a[2] * b[2]);
    const double p2 = fma(a[5], b[5], a[4] * b[4]);
    return (p0 + p1) + p2;
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
// CPU path (NdtOptimizer::align, solver.rs:135-305), first half of a Newton step: the
// correspondence check, the best score and pose, the singular and converged exits; else the
// unit ascent direction in x (reversed when g.x <= 0) and the Newton step's norm in *dn.
// Returns 1 when the alignment is finished (outputs written). Lane 0.
__device__ int cpu_direction(const AlignParams& P, AlignShared& sh, const AlignJob& job,
                             AlignOut& o, int it, double score, int ncorr, double* x,
                             double* dn_out) {
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
    for (int i = 0; i < 36; ++i) sh.last_H[i] = sh.H[i];
    if (score > sh.best_score) {
        sh.best_score = score;
        for (int i = 0; i < 6; ++i) sh.best_pose[i] = sh.pose[i];
    }
    for (int i = 0; i < 6; ++i) x[i] = sh.solve.x[i];
    if (!sh.solve.ok) {
        write_out(o, sh.best_pose, sh.best_score, sh.last_H, it, 0, sh.last_corr, sh.max_osc,
                  NDT_STATUS_SINGULAR_HESSIAN);
        return 1;
    }
    const double dn = sqrt(dot6(x, x));
    if (dn < P.eps) {
        write_out(o, sh.pose, score, sh.H, it + 1, 1, ncorr, sh.max_osc, NDT_STATUS_CONVERGED);
        return 1;
    }
    double gd = 0.0;
    for (int i = 0; i < 6; ++i) {
        x[i] /= dn;
        gd += sh.g[i] * x[i];
    }
    if (gd <= 0.0)
        for (int i = 0; i < 6; ++i) x[i] = -x[i];
    *dn_out = dn;
    return 0;
}

// CPU path, second half: pose += step x (apply_pose_delta, types.rs:183-200), the oscillation
// history, the max-iteration exit (best pose). Returns 1 when the alignment is finished.
__device__ int cpu_step(const AlignParams& P, AlignShared& sh, AlignOut& o, int it,
                        const double* x, double step) {
    for (int i = 0; i < 6; ++i) sh.pose[i] += x[i] * step;
    osc_update(sh, sh.pose, it);
    if (it + 1 >= P.max_iter) {
        write_out(o, sh.best_pose, sh.best_score, sh.last_H, P.max_iter, 0, sh.last_corr,
                  sh.max_osc, NDT_STATUS_MAX_ITERATIONS);
        return 1;
    }
    return 0;
}

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
        const double dphi = dot6(g, x);
        if (dphi <= 0.0)
            for (int i = 0; i < 6; ++i) x[i] = -x[i];
        const double dn = sqrt(dot6(x, x));
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
    double x[6], dn;
    if (cpu_direction(P, sh, job, o, it, score, ncorr, x, &dn)) return 1;
    return cpu_step(P, sh, o, it, x, dn < P.step_size ? dn : P.step_size);
}

// GPU global timer (ns): per-alignment start / finish times for latency percentiles
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// TwoSum: s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

// Warp sums of the NACC per-thread accumulators, compensated (two-sum) and written as FP64
// to out[0..NACC). Values 0..31 are reduced by recursive halving: at each exchange a lane
// sends the half of its remaining values that its partner keeps, so lane l ends holding the
// sum of value l (31 exchanges instead of 5 per value). Values 32.. use a butterfly.
__device__ __forceinline__ void warp_sum_acc(const float* acc, int lane, double* out) {
    static_assert(NACC >= 32, "recursive halving covers 32 values");
    float s[16], c[16];
    {
        const bool up = (lane & 16) != 0;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float send = up ? acc[j] : acc[j + 16];
            const float keep = up ? acc[j + 16] : acc[j];
            const float recv = __shfl_xor_sync(0xffffffffu, send, 16);
            two_sum(keep, recv, s[j], c[j]);
        }
    }
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < o; ++j) {
            const float ss = up ? s[j] : s[j + o], cs = up ? c[j] : c[j + o];
            const float sk = up ? s[j + o] : s[j], ck = up ? c[j + o] : c[j];
            const float sr = __shfl_xor_sync(0xffffffffu, ss, o);
            const float cr = __shfl_xor_sync(0xffffffffu, cs, o);
            float e;
            two_sum(sk, sr, s[j], e);
            c[j] = ck + cr + e;
        }
    }
    out[lane] = (double)s[0] + (double)c[0];
#pragma unroll
    for (int k = 32; k < NACC; ++k) {
        float v = acc[k], cv = 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float vo = __shfl_xor_sync(0xffffffffu, v, o);
            const float co = __shfl_xor_sync(0xffffffffu, cv, o);
            float e;
            two_sum(v, vo, v, e);
            cv = cv + co + e;
        }
        if (lane == 0) out[k] = (double)v + (double)cv;
    }
}

// Warp sums of the first `nv` (<= 16) of 16 f32 values, compensated, written as FP64 to
// out[0..nv): a butterfly over lane distance 16, then recursive halving as in warp_sum_acc,
// after which lane l holds the sum of value l & 15.
__device__ __forceinline__ void warp_sum16(const float* v, int lane, int nv, double* out) {
    float s[16], c[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) two_sum(v[j], __shfl_xor_sync(0xffffffffu, v[j], 16), s[j], c[j]);
#pragma unroll
    for (int o = 8; o >= 1; o >>= 1) {
        const bool up = (lane & o) != 0;
#pragma unroll
        for (int j = 0; j < o; ++j) {
            const float ss = up ? s[j] : s[j + o], cs = up ? c[j] : c[j + o];
            const float sk = up ? s[j + o] : s[j], ck = up ? c[j + o] : c[j];
            const float sr = __shfl_xor_sync(0xffffffffu, ss, o);
            const float cr = __shfl_xor_sync(0xffffffffu, cs, o);
            float e;
            two_sum(sk, sr, s[j], e);
            c[j] = ck + cr + e;
        }
    }
    if (lane < nv) out[lane] = (double)s[0] + (double)c[0];
}

// ---- More-Thuente line search of the CPU path (use_line_search, CPU semantics) ----
// more_thuente_search (src/ndt_cuda/src/optimization/more_thuente.rs:236-410), after More &
// Thuente (1994) with the interpolants of Sun & Yuan (2006): it minimises phi = -score along
// the unit ascent direction, keeping the interval [a_l, a_u] on the auxiliary
// psi(a) = phi(a) - phi(0) - mu phi'(0) a until a trial has psi <= 0 and psi' >= 0, then on
// phi. Each trial is one round of the candidate pass (score and gradient at the trial pose);
// lane 0 of rank 0's controller warp runs the search between rounds, in FP64.
__device__ __forceinline__ double mt_clamp(double a) {
    return a < MT_STEP_MIN ? MT_STEP_MIN : (a > MT_STEP_MAX ? MT_STEP_MAX : a);
}

// minimiser of the cubic through (a, fa, ga) and (b, fb, gb); false when it is complex
__device__ bool mt_cubic(double a, double fa, double ga, double b, double fb, double gb,
                         double& out) {
    const double z = 3.0 * (fb - fa) / (b - a) - gb - ga;
    const double w2 = z * z - gb * ga;
    if (w2 < 0.0) return false;
    const double w = sqrt(w2);
    out = a + (b - a) * (w - ga - z) / (gb - ga + 2.0 * w);
    return true;
}

// next trial (trial_value_selection, more_thuente.rs:83-194); l: the best end so far,
// u: the other end, t: the last trial
__device__ double mt_next(double al, double fl, double gl, double au, double fu, double gu,
                          double at, double ft, double gt) {
    double ac;
    if (ft > fl) {  // bracketed by [al, at]
        if (!mt_cubic(al, fl, gl, at, ft, gt, ac))
            return al - 0.5 * (al - at) * gl / (gl - (fl - ft) / (al - at));
        const double den = gl - (fl - ft) / (al - at);
        if (fabs(den) < 1e-15) return ac;
        const double aq = al - 0.5 * (al - at) * gl / den;
        return fabs(ac - al) < fabs(aq - al) ? ac : 0.5 * (aq + ac);
    }
    if (gt * gl < 0.0) {  // slopes of opposite sign
        const bool ok = mt_cubic(al, fl, gl, at, ft, gt, ac);
        const double as = al - (al - at) / (gl - gt) * gl;
        if (!ok) return as;
        return fabs(ac - at) >= fabs(as - at) ? ac : as;
    }
    if (fabs(gt) <= fabs(gl)) {  // slope shrinking in magnitude
        if (!mt_cubic(al, fl, gl, at, ft, gt, ac))
            ac = at > al ? at + 0.66 * (au - at) : at - 0.66 * (at - au);
        const double as = fabs(gl - gt) > 1e-15 ? al - (al - at) / (gl - gt) * gl : ac;
        const double an = fabs(ac - at) < fabs(as - at) ? ac : as;
        const double lim = at + 0.66 * (au - at);
        return at > al ? fmin(lim, an) : fmax(lim, an);
    }
    if (mt_cubic(au, fu, gu, at, ft, gt, ac)) return ac;  // through the trial and u
    return 0.5 * (al + au);
}

// interval update (update_interval, more_thuente.rs:196-234); true when it shrank to a point
__device__ bool mt_update(AlignShared& sh, double at, double ft, double gt) {
    if (ft > sh.mt_fl) {
        sh.mt_au = at;
        sh.mt_fu = ft;
        sh.mt_gu = gt;
        return false;
    }
    const double side = gt * (sh.mt_al - at);
    if (side > 0.0) {
        sh.mt_al = at;
        sh.mt_fl = ft;
        sh.mt_gl = gt;
        return false;
    }
    if (side < 0.0) {
        sh.mt_au = sh.mt_al;
        sh.mt_fu = sh.mt_fl;
        sh.mt_gu = sh.mt_gl;
        sh.mt_al = at;
        sh.mt_fl = ft;
        sh.mt_gl = gt;
        return false;
    }
    return true;
}

// After the Newton solve (lane 0): the first half of the CPU step, then the search from
// step_size (solver.rs:268-276, 640-660) with its first trial pose in ls_pose[0]; without an
// ascent direction (g.x <= 0) the step is step_size at once. Returns 1 when the alignment is
// finished; sh.ls_active tells whether trials follow.
__device__ __noinline__ int mt_prepare(const AlignParams& P, AlignShared& sh,
                                       const AlignJob& job, AlignOut& o, int it, double score,
                                       int ncorr) {
    double x[6], dn;
    sh.ls_active = 0;
    if (cpu_direction(P, sh, job, o, it, score, ncorr, x, &dn)) return 1;
    const double d0 = dot6(sh.g, x);
    if (d0 <= 0.0) return cpu_step(P, sh, o, it, x, P.step_size);
    for (int i = 0; i < 6; ++i) {
        sh.ls_delta[i] = x[i];
        sh.ls_orig[i] = sh.pose[i];
    }
    sh.ls_phi0 = score;
    sh.ls_dphi0 = d0;
    sh.mt_first = 1;
    sh.mt_at = mt_clamp(P.step_size);
    for (int i = 0; i < 6; ++i) sh.ls_pose[0][i] = sh.pose[i] + x[i] * sh.mt_at;
    sh.ls_active = 1;
    return 0;
}

// After a trial (lane 0; its score and slope in ls_phi[0], ls_dphi[0]): the search's next
// move. Returns -1 with the next trial pose in ls_pose[0], else takes the step (the trial
// meeting the strong Wolfe conditions, or step_max when the search ends without one:
// solver.rs:694-698) and returns cpu_step's result.
__device__ __noinline__ int mt_decide(const AlignParams& P, AlignShared& sh, AlignOut& o,
                                      int it) {
    const double mu = P.ls_mu, nu = P.ls_nu;
    const double phi0 = -sh.ls_phi0, dphi0 = -sh.ls_dphi0;
    const double at = sh.mt_at, phi = -sh.ls_phi[0], dphi = -sh.ls_dphi[0];
    const double psi = phi - phi0 - mu * dphi0 * at, dpsi = dphi - mu * dphi0;
    double step = -1.0;
    if (sh.mt_first) {  // both ends at 0, on psi
        sh.mt_first = 0;
        sh.mt_al = sh.mt_au = 0.0;
        sh.mt_fl = phi0 - phi0 - mu * dphi0 * sh.mt_al;
        sh.mt_fu = phi0 - phi0 - mu * dphi0 * sh.mt_au;
        sh.mt_gl = sh.mt_gu = dphi0 - mu * dphi0;
        sh.mt_open = 1;
        sh.mt_iter = 0;
    } else {
        if (sh.mt_open && psi <= 0.0 && dpsi >= 0.0) {  // from psi to phi
            sh.mt_open = 0;
            sh.mt_fl = sh.mt_fl + phi0 - mu * dphi0 * sh.mt_al;
            sh.mt_gl += mu * dphi0;
            sh.mt_fu = sh.mt_fu + phi0 - mu * dphi0 * sh.mt_au;
            sh.mt_gu += mu * dphi0;
        }
        const bool point = sh.mt_open ? mt_update(sh, at, psi, dpsi) : mt_update(sh, at, phi, dphi);
        if (point || ++sh.mt_iter >= MT_MAX_ITER) step = MT_STEP_MAX;
    }
    if (step < 0.0) {
        if (psi <= 0.0 && fabs(dphi) <= nu * fabs(dphi0)) {
            step = at;
        } else {
            const double an = mt_clamp(
                sh.mt_open ? mt_next(sh.mt_al, sh.mt_fl, sh.mt_gl, sh.mt_au, sh.mt_fu, sh.mt_gu,
                                     at, psi, dpsi)
                           : mt_next(sh.mt_al, sh.mt_fl, sh.mt_gl, sh.mt_au, sh.mt_fu, sh.mt_gu,
                                     at, phi, dphi));
            sh.mt_at = an;
            for (int i = 0; i < 6; ++i) sh.ls_pose[0][i] = sh.ls_orig[i] + sh.ls_delta[i] * an;
            return -1;
        }
    }
    return cpu_step(P, sh, o, it, sh.ls_delta, step);
}

// Line-search set-up after the Newton solve (graph path; ndt_graph_solve_kernel,
// ndt_graph_kernels.cu:388-430): the direction is the raw solve (or -1e-4 g when it failed),
// reversed when g.delta <= 0; phi(0) = score, phi'(0) = g.delta; candidate step lengths 1,
// 0.618, 0.618^2, ... formed as an f32 product as the reference forms them; their poses.
// Lane 0 of the controller warp.
__device__ __noinline__ void ls_prepare(const AlignParams& P, AlignShared& sh) {
    double x[6];
    for (int i = 0; i < 6; ++i) x[i] = sh.solve.ok ? sh.solve.x[i] : -sh.g[i] * 1e-4;
    double dphi = dot6(sh.g, x);
    if (dphi <= 0.0) {
        for (int i = 0; i < 6; ++i) x[i] = -x[i];
        dphi = -dphi;
    }
    for (int i = 0; i < 6; ++i) {
        sh.ls_delta[i] = x[i];
        sh.ls_orig[i] = sh.pose[i];
    }
    sh.ls_phi0 = sh.tot[A_SC];
    sh.ls_dphi0 = dphi;
    sh.ls_best = sh.ls_phi0;  // no candidate above phi(0) yet: no move
    sh.ls_best_alpha = 0.0;
    float a = 1.0f;
    for (int k = 0; k < P.ls_cands; ++k, a *= 0.618f) {
        sh.ls_alpha[k] = (double)a;
        for (int i = 0; i < 6; ++i) sh.ls_pose[k][i] = sh.pose[i] + (double)a * x[i];
    }
}

// phi(alpha_k) and phi'(alpha_k) = g(alpha_k).delta of candidates c_lo <= k < c_hi from the
// cluster sums (lane k, as finalize_gH forms the gradient)
__device__ __forceinline__ void ls_candidates_warp(const AlignParams& P, AlignShared& sh,
                                                   int lane, int c_lo, int c_hi) {
    if (lane >= c_lo && lane < c_hi) {
        const double* t = sh.ls_tot[lane];
        const double(*A)[9] = reinterpret_cast<const double(*)[9]>(sh.ls_Ad[lane]);
        double g[6];
        for (int i = 0; i < 3; ++i) g[i] = t[1 + i];
        for (int r = 0; r < 3; ++r) {
            double v = 0.0;
            for (int q = 0; q < 9; ++q) v += A[r][q] * t[4 + q];
            g[3 + r] = v;
        }
        sh.ls_phi[lane] = t[0];
        sh.ls_dphi[lane] = dot6(g, sh.ls_delta);
    }
}

// Candidate selection and step (ndt_graph_update_kernel, ndt_graph_kernels.cu:626-710): the
// first candidate meeting the strong Wolfe conditions, else the best score above phi(0), else
// no move; step length alpha |delta| (no clamp); then the oscillation and convergence rules
// of the graph path. Applied to candidates c_lo <= k < c_hi on top of the earlier rounds'
// running best. Lane 0 of the controller warp; returns -1 when the round found no Wolfe
// candidate and candidates remain, else 1 when the alignment is finished, 0 when it goes on.
__device__ __noinline__ int ls_decide(const AlignParams& P, AlignShared& sh, AlignOut& o, int it,
                                      int ncorr, int c_lo, int c_hi) {
    const double phi0 = sh.ls_phi0, dphi0 = sh.ls_dphi0;
    double best_alpha = sh.ls_best_alpha, best = sh.ls_best;
    bool wolfe = false;
    for (int k = c_lo; k < c_hi; ++k) {
        const double phi = sh.ls_phi[k], a = sh.ls_alpha[k];
        const bool armijo = phi >= phi0 + P.ls_mu * a * dphi0;
        const bool curvature = fabs(sh.ls_dphi[k]) <= P.ls_nu * fabs(dphi0);
        if (armijo && curvature) {
            best_alpha = a;
            wolfe = true;
            break;
        }
        if (phi > best) {
            best = phi;
            best_alpha = a;
        }
    }
    if (!wolfe && c_hi < P.ls_cands) {
        sh.ls_best = best;
        sh.ls_best_alpha = best_alpha;
        return -1;
    }
    for (int i = 0; i < 6; ++i) sh.pose[i] = sh.ls_orig[i] + best_alpha * sh.ls_delta[i];
    const double step = best_alpha * sqrt(dot6(sh.ls_delta, sh.ls_delta));
    osc_update(sh, sh.pose, it);
    const int conv = step < P.eps;
    if (conv || it + 1 >= P.max_iter) {
        const int status = ncorr == 0 ? NDT_STATUS_NO_CORRESPONDENCES
                                      : (conv ? NDT_STATUS_CONVERGED : NDT_STATUS_MAX_ITERATIONS);
        write_out(o, sh.pose, phi0, sh.H, it + 1, conv && ncorr > 0, ncorr, sh.max_osc, status);
        return 1;
    }
    return 0;
}

// REGCAP: registers per thread the launch bounds allow (128: the default; 80 and 64: more
// resident CTAs per SM at the price of some spills; the autotuner picks)
// LS: the line-search code is compiled in (always for the graph path, where it is switched
// at run time; for the CPU path only in the variants that run its More-Thuente search, so
// the plain CPU kernels keep their registers)
template <int THREADS, bool CPU_SEM, int REGCAP, bool LS>
__global__ void __launch_bounds__(THREADS, 65536 / (THREADS * REGCAP))
    k_ndt_align(const AlignParams P) {
    constexpr int NW = THREADS / 32;
    __shared__ AlignShared sh;
    __shared__ uint32_t s_off27[32];  // neighbour offsets of the dense index
    // dynamic shared memory: [max_nb][THREADS] accepted slots per thread, then the trailing
    // NACC - A_HTR accumulators [NACC - A_HTR][THREADS], then the line search's warp sums
    extern __shared__ uint32_t nbl_smem[];
    float* const sacc =
        reinterpret_cast<float*>(nbl_smem + (size_t)P.max_nb * THREADS) + threadIdx.x;
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
    // line search: every iteration adds candidate passes (two more barriers each); the graph
    // path scores up to 8 candidates in three rounds, the CPU path one More-Thuente trial per
    // round
    const bool line_search = LS && P.ls_cands > 0;

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
        sh.ls_active = 0;
        sh.solve.have_w = 0;
    }
    nbhd_offsets(m, s_off27);
    __syncthreads();
    if (warp == 0) make_frame_warp(sh.pose, CPU_SEM, sh.fr, sh.trig, sh.Ad, sh.Bd, lane);
    __syncthreads();

    uint64_t point_iters = 0, corr_total = 0;
    const uint64_t t_start = global_ns();
    if (tid == 0) {
        sh.cyc[0] = sh.cyc[1] = sh.cyc[2] = sh.cyc[3] = 0ull;
        sh.n_eigen = 0;
    }
    unsigned long long t0 = clock64();
    for (int it = 0;; ++it) {
        const float* fr = sh.fr;
        float acc[NACC];
#pragma unroll
        for (int i = 0; i < A_HTR; ++i) acc[i] = 0.f;
#pragma unroll
        for (int k = 0; k < NACC - A_HTR; ++k) sacc[k * THREADS] = 0.f;
        int nc = 0;
        for (uint32_t i = (uint32_t)rank * THREADS + tid; i < n; i += (uint32_t)K * THREADS) {
            float px = __ldg(pts + 3 * (size_t)i), py = __ldg(pts + 3 * (size_t)i + 1),
                  pz = __ldg(pts + 3 * (size_t)i + 2);
            if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;
            point_terms<CPU_SEM>(m, s_off27, px, py, pz, fr, P.max_nb, P.d1f, P.d2f, acc, sacc, nc,
                                 nbl_smem + tid, THREADS);
        }
#pragma unroll
        for (int k = 0; k < NACC - A_HTR; ++k) acc[A_HTR + k] = sacc[k * THREADS];
        warp_sum_acc(acc, lane, sh.warp_part[warp]);
        nc = __reduce_add_sync(0xffffffffu, nc);
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
                // all remote loads first, then a fixed-order tree (deterministic)
                double v[8];
#pragma unroll
                for (int r = 0; r < 8; ++r)
                    v[r] = r < K ? cluster.map_shared_rank(sh.part, r)[k] : 0.0;
                sh.tot[k] = ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
            }
            __syncthreads();
            if (warp == 0) {
                const unsigned long long ca = clock64();
                finalize_gH(sh.tot, sh.Ad, sh.Bd, sh.g, sh.H, lane);
                __syncwarp();
                const unsigned long long cb = clock64();
                solve_warp<CPU_SEM>(sh.H, sh.g, sh.solve, lane);
                const unsigned long long cc = clock64();
                double* t = nullptr;
                if (lane == 0) {
                    sh.n_eigen += sh.solve.path;
                    if (P.trace && it < P.max_iter) {  // per-iteration record (opt-in)
                        t = P.trace + ((size_t)jid * P.max_iter + it) * TRACE_REC;
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
                    int done = 0;
                    if (!line_search) {
                        done = control_step<CPU_SEM>(P, sh, job, o, it, sh.tot[A_SC], ncorr);
                    } else if (CPU_SEM) {  // trials follow unless the step is already taken
                        done = mt_prepare(P, sh, job, o, it, sh.tot[A_SC], ncorr);
                    } else {
                        ls_prepare(P, sh);  // the step is taken after the candidate pass
                        sh.ls_active = 1;
                    }
                    if (done) {
                        o.point_iters = point_iters;
                        o.corr_total = corr_total;
                    }
                    sh.done = done;
                }
                __syncwarp();
                if (!sh.ls_active) {  // the step is taken: the new pose's frame to every rank
                    make_frame_warp(sh.pose, CPU_SEM, sh.fr, sh.trig, sh.Ad, sh.Bd, lane);
                    if (lane > 0 && lane < K) {
                        AlignShared* rs = cluster.map_shared_rank(&sh, lane);
                        for (int i = 0; i < 6; ++i) rs->pose[i] = sh.pose[i];
                        for (int i = 0; i < NFR; ++i) rs->fr[i] = sh.fr[i];
                    }
                }
                if (lane > 0 && lane < K) {
                    AlignShared* rs = cluster.map_shared_rank(&sh, lane);
                    rs->done = sh.done;
                    rs->ls_active = sh.ls_active;
                }
                if (t) {  // controller sub-phase cycles: assembly, solve, step + next frame
                    t[44] = (double)(cb - ca);
                    t[45] = (double)(cc - cb);
                    t[46] = (double)(clock64() - cc);
                    t[47] = sh.solve.sweeps;
                }
            }
            if (line_search) {  // candidate frames, one warp per candidate, to every rank
                __syncthreads();  // warp 0's decision (ls_active) is visible to the CTA
                const int ncand = !sh.ls_active ? 0 : (CPU_SEM ? 1 : P.ls_cands);
                for (int c = warp; c < ncand; c += NW) {
                    make_frame_warp(sh.ls_pose[c], CPU_SEM, sh.ls_fr[c], sh.ls_trig[c],
                                    sh.ls_Ad[c], nullptr, lane);
                    if (lane > 0 && lane < K) {
                        AlignShared* rs = cluster.map_shared_rank(&sh, lane);
                        for (int i = 0; i < NFR; ++i) rs->ls_fr[c][i] = sh.ls_fr[c][i];
                    }
                }
            }
        }
        unsigned long long t3 = clock64();
        cluster.sync();  // next pose (or done, or the candidate frames) visible in every CTA
        unsigned long long t4 = clock64();
        if (rank == 0 && tid == 0) {
            sh.cyc[0] += t1 - t0;
            sh.cyc[1] += t2 - t1;
            sh.cyc[2] += t3 - t2;
            sh.cyc[3] += t4 - t3;
        }
        t0 = t4;
        if (sh.done) break;
        // Line search: candidates are scored in rounds (step lengths [0, 1), [1, 3), [3, 8));
        // after each round rank 0 applies the selection rule to the candidates scored so far,
        // in order, and stops at the first that meets the strong Wolfe conditions. The rule
        // never looks past that candidate, so the outcome equals scoring all 8 at once, while
        // the common full step (alpha = 1 accepted) costs one candidate pass instead of 8.
        for (int round = 0; line_search && sh.ls_active; ++round) {
            const int c_lo = CPU_SEM ? 0 : (round == 0 ? 0 : (round == 1 ? 1 : 3));
            const int c_hi =
                CPU_SEM ? 1 : min(round == 0 ? 1 : (round == 1 ? 3 : LS_MAX), P.ls_cands);
            // candidate pass: score and gradient of each candidate pose of the round over this
            // rank's points, one candidate after another; FP64 warp sums of each candidate
            // kept in shared memory, summed over the CTA, then over the cluster by rank 0
            double* lsw = reinterpret_cast<double*>(
                nbl_smem + (size_t)(P.max_nb + NACC - A_HTR) * THREADS);
            for (int c = c_lo; c < c_hi; ++c) {
                float a[LS_VALS];
#pragma unroll
                for (int v = 0; v < LS_VALS; ++v) a[v] = 0.f;
                int lc = 0;
                for (uint32_t i = (uint32_t)rank * THREADS + tid; i < n;
                     i += (uint32_t)K * THREADS) {
                    float px = __ldg(pts + 3 * (size_t)i), py = __ldg(pts + 3 * (size_t)i + 1),
                          pz = __ldg(pts + 3 * (size_t)i + 2);
                    if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;
                    point_terms_ls<CPU_SEM>(m, s_off27, px, py, pz, sh.ls_fr[c], P.max_nb, P.d1f,
                                            P.d2f, a, lc, nbl_smem + tid, THREADS);
                }
                double* wout = lsw + ((size_t)warp * LS_MAX + c) * LS_VALS;
                warp_sum16(a, lane, LS_USED - 1, wout);
                lc = __reduce_add_sync(0xffffffffu, lc);
                if (lane == 0) wout[LS_USED - 1] = (double)lc;
            }
            __syncthreads();
            const int nk = (c_hi - c_lo) * LS_USED;
            for (int k = tid; k < nk; k += THREADS) {
                const int c = c_lo + k / LS_USED, v = k % LS_USED;
                double s = 0.0;
                for (int w = 0; w < NW; ++w) s += lsw[((size_t)w * LS_MAX + c) * LS_VALS + v];
                sh.ls_part[c][v] = s;
            }
            const unsigned long long t5 = clock64();
            cluster.sync();  // candidate partials of every CTA are ready
            if (rank == 0) {
                for (int k = tid; k < nk; k += THREADS) {
                    const int c = c_lo + k / LS_USED, v = k % LS_USED;
                    double w8[8];
#pragma unroll
                    for (int r = 0; r < 8; ++r)
                        w8[r] = r < K ? cluster.map_shared_rank(&sh.ls_part[c][v], r)[0] : 0.0;
                    sh.ls_tot[c][v] =
                        ((w8[0] + w8[1]) + (w8[2] + w8[3])) + ((w8[4] + w8[5]) + (w8[6] + w8[7]));
                }
                __syncthreads();
                if (warp == 0) {
                    ls_candidates_warp(P, sh, lane, c_lo, c_hi);
                    __syncwarp();
                    if (lane == 0) {
                        AlignOut& o = P.out[jid];
                        const int r = CPU_SEM ? mt_decide(P, sh, o, it)
                                              : ls_decide(P, sh, o, it, (int)sh.tot[NACC], c_lo,
                                                          c_hi);
                        if (r == 1) {
                            o.point_iters = point_iters;
                            o.corr_total = corr_total;
                        }
                        sh.ls_more = r < 0;
                        sh.done = r == 1;
                    }
                    __syncwarp();
                    if (!sh.ls_more)
                        make_frame_warp(sh.pose, CPU_SEM, sh.fr, sh.trig, sh.Ad, sh.Bd, lane);
                    else if (CPU_SEM)  // the search's next trial
                        make_frame_warp(sh.ls_pose[0], true, sh.ls_fr[0], sh.ls_trig[0],
                                        sh.ls_Ad[0], nullptr, lane);
                    if (lane > 0 && lane < K) {
                        AlignShared* rs = cluster.map_shared_rank(&sh, lane);
                        if (!sh.ls_more) {
                            for (int i = 0; i < 6; ++i) rs->pose[i] = sh.pose[i];
                            for (int i = 0; i < NFR; ++i) rs->fr[i] = sh.fr[i];
                        } else if (CPU_SEM) {
                            for (int i = 0; i < NFR; ++i) rs->ls_fr[0][i] = sh.ls_fr[0][i];
                        }
                        rs->done = sh.done;
                        rs->ls_more = sh.ls_more;
                    }
                }
            }
            const unsigned long long t6 = clock64();
            cluster.sync();  // another round, or the stepped pose (or done), in every CTA
            const unsigned long long t7 = clock64();
            if (rank == 0 && tid == 0) {  // candidate pass as point work, selection as control
                sh.cyc[0] += t5 - t4;
                sh.cyc[2] += t6 - t5;
                sh.cyc[3] += t7 - t6;
            }
            t0 = t4 = t7;
            if (!sh.ls_more) break;
        }
        if (sh.done) break;
    }
    if (rank == 0 && tid == 0) {
        AlignOut& o = P.out[jid];
        for (int i = 0; i < 4; ++i) o.cycles[i] = sh.cyc[i];
        o.n_eigen = sh.n_eigen;
        o.t_start = t_start;
        o.t_end = global_ns();
    }
}

// ------------------------------------------------------------------------------------
// Work-queue Newton kernel
//
// In k_ndt_align a cluster owns one alignment for all its iterations, so a batch runs in
// waves: alignments that need many iterations and start late set the batch's makespan, and
// the cluster's other warps idle while rank 0 runs the FP64 step. Here the unit of work is a
// chunk of one alignment's points for one iteration. A persistent grid of CTAs (all resident)
// claims chunks of any open alignment, oldest alignment first; each chunk's sums go to global
// memory in FP64, and the CTA that finishes the last chunk of an iteration runs that
// alignment's Newton step (the same controller code) and publishes the next frame. Other
// alignments' chunks keep every SM busy meanwhile, and the last alignments of a batch spread
// over the whole GPU.
//
// Claims: QJob.gen_claim packs the alignment's iteration (high word) and the chunks claimed
// so far (low word), so one atomicAdd both claims a chunk and names its iteration. The
// controller resets it to (iteration + 1, 0) after writing the frame, behind a fence; readers
// fence after a claim and read shared state through L2 (__ldcg), since L1 is not coherent
// across SMs. A chunk's partial sums are written behind a fence before its done counter is
// incremented; the controller, after the increment that completes the iteration, fences and
// sums the partials in chunk order, so results do not depend on which CTA ran which chunk.
// No CTA ever waits for another; a CTA that finds nothing to claim polls, and gives up with a
// status bit after P.stall_ns (2 s) without work (every alignment ends within max_iterations
// steps).
// Host batches may still be copying in when the kernel starts (P.qarrive): the points are laid
// out largest alignment first, in copy chunks that start on 768-byte boundaries, and a copy
// stream writes the count of resident points after each chunk. An alignment's first
// iteration is claimable once its last point is resident; the chunks' alignment keeps every
// L1 line a CTA reads inside chunks already copied. Nothing guarantees that the copies run
// while the kernel does (a tool may serialise them), so a CTA never waits for input beyond
// QSTARVE_NS without progress: it leaves, and a continuation launch (P.qresume) queued after
// the last copy finishes whatever is left from the state in global memory.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ld_volatile(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}
__device__ __forceinline__ uint32_t ld_volatile32(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}

// Claim word of an alignment: iteration (16 bits; QDONE once finished), the iteration's chunk
// count (16 bits) and the chunks claimed so far (32 bits). One atomicAdd claims a chunk and
// returns all three consistently.
__device__ __forceinline__ unsigned long long qword(uint32_t gen, uint32_t nch) {
    return ((unsigned long long)gen << 48) | ((unsigned long long)nch << 32);
}
__device__ __forceinline__ uint32_t qw_gen(unsigned long long w) { return (uint32_t)(w >> 48); }
__device__ __forceinline__ uint32_t qw_nch(unsigned long long w) {
    return (uint32_t)(w >> 32) & 0xFFFFu;
}

// Chunks of iteration `it` of an alignment with n points: n / qchunk for its first
// QSPLIT_ITER iterations, then QSPLIT_DIV times as many, that much smaller, and from
// QSPLIT_ITER2 on twice as many again (few alignments run that long). The alignments that
// run long are the ones that finish a batch, on an otherwise idle GPU: smaller chunks spread
// each of their iterations over more SMs. The rule depends on the iteration alone, so every
// run sums an alignment's chunks over the same tree (results are identical run to run). At
// most QMAXCH.
constexpr uint32_t QSPLIT_ITER = 10, QSPLIT_ITER2 = 20;
__device__ __forceinline__ uint32_t queue_chunks(const AlignParams& P, uint32_t n, uint32_t it) {
    const uint32_t size =
        it < QSPLIT_ITER ? (uint32_t)P.qchunk
                         : max(1u, (uint32_t)P.qchunk / (it < QSPLIT_ITER2 ? QSPLIT_DIV
                                                                          : 2 * QSPLIT_DIV));
    return min(n ? (n + size - 1u) / size : 1u, QMAXCH);
}

// Initial state of every alignment: controller state at the initial pose, the first frame,
// the claim word of iteration 0; one warp per alignment.
template <bool CPU_SEM>
__global__ void __launch_bounds__(128) k_queue_init(const AlignParams P) {
    __shared__ double s_trig[4][16];
    __shared__ double s_pose[4][6];
    __shared__ float s_fr[4][NFR];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t j = blockIdx.x * 4 + w;
    if (j >= P.num_jobs) return;
    const AlignJob job = P.jobs[j];
    QCtl* q = P.qctl + j;
    if (lane < 6) s_pose[w][lane] = job.pose[lane];
    __syncwarp();
    make_frame_warp(s_pose[w], CPU_SEM, s_fr[w], s_trig[w], q->Ad, q->Bd, lane);
    for (int i = lane; i < NFR; i += 32) P.qframe[(size_t)j * NFR + i] = s_fr[w][i];
    if (lane < 6) q->pose[lane] = q->best_pose[lane] = job.pose[lane];
    if (lane < 3) q->prev[lane] = q->prev2[lane] = job.pose[lane];
    for (int i = lane; i < 36; i += 32) q->last_H[i] = 0.0;
    if (lane == 0) {
        q->best_score = -INFINITY;
        q->last_corr = q->osc = q->max_osc = q->n_eigen = q->have_w = 0;
        q->point_iters = q->corr_total = 0;
        q->cyc_chunks = q->cyc_ctl = 0;
        q->t_start = 0;
        const uint32_t nch0 = queue_chunks(P, job.n, 0u);
        // withhold (test hook): every chunk of the first iteration already claimed
        P.qjobs[j].gen_claim = qword(0u, nch0) | (P.withhold ? (unsigned long long)nch0 : 0ull);
        P.qjobs[j].done = 0u;
    }
}

// The graph path's step (control_step's !CPU_SEM branch: K3 direction and clamp,
// ndt_graph_kernels.cu:311-463, then K5's oscillation and convergence rules) by the whole
// warp: lanes 0-5 hold the direction's components and the two dot products run as one
// shuffle tree; the scale needs no division unless the step is clamped (dn / dn is 1). Lane 0
// keeps the oscillation history and writes the outputs. Returns 1 (every lane) when the
// alignment is finished.
// osc_update by the warp: lanes 0-2 take one axis each (the differences and their products),
// two shuffle rounds add them, lane 0 decides. A dependent FP64 instruction costs about 170
// cycles on this part, so the three axes in parallel shorten the chain from about 20 such
// instructions to 6. Same tests as osc_update.
__device__ __forceinline__ void osc_update_warp(AlignShared& sh, int it, int lane) {
    double cc = 0.0, pp = 0.0, cp = 0.0;
    if (it >= 1 && lane < 3) {
        const double c = sh.pose[lane] - sh.prev[lane];
        const double q = sh.prev[lane] - sh.prev2[lane];
        cc = c * c;
        pp = q * q;
        cp = c * q;
    }
#pragma unroll
    for (int m = 2; m > 0; m >>= 1) {
        cc += __shfl_xor_sync(0xffffffffu, cc, m);
        pp += __shfl_xor_sync(0xffffffffu, pp, m);
        cp += __shfl_xor_sync(0xffffffffu, cp, m);
    }
    __syncwarp();
    if (lane < 3) {
        sh.prev2[lane] = sh.prev[lane];
        sh.prev[lane] = sh.pose[lane];
    }
    if (lane == 0 && it >= 1) {
        if (cc > 1e-20 && pp > 1e-20) {
            const bool rev = cp < 0.0 && cp * cp > 0.81 * (cc * pp);
            sh.osc = rev ? sh.osc + 1 : 0;
            if (sh.osc > sh.max_osc) sh.max_osc = sh.osc;
        } else {
            sh.osc = 0;
        }
    }
    __syncwarp();
}

// The graph path's step (K5, ndt_graph_kernels.cu:618-847) by the warp: delta = the solve's
// x (or -1e-4 g when it failed), reversed when g . delta <= 0; step = min(|delta|, step_size);
// the pose moves by delta scaled to that step; converged when step < eps. The length is
// compared on its square, and the clamp's scale step_size / |delta| comes from an f32
// reciprocal square root refined by one FP64 Newton step (relative error below 1e-14), so the
// FP64 chain has no square root or division.
__device__ __noinline__ int control_step_graph_warp(const AlignParams& P, AlignShared& sh,
                                                    AlignOut& o, int it, double score,
                                                    int ncorr, int lane) {
    double xi = 0.0, gi = 0.0;
    if (lane < 6) {
        gi = sh.g[lane];
        xi = sh.solve.ok ? sh.solve.x[lane] : -gi * 1e-4;
    }
    double dphi = gi * xi, dn2 = xi * xi;
#pragma unroll
    for (int m = 4; m > 0; m >>= 1) {
        dphi += __shfl_xor_sync(0xffffffffu, dphi, m);
        dn2 += __shfl_xor_sync(0xffffffffu, dn2, m);
    }
    dphi = __shfl_sync(0xffffffffu, dphi, 0);
    dn2 = __shfl_sync(0xffffffffu, dn2, 0);
    if (dphi <= 0.0) xi = -xi;
    double scale;
    int conv;
    if (dn2 > P.step_size * P.step_size) {
        const double r0 = (double)rsqrtf((float)dn2);
        const double r = r0 * fma(-0.5 * dn2, r0 * r0, 1.5);
        scale = P.step_size * r;
        conv = P.step_size < P.eps;
    } else {
        scale = dn2 > 1e-20 ? 1.0 : 0.0;
        conv = dn2 < P.eps * P.eps;
    }
    if (lane < 6) sh.pose[lane] += scale * xi;
    __syncwarp();
    osc_update_warp(sh, it, lane);
    int done = 0;
    if (lane == 0 && (conv || it + 1 >= P.max_iter)) {
        const int status = ncorr == 0 ? NDT_STATUS_NO_CORRESPONDENCES
                                      : (conv ? NDT_STATUS_CONVERGED : NDT_STATUS_MAX_ITERATIONS);
        write_out(o, sh.pose, score, sh.H, it + 1, conv && ncorr > 0, ncorr, sh.max_osc, status);
        done = 1;
    }
    return __shfl_sync(0xffffffffu, done, 0);
}

// Element e of QCtl's FP64 block, in the controller's shared state
__device__ __forceinline__ double* qctl_slot(AlignShared& sh, int e) {
    if (e < 6) return sh.pose + e;
    if (e < 12) return sh.best_pose + (e - 6);
    if (e < 13) return &sh.best_score;
    if (e < 49) return sh.last_H + (e - 13);
    if (e < 52) return sh.prev + (e - 49);
    if (e < 55) return sh.prev2 + (e - 52);
    if (e < 91) return sh.solve.W + (e - 55);
    if (e < 118) return sh.Ad + (e - 91);
    return sh.Bd + (e - 118);
}

// Newton step of alignment `job` after its iteration `it` (warp 0 of the CTA that finished
// the iteration's last chunk, once the CTA has summed the chunk partials into sh.tot):
// state from global memory, the controller of k_ndt_align, then the next frame and claim
// word (or the outputs) published.
template <bool CPU_SEM>
__device__ __noinline__ void queue_control(const AlignParams& P, AlignShared& sh, int job,
                                           uint32_t it, int lane) {
    const unsigned long long c0 = clock64();
    QCtl* q = P.qctl + job;
    const AlignJob jb = P.jobs[job];  // loaded with the state, used after the solve
    uint64_t cnt[2] = {0, 0};  // lane 0: point-iterations and correspondences so far
    {  // the state: every load in flight at once (one L2 round trip), then into shared memory
        const double* qd = reinterpret_cast<const double*>(q);
        double v[6];
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const int e = lane + 32 * r;
            v[r] = e < QCTL_DOUBLES ? __ldcg(qd + e) : 0.0;
        }
        int iv[5] = {0, 0, 0, 0, 0};
        if (lane == 0) {
            cnt[0] = __ldcg(&q->point_iters);
            cnt[1] = __ldcg(&q->corr_total);
            iv[0] = __ldcg(&q->last_corr);
            iv[1] = __ldcg(&q->osc);
            iv[2] = __ldcg(&q->max_osc);
            iv[3] = __ldcg(&q->n_eigen);
            iv[4] = __ldcg(&q->have_w);
        }
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const int e = lane + 32 * r;
            if (e < QCTL_DOUBLES) *qctl_slot(sh, e) = v[r];
        }
        if (lane == 0) {
            sh.last_corr = iv[0];
            sh.osc = iv[1];
            sh.max_osc = iv[2];
            sh.n_eigen = iv[3];
            sh.solve.have_w = iv[4];
        }
    }
    __syncwarp();
    const unsigned long long c1 = clock64();
    finalize_gH(sh.tot, sh.Ad, sh.Bd, sh.g, sh.H, lane);
    __syncwarp();
    solve_warp<CPU_SEM>(sh.H, sh.g, sh.solve, lane);
    const unsigned long long c2 = clock64();
    int done = 0;
    double* t = nullptr;
    if (lane == 0) {
        sh.n_eigen += sh.solve.path;
        if (P.trace && (int)it < P.max_iter) {
            t = P.trace + ((size_t)job * P.max_iter + it) * TRACE_REC;
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
            t[44] = (double)(c1 - c0);  // state load
            t[45] = (double)(c2 - c1);  // assembly + solve
            t[47] = sh.solve.sweeps;
        }
    }
    const int ncorr = (int)sh.tot[NACC];
    AlignOut& o = P.out[job];
    if (CPU_SEM) {
        if (lane == 0) done = control_step<CPU_SEM>(P, sh, jb, o, (int)it, sh.tot[A_SC], ncorr);
    } else {
        done = control_step_graph_warp(P, sh, o, (int)it, sh.tot[A_SC], ncorr, lane);
    }
    if (lane == 0) {
        const uint64_t pi = cnt[0] + jb.n;
        const uint64_t ct = cnt[1] + (uint64_t)ncorr;
        __stcg(&q->point_iters, pi);
        __stcg(&q->corr_total, ct);
        if (done) {
            o.point_iters = pi;
            o.corr_total = ct;
        }
    }
    done = __shfl_sync(0xffffffffu, done, 0);
    if (!done) make_frame_warp(sh.pose, CPU_SEM, sh.fr, sh.trig, sh.Ad, sh.Bd, lane);
    __syncwarp();
    if (!done) {
        double* qd = reinterpret_cast<double*>(q);
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const int e = lane + 32 * r;
            if (e < QCTL_DOUBLES) __stcg(qd + e, *qctl_slot(sh, e));
        }
        for (int i = lane; i < NFR; i += 32) __stcg(P.qframe + (size_t)job * NFR + i, sh.fr[i]);
        if (lane == 0) {
            __stcg(&q->last_corr, sh.last_corr);
            __stcg(&q->osc, sh.osc);
            __stcg(&q->max_osc, sh.max_osc);
            __stcg(&q->n_eigen, sh.n_eigen);
            __stcg(&q->have_w, sh.solve.have_w);
            // every chunk of this iteration has reported: nothing else touches the counter
            // until the claim word below opens the next iteration
            P.qjobs[job].done = 0u;
        }
    }
    if (lane == 0) {
        const unsigned long long c3 = clock64();
        if (t) t[46] = (double)(c3 - c2);  // step + next frame + state store
        const unsigned long long cyc = __ldcg(&q->cyc_ctl) + (c3 - c0);
        __stcg(&q->cyc_ctl, cyc);
        if (done) {
            AlignOut& o = P.out[job];
            o.cycles[0] = __ldcg(&q->cyc_chunks);
            o.cycles[1] = 0;
            o.cycles[2] = cyc;
            o.cycles[3] = 0;
            o.n_eigen = sh.n_eigen;
            o.t_start = __ldcg(&q->t_start);
            o.t_end = global_ns();
        }
    }
    // one release fence for every lane's stores (state, frame, outputs), then the claim word
    __threadfence();
    __syncwarp();
    if (lane == 0) {
        if (done) {
            atomicExch(&P.qjobs[job].gen_claim, qword(QDONE, 0u));
            atomicAdd(P.qcount, 1u);
        } else {
            atomicExch(&P.qjobs[job].gen_claim, qword(it + 1u, queue_chunks(P, jb.n, it + 1u)));
        }
    }
    __syncwarp();
}

template <int THREADS, bool CPU_SEM, int REGCAP, int NPW>
__global__ void __launch_bounds__(THREADS, 65536 / (THREADS * REGCAP))
    k_ndt_queue(const AlignParams P) {
    constexpr int NW = THREADS / 32;
    __shared__ AlignShared sh;
    __shared__ uint32_t s_off27[32];  // neighbour offsets of the dense index
    __shared__ int s_job, s_lw, s_flag;
    __shared__ uint32_t s_chunk, s_gen, s_nch;
    // dynamic shared memory as in k_ndt_align: neighbour lists, then the trailing accumulators
    extern __shared__ uint32_t nbl_smem[];
    float* const sacc =
        reinterpret_cast<float*>(nbl_smem + (size_t)P.max_nb * THREADS) + threadIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const MapView& m = P.map;
    const uint32_t B = P.num_jobs;
    uint64_t idle_since = 0;    // thread 0
    uint32_t seen_arrive = 0;   // thread 0: last value of the input counter seen
    // the chunk's points, staged by one bulk copy (the TMA engine) into shared memory after
    // the neighbour lists and accumulators: P.qchunk + 4 points (the copy starts on a 16-byte
    // boundary, up to 3 points early)
    __shared__ __align__(8) uint64_t s_stage_bar;
    float* const stage =
        reinterpret_cast<float*>(nbl_smem + (size_t)(P.max_nb + NACC - A_HTR) * THREADS);
    uint32_t stage_phase = 0;
    if (tid == 0) {
        s_lw = 0;
        if (P.qstage) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(
                (uint32_t)__cvta_generic_to_shared(&s_stage_bar)));
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    }
    nbhd_offsets(m, s_off27);  // read after the loop's first barrier
    for (;;) {
        __syncthreads();  // the previous chunk (and controller) is finished with shared memory
        if (warp == 0) {
            // claim, lowest iteration first: alignments that need many iterations form the
            // batch's tail, so none may fall behind while others run ahead. Pass 0 finds the
            // lowest iteration (saturated at 255) among the claimable alignments, from the
            // first one not known to be finished; pass 1 tries the claimable ones at that
            // iteration in order (from the oldest); if other CTAs took all of their chunks
            // meanwhile, pass 2 takes any claimable chunk, oldest alignment first.
            int job = -1, first_open = -1;
            uint32_t chunk = 0, gen = 0, nchunks = 0;
            // points resident while the batch is still being copied in (all: ~0)
            uint32_t arrived = 0xFFFFFFFFu;
            if (P.qarrive) {
                arrived = ld_volatile32(P.qarrive);
                if (arrived >= P.qarrive_total) arrived = 0xFFFFFFFFu;
            }
            // whether alignment j has a chunk to claim; open: not finished; g: its iteration
            // (saturated at 255)
            auto claimable = [&](uint32_t j, bool& open, uint32_t& g) -> bool {
                const unsigned long long w = ld_volatile(&P.qjobs[j].gen_claim);
                open = qw_gen(w) != QDONE;
                g = min(qw_gen(w), 255u);
                bool ok = open && (uint32_t)w < qw_nch(w);
                if (ok && arrived != 0xFFFFFFFFu && qw_gen(w) == 0u)
                    ok = P.jobs[j].offset + P.jobs[j].n <= (uint64_t)arrived;
                return ok;
            };
            uint32_t best = 0xFFFFFFFFu;  // min over claimable j of min(iteration, 255) << 24 | j
#pragma unroll 4
            for (uint32_t base = (uint32_t)s_lw; base < B; base += 32) {
                const uint32_t j = base + lane;
                bool open = false;
                uint32_t g = 0;
                if (j < B && claimable(j, open, g)) best = min(best, (g << 24) | j);
                const unsigned om = __ballot_sync(0xffffffffu, open);
                if (first_open < 0 && om) first_open = (int)base + __ffs(om) - 1;
            }
            best = __reduce_min_sync(0xffffffffu, best);
            for (int pass = 1; pass <= 2 && job < 0 && best != 0xFFFFFFFFu; ++pass) {
                const uint32_t gsel = best >> 24;
                const uint32_t start =
                    pass == 1 ? ((best & 0xFFFFFFu) & ~31u) : (uint32_t)max(first_open, 0);
                for (uint32_t base = start; base < B && job < 0; base += 32) {
                    const uint32_t j = base + lane;
                    bool ok = false, open = false;
                    uint32_t g = 0;
                    if (j < B) ok = claimable(j, open, g) && (pass == 2 || g == gsel);
                    unsigned okm = __ballot_sync(0xffffffffu, ok);
                    while (okm != 0u && job < 0) {
                        const int src = __ffs(okm) - 1;
                        okm &= okm - 1u;
                        unsigned long long old = 0ull;
                        if (lane == src) old = atomicAdd(&P.qjobs[j].gen_claim, 1ull);
                        old = __shfl_sync(0xffffffffu, old, src);
                        if (qw_gen(old) != QDONE && (uint32_t)old < qw_nch(old)) {
                            job = (int)base + src;
                            chunk = (uint32_t)old;
                            gen = qw_gen(old);
                            nchunks = qw_nch(old);
                        }
                    }
                }
            }
            __threadfence();  // acquire: the frame of the claimed iteration is published
            if (lane == 0) {
                s_lw = first_open >= 0 ? first_open : (int)B;
                s_job = job;
                s_chunk = chunk;
                s_gen = gen;
                s_nch = nchunks;
            }
        }
        __syncthreads();
        const int job = s_job;
        if (job < 0) {
            // nothing claimable: every alignment finished, or the open ones wait for their
            // Newton step
            if (tid == 0) {
                int stop = s_lw >= (int)B;
                if (!stop) {
                    const uint64_t now = global_ns();
                    bool fed = true;  // every point of the batch is resident
                    if (P.qarrive) {
                        const uint32_t a = ld_volatile32(P.qarrive);
                        fed = a >= P.qarrive_total;
                        if (a != seen_arrive) {  // input still arriving: not a stall
                            seen_arrive = a;
                            idle_since = 0;
                        }
                    }
                    if (idle_since == 0) {
                        idle_since = now;
                    } else if (!fed && now - idle_since > QSTARVE_NS) {
                        stop = 1;  // starved of input: the continuation launch finishes
                    } else if (now - idle_since > P.stall_ns) {
                        atomicOr(P.status, ST_QUEUE_STALL);
                        stop = 1;
                    } else if (fed && blockIdx.x >= gridDim.x / 4u &&
                               now - idle_since > 20000ull) {
                        // near the end of a batch: all but the first quarter of the grid
                        // (by CTA index) leave after 20 us without work, so a kernel queued
                        // on another stream (the next asynchronous batch) can take their
                        // SMs; the quarter that stays serves the remaining iterations (with
                        // fewer than 4 CTAs none stays idle, and the CTA running a Newton
                        // step still claims the next iteration's chunks when it ends)
                        stop = 1;
                    }
                }
                s_flag = stop;
            }
            __syncthreads();
            if (s_flag) break;
            __nanosleep(500);
            continue;
        }
        if (tid == 0) idle_since = 0;
        const unsigned long long c0 = clock64();
        const uint32_t chunk = s_chunk, gen = s_gen, nchunks = s_nch;
        const AlignJob& jb = P.jobs[job];
        if (tid < NFR) sh.fr[tid] = __ldcg(P.qframe + (size_t)job * NFR + tid);
        if (tid == 0 && gen == 0 && chunk == 0) __stcg(&P.qctl[job].t_start, global_ns());
        __syncthreads();
        const float* pts = P.pts + 3 * jb.offset;
        const uint32_t csize = (jb.n + nchunks - 1u) / nchunks;  // this iteration's chunk size
        const uint32_t first = min(jb.n, chunk * csize);
        const uint32_t last = min(jb.n, first + csize);
        // staged points: job-local indices below stage_end come from shared memory (point i
        // at stage[3 (i - stage_first)]); the rest of the chunk (a ragged tail of less than
        // 16 bytes, or every point when staging is off) from global memory
        int64_t stage_first = 0, stage_end = 0;
        if (P.qstage && last > first) {
            const uint64_t g0 = (jb.offset + first) & ~3ull;  // 16-byte aligned point index
            const uint64_t gend = jb.offset + last;
            const uint32_t bytes = (uint32_t)(((gend - g0) * 12ull) & ~15ull);
            if (bytes >= 16 && gend - g0 <= (uint64_t)P.qchunk + 4) {
                const uint32_t bar = (uint32_t)__cvta_generic_to_shared(&s_stage_bar);
                if (tid == 0) {
                    // the CTA's reads of the previous chunk (generic proxy) precede this write
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                                     bar),
                                 "r"(bytes)
                                 : "memory");
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
                        "[%0], [%1], %2, [%3];" ::"r"((uint32_t)__cvta_generic_to_shared(stage)),
                        "l"(P.pts + 3 * g0), "r"(bytes), "r"(bar)
                        : "memory");
                }
                // bounded wait (1 s of the global timer); a copy from global memory that does
                // not land means the device is in trouble: report it and stop this CTA
                const uint64_t t0 = global_ns();
                bool done = false;
                while (!done) {
                    uint32_t ok;
                    asm volatile(
                        "{\n\t.reg .pred p;\n\t"
                        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                        "selp.u32 %0, 1, 0, p;\n\t}"
                        : "=r"(ok)
                        : "r"(bar), "r"(stage_phase)
                        : "memory");
                    done = ok != 0;
                    if (!done && global_ns() - t0 > 1000000000ull) break;
                }
                if (!__syncthreads_and(done ? 1 : 0)) {
                    if (tid == 0) atomicOr(P.status, ST_STAGE_TIMEOUT);
                    return;
                }
                stage_phase ^= 1u;
                stage_first = (int64_t)g0 - (int64_t)jb.offset;
                stage_end = stage_first + (int64_t)(bytes / 12u);
            }
        }
        auto load_point = [&](uint32_t i, float* pv) {
            if ((int64_t)i < stage_end) {
                const float* q = stage + 3 * ((int64_t)i - stage_first);
                pv[0] = q[0];
                pv[1] = q[1];
                pv[2] = q[2];
            } else {
                pv[0] = __ldg(pts + 3 * (size_t)i);
                pv[1] = __ldg(pts + 3 * (size_t)i + 1);
                pv[2] = __ldg(pts + 3 * (size_t)i + 2);
            }
        };
        float acc[NACC];
#pragma unroll
        for (int i = 0; i < A_HTR; ++i) acc[i] = 0.f;
#pragma unroll
        for (int k = 0; k < NACC - A_HTR; ++k) sacc[k * THREADS] = 0.f;
        int nc = 0;
        if (NPW > 1 && m.grid) {
            // groups of NPW lanes share each point's neighbour search (search_group); every
            // lane of a warp runs every round, with or without a point of its own
            for (uint32_t i0 = first; i0 < last; i0 += THREADS) {
                const uint32_t i = i0 + tid;
                float pv[3] = {0.f, 0.f, 0.f}, qh[3] = {0.f, 0.f, 0.f}, ql[3] = {0.f, 0.f, 0.f};
                uint32_t bits = 0u, corner = 0u;
                if (i < last) {
                    load_point(i, pv);
                    if (isfinite(pv[0]) && isfinite(pv[1]) && isfinite(pv[2])) {
                        transform_point(sh.fr, pv, qh, ql);
                        int32_t gc[3];
                        const uint32_t oct = cell_oct_of_sum(m, qh, ql, gc);
                        bits = nbhd_mask(m, gc, oct, corner);
                    }
                }
                const int cnt = search_group<NPW>(m, s_off27, qh, ql, bits, corner, P.max_nb,
                                                  nbl_smem + tid, THREADS, lane);
                __syncwarp();  // the group's list entries are visible to the point's lane
                if (cnt > 0)
                    point_pairs<CPU_SEM>(m, pv, qh, ql, cnt, sh.fr, P.d1f, P.d2f, acc, sacc, nc,
                                         nbl_smem + tid, THREADS);
                __syncwarp();  // lists are read before the next round rewrites them
            }
        } else {
            for (uint32_t i = first + tid; i < last; i += THREADS) {
                float pv[3];
                load_point(i, pv);
                if (!(isfinite(pv[0]) && isfinite(pv[1]) && isfinite(pv[2]))) continue;
                point_terms<CPU_SEM>(m, s_off27, pv[0], pv[1], pv[2], sh.fr, P.max_nb, P.d1f,
                                     P.d2f, acc, sacc, nc, nbl_smem + tid, THREADS);
            }
        }
#pragma unroll
        for (int k = 0; k < NACC - A_HTR; ++k) acc[A_HTR + k] = sacc[k * THREADS];
        warp_sum_acc(acc, lane, sh.warp_part[warp]);
        nc = __reduce_add_sync(0xffffffffu, nc);
        if (lane == 0) sh.warp_part[warp][NACC] = (double)nc;
        __syncthreads();
        double* part = P.qpart + ((size_t)P.qpart_off[job] + chunk) * NRED;
        for (int k = tid; k < NRED; k += THREADS) {
            double s = 0.0;
            for (int w = 0; w < NW; ++w) s += sh.warp_part[w][k];
            __stcg(part + k, s);
        }
        __threadfence();
        __syncthreads();
        if (tid == 0) {
            const uint32_t prev = atomicAdd(&P.qjobs[job].done, 1u);
            s_flag = prev + 1u == nchunks;
            atomicAdd(&P.qctl[job].cyc_chunks, (unsigned long long)(clock64() - c0));
        }
        __syncthreads();
        if (!s_flag) continue;
        __threadfence();  // acquire: every chunk's partials of this iteration are visible
        // the iteration's sums, by the whole CTA in a fixed order: thread (value k, segment s)
        // sums a contiguous run of chunks, then the segments are added in order
        {
            constexpr int NSEG = (THREADS / NRED) < MAX_WARPS ? (THREADS / NRED) : MAX_WARPS;
            const uint32_t seg = (nchunks + NSEG - 1u) / NSEG;
            const double* part0 = P.qpart + (size_t)P.qpart_off[job] * NRED;
            if (tid < NSEG * NRED) {
                const int k = tid % NRED, s = tid / NRED;
                const uint32_t c_lo = min(nchunks, (uint32_t)s * seg);
                const uint32_t c_hi = min(nchunks, c_lo + seg);
                double v = 0.0;
                for (uint32_t c = c_lo; c < c_hi; ++c) v += __ldcg(part0 + (size_t)c * NRED + k);
                sh.warp_part[s][k] = v;
            }
            __syncthreads();
            if (tid < NRED) {
                double v = 0.0;
                for (int s = 0; s < NSEG; ++s) v += sh.warp_part[s][tid];
                sh.tot[tid] = v;
            }
            __syncthreads();
        }
        if (warp == 0) queue_control<CPU_SEM>(P, sh, job, gen, lane);
    }
}

template <int T, bool SEM, int CAP, int NPW>
static cudaError_t launch_queue_k(const AlignParams& p, size_t smem, uint32_t chunks,
                                  cudaStream_t s) {
    auto kern = k_ndt_queue<T, SEM, CAP, NPW>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    // persistent grid: every CTA resident (the kernel's CTAs never wait for each other, so
    // residency is a matter of speed only), at most one CTA per chunk of the batch
    static std::mutex mu;
    static std::map<std::pair<int, size_t>, int> cache;  // (device, smem) -> CTAs, per instance
    int dev = 0;
    cudaGetDevice(&dev);
    int ctas = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find({dev, smem});
        if (it != cache.end()) {
            ctas = it->second;
        } else {
            int per_sm = 0, sms = 0;
            cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, T, smem);
            if (e != cudaSuccess) return e;
            if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)))
                return e;
            ctas = std::max(1, per_sm * sms);
            cache[{dev, smem}] = ctas;
        }
    }
    // at most one CTA per chunk of the batch at the late-iteration chunk size
    const unsigned grid = (unsigned)std::min<uint64_t>(
        (uint64_t)ctas, (uint64_t)QSPLIT_DIV * std::max(1u, chunks));
    AlignParams q = p;
    q.qgrid = grid;
    if (!q.qresume) k_queue_init<SEM><<<(q.num_jobs + 3) / 4, 128, 0, s>>>(q);
    kern<<<grid, T, smem, s>>>(q);
    return cudaGetLastError();
}

template <int T, int CAP>
static int launch_queue_t(const AlignParams& p, uint32_t chunks, cudaStream_t s, int npw) {
    // neighbour lists, trailing accumulators, then (staging) the chunk's points
    const size_t smem = (size_t)T * (p.max_nb + NACC - A_HTR) * sizeof(uint32_t) +
                        (p.qstage ? ((size_t)p.qchunk + 4) * 12 : 0);
    cudaError_t e;
    if (p.semantics == NDT_SEMANTICS_CPU) {
        e = launch_queue_k<T, true, CAP, 1>(p, smem, chunks, s);
    } else if (T == 256 && CAP == 64 && npw == 2) {
        e = launch_queue_k<T, false, CAP, 2>(p, smem, chunks, s);
    } else if (T == 256 && CAP == 64 && npw == 4) {
        e = launch_queue_k<T, false, CAP, 4>(p, smem, chunks, s);
    } else {
        e = launch_queue_k<T, false, CAP, 1>(p, smem, chunks, s);
    }
    return cuda_fail(e, "work-queue align launch");
}

template <int T, bool SEM, int CAP, bool LS>
static cudaError_t launch_k(cudaLaunchConfig_t& cfg, const AlignParams& p, int K) {
    auto kern = k_ndt_align<T, SEM, CAP, LS>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cfg.dynamicSmemBytes);
    if (K > 8) cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return cudaLaunchKernelEx(&cfg, kern, p);
}

template <int T, int CAP>
static int launch_t(const AlignParams& p, int K, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.num_jobs * K, 1, 1);
    cfg.blockDim = dim3(T, 1, 1);
    // [max_nb][T] neighbour lists, [NACC - A_HTR][T] accumulators, then (line search)
    // [T/32][LS_MAX][LS_VALS] FP64 warp sums; the first two are multiples of 8 bytes (T is)
    cfg.dynamicSmemBytes = (size_t)T * (p.max_nb + NACC - A_HTR) * sizeof(uint32_t) +
                           (p.ls_cands > 0 ? (size_t)(T / 32) * LS_MAX * LS_VALS * sizeof(double)
                                           : 0);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // the CPU path's line search runs in the 128-register variant of the shape
    cudaError_t e = p.semantics != NDT_SEMANTICS_CPU
                        ? launch_k<T, false, CAP, true>(cfg, p, K)
                        : (p.ls_cands > 0 ? launch_k<T, true, 128, true>(cfg, p, K)
                                          : launch_k<T, true, CAP, false>(cfg, p, K));
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
    const int R = shape.regcap;
    if (shape.queue > 0) {
        if (p.ls_cands > 0 || !p.qjobs) {
            set_error("the work-queue kernel takes no line search and needs its buffers");
            return NDT_ERR_INVALID_ARGUMENT;
        }
        q.qchunk = shape.threads * shape.queue;
        // staging needs a 16-byte aligned points buffer (the bulk copy's rule)
        q.qstage = shape.stage > 0 && ((uintptr_t)p.pts & 15u) == 0 ? 1 : 0;
        const int npw = shape.npw;
        if (npw > 1 && !(shape.threads == 256 && R != 80 && (npw == 2 || npw == 4) &&
                         p.semantics != NDT_SEMANTICS_CPU)) {
            set_error("lanes per point 2 or 4 are built for the graph semantics' 256-thread, "
                      "64-register work-queue kernel");
            return NDT_ERR_INVALID_ARGUMENT;
        }
        switch (shape.threads) {
            case 128: return launch_queue_t<128, 64>(q, p.qchunks_total, s, 1);
            case 256:
                return R == 80 ? launch_queue_t<256, 80>(q, p.qchunks_total, s, 1)
                               : launch_queue_t<256, 64>(q, p.qchunks_total, s, npw);
            case 512: return launch_queue_t<512, 128>(q, p.qchunks_total, s, 1);
            default:
                set_error("threads per CTA must be 128, 256 or 512");
                return NDT_ERR_INVALID_ARGUMENT;
        }
    }
    switch (shape.threads) {
        case 128:
            return R == 64 ? launch_t<128, 64>(q, K, s)
                           : (R == 80 ? launch_t<128, 80>(q, K, s) : launch_t<128, 128>(q, K, s));
        case 256:
            return R == 48   ? launch_t<256, 48>(q, K, s)
                   : R == 64 ? launch_t<256, 64>(q, K, s)
                   : R == 80 ? launch_t<256, 80>(q, K, s)
                             : launch_t<256, 128>(q, K, s);
        case 512: return launch_t<512, 128>(q, K, s);
        default:
            set_error("threads per CTA must be 128, 256 or 512");
            return NDT_ERR_INVALID_ARGUMENT;
    }
}

}  // namespace ndtgb
