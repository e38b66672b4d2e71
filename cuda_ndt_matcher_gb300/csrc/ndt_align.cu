// ndt_align.cu — persistent Newton kernel for NDT alignment on sm_103a.
//
// One thread-block cluster owns one alignment for all of its iterations (graph kernels
// K1-K5 of src/cuda_ffi/csrc/ndt_graph_kernels.cu fused into one launch; many alignments
// of uneven size share the launch, one cluster each). Per iteration:
//   1. every thread transforms its points (f32), finds the voxels of the 27 surrounding cells
//      through the hash (graph_hash_query_inline semantics: fixed offset order, one voxel per
//      cell, dist^2 <= res^2, at most max_nb), and aggregates per point
//        S = sum -d1 e,  G = sum w c,  M = sum w (C - d2 c c^T)    (w = d1 d2 e, c = C x)
//      which it folds into 73 FP32 moment accumulators
//        score, G, G p^T, M, M (x) p, M (x) p p^T                   (FP32 per-point terms)
//      — the Hessian/gradient of Magnusson eqs. 6.12-6.13 factor through the pose-constant
//      angular derivative matrices, so the 6x6 contraction happens once per iteration;
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

constexpr int NACC = 73;          // float moment accumulators
constexpr int NRED = NACC + 1;    // + correspondence count
constexpr int MAX_WARPS = 16;

// accumulator offsets
constexpr int A_SC = 0, A_G = 1, A_GP = 4, A_M = 13, A_MP = 19, A_MPP = 37;

struct AlignShared {
    double warp_part[MAX_WARPS][NRED];
    double part[NRED];
    double tot[NRED];
    double pose[6];
    double H[36];
    double g[6];
    float Rt[12];
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

// R = Rx(roll) Ry(pitch) Rz(yaw) and t, rounded to f32 for the per-point transform.
__device__ void pose_to_Rt(const double* pose, float* Rt) {
    double sr, cr, sp, cp, sy, cy;
    sincos(pose[3], &sr, &cr);
    sincos(pose[4], &sp, &cp);
    sincos(pose[5], &sy, &cy);
    Rt[0] = (float)(cp * cy);
    Rt[1] = (float)(-cp * sy);
    Rt[2] = (float)sp;
    Rt[3] = (float)(sr * sp * cy + cr * sy);
    Rt[4] = (float)(cr * cy - sr * sp * sy);
    Rt[5] = (float)(-sr * cp);
    Rt[6] = (float)(sr * sy - cr * sp * cy);
    Rt[7] = (float)(cr * sp * sy + sr * cy);
    Rt[8] = (float)(cr * cp);
    Rt[9] = (float)pose[0];
    Rt[10] = (float)pose[1];
    Rt[11] = (float)pose[2];
}

// ------------------------------------------------------------------------------------
// 6x6 solvers (FP64, one thread)
// ------------------------------------------------------------------------------------
// Cholesky of a symmetric matrix; false if a pivot is not positive or the pivot ratio
// falls below 1e-6 (then the caller takes the eigen path).
__device__ bool chol6(const double* M, double* L) {
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

// Cyclic Jacobi eigen-decomposition with the reference's stopping rules
// (jacobi_svd_6x6.cuh:135-210): A becomes diagonal, V accumulates the rotations.
__device__ void jacobi6(double* A, double* V) {
    for (int i = 0; i < 36; ++i) V[i] = (i % 7 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0, dg = 0.0;
        for (int i = 0; i < 6; ++i) {
            dg += A[i * 6 + i] * A[i * 6 + i];
            for (int j = i + 1; j < 6; ++j) off += A[i * 6 + j] * A[i * 6 + j];
        }
        off *= 2.0;
        if (off < 1e-28 * dg) break;
        for (int p = 0; p < 5; ++p) {
            for (int q = p + 1; q < 6; ++q) {
                double apq = A[p * 6 + q];
                if (fabs(apq) < 1e-15) continue;
                double app = A[p * 6 + p], aqq = A[q * 6 + q];
                double tau = (aqq - app) / (2.0 * apq);
                double t = tau >= 0.0 ? 1.0 / (tau + sqrt(tau * tau + 1.0))
                                      : -1.0 / (-tau + sqrt(tau * tau + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                double c2 = c * c, s2 = s * s, cs = c * s;
                A[p * 6 + p] = c2 * app + s2 * aqq - 2.0 * cs * apq;
                A[q * 6 + q] = s2 * app + c2 * aqq + 2.0 * cs * apq;
                A[p * 6 + q] = 0.0;
                A[q * 6 + p] = 0.0;
                for (int k = 0; k < 6; ++k) {
                    if (k == p || k == q) continue;
                    double apk = A[p * 6 + k], aqk = A[q * 6 + k];
                    double np = c * apk - s * aqk, nq = s * apk + c * aqk;
                    A[p * 6 + k] = np;
                    A[k * 6 + p] = np;
                    A[q * 6 + k] = nq;
                    A[k * 6 + q] = nq;
                }
                for (int i = 0; i < 6; ++i) {
                    double vip = V[i * 6 + p], viq = V[i * 6 + q];
                    V[i * 6 + p] = c * vip - s * viq;
                    V[i * 6 + q] = s * vip + c * viq;
                }
            }
        }
    }
}

// x = V f(lambda) V^T (-g) with f(l) = 1/|l| (graph semantics) or 1/l (CPU semantics)
__device__ int eig_apply(const double* A, const double* V, const double* g, bool use_abs,
                         double thr, double* x) {
    double z[6];
    int nz = 0;
    for (int i = 0; i < 6; ++i) {
        double y = 0.0;
        for (int j = 0; j < 6; ++j) y += V[j * 6 + i] * (-g[j]);
        double l = A[i * 6 + i];
        double al = fabs(l);
        if (al > thr) {
            z[i] = y / (use_abs ? al : l);
            nz++;
        } else {
            z[i] = 0.0;
        }
    }
    for (int i = 0; i < 6; ++i) {
        double s = 0.0;
        for (int j = 0; j < 6; ++j) s += V[i * 6 + j] * z[j];
        x[i] = s;
    }
    return nz;
}

// Graph semantics (K3): pseudo-inverse with |lambda|, relative cut 1e-10 (min 1e-15).
__device__ bool solve_graph(const double* H, const double* g, double* x) {
    double M[36], L[36];
    // definite and well conditioned: the pseudo-inverse is (sH)^-1 (-g), s = sign
    for (int sgn = 1; sgn >= -1; sgn -= 2) {
        for (int i = 0; i < 36; ++i) M[i] = sgn * H[i];
        if (chol6(M, L)) {
            double b[6];
            for (int i = 0; i < 6; ++i) b[i] = -g[i];
            chol6_solve(L, b, x);
            return true;
        }
    }
    double A[36], V[36];
    for (int i = 0; i < 36; ++i) A[i] = H[i];
    jacobi6(A, V);
    double mx = 0.0;
    for (int i = 0; i < 6; ++i) mx = fmax(mx, fabs(A[i * 6 + i]));
    double thr = fmax(1e-10 * mx, 1e-15);
    return eig_apply(A, V, g, true, thr, x) > 0;
}

// CPU semantics: newton_step_negative_definite(g, H, -1e-3, 1e-10).
__device__ bool solve_cpu(const double* H, const double* g, double* x) {
    double M[36], L[36];
    for (int i = 0; i < 36; ++i) M[i] = -H[i];
    if (chol6(M, L)) {  // H negative definite: x = H^-1 (-g) = (-H)^-1 g
        chol6_solve(L, g, x);
        return true;
    }
    double A[36], V[36];
    for (int i = 0; i < 36; ++i) A[i] = H[i];
    jacobi6(A, V);
    bool nd = true;
    for (int i = 0; i < 6; ++i)
        if (!(A[i * 6 + i] < 0.0)) nd = false;
    if (!nd)
        for (int i = 0; i < 6; ++i)
            if (A[i * 6 + i] > -1e-3) A[i * 6 + i] = -1e-3;
    double mx = 0.0;
    for (int i = 0; i < 6; ++i) mx = fmax(mx, fabs(A[i * 6 + i]));
    if (mx < 1e-10) return false;
    eig_apply(A, V, g, false, 1e-10, x);
    return true;
}

// ------------------------------------------------------------------------------------
// Per-point work
// ------------------------------------------------------------------------------------
template <bool CPU_SEM>
__device__ __forceinline__ void point_terms(const MapView& m, float px, float py, float pz,
                                            const float* Rt, int max_nb, float d1f, float d2f,
                                            float* acc, int& ncorr) {
    float qx = fmaf(Rt[0], px, fmaf(Rt[1], py, fmaf(Rt[2], pz, Rt[9])));
    float qy = fmaf(Rt[3], px, fmaf(Rt[4], py, fmaf(Rt[5], pz, Rt[10])));
    float qz = fmaf(Rt[6], px, fmaf(Rt[7], py, fmaf(Rt[8], pz, Rt[11])));
    int32_t gx = (int32_t)floorf(__fmul_rn(qx, m.inv_res));
    int32_t gy = (int32_t)floorf(__fmul_rn(qy, m.inv_res));
    int32_t gz = (int32_t)floorf(__fmul_rn(qz, m.inv_res));
    float S = 0.f, G0 = 0.f, G1 = 0.f, G2 = 0.f;
    float M0 = 0.f, M1 = 0.f, M2 = 0.f, M3 = 0.f, M4 = 0.f, M5 = 0.f;
    int cnt = 0;
    const float d1d2 = d1f * d2f;
#pragma unroll 1
    for (int c = 0; c < 27; ++c) {
        if (cnt >= max_nb) break;
        int dx, dy, dz;
        offset27(c, dx, dy, dz);
        int32_t cx = gx + dx, cy = gy + dy, cz = gz + dz;
        uint32_t key = local_key(m, cx, cy, cz);
        if (key == EMPTY_KEY) continue;
        uint32_t home = (uint32_t)fmix64(pack21(cx, cy, cz)) & m.mask;
        uint4 sv;
        int32_t s = probe(m, key, home, &sv);
        if (s < 0) continue;
        float mx = __uint_as_float(sv.y), my = __uint_as_float(sv.z), mz = __uint_as_float(sv.w);
        if (dist2_rn(qx, qy, qz, mx, my, mz) > m.r2) continue;
        cnt++;
        float4 ca = __ldg(m.slot_icov + 2 * (size_t)s);
        float4 cb = __ldg(m.slot_icov + 2 * (size_t)s + 1);
        // C = [[ca.x ca.y ca.z] [ca.y ca.w cb.x] [ca.z cb.x cb.y]]
        float x0 = qx - mx, x1 = qy - my, x2 = qz - mz;
        float c0 = fmaf(ca.x, x0, fmaf(ca.y, x1, ca.z * x2));
        float c1 = fmaf(ca.y, x0, fmaf(ca.w, x1, cb.x * x2));
        float c2 = fmaf(ca.z, x0, fmaf(cb.x, x1, cb.y * x2));
        float sq = fmaf(x0, c0, fmaf(x1, c1, x2 * c2));
        float e = expf(-0.5f * d2f * sq);
        if (CPU_SEM) {
            float wn = d2f * e;  // compute_derivative_single: zero unless d2*e in [0, 1]
            if (!(wn >= 0.f && wn <= 1.f)) continue;
        }
        float w = d1d2 * e;
        float wd = w * d2f;
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
    const float p[3] = {px, py, pz};
    const float G[3] = {G0, G1, G2};
    const float M[6] = {M0, M1, M2, M3, M4, M5};
    const float pp[6] = {px * px, px * py, px * pz, py * py, py * pz, pz * pz};
    acc[A_SC] += S;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        acc[A_G + a] += G[a];
#pragma unroll
        for (int b = 0; b < 3; ++b) acc[A_GP + 3 * a + b] = fmaf(G[a], p[b], acc[A_GP + 3 * a + b]);
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        acc[A_M + k] += M[k];
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[A_MP + 3 * k + c] = fmaf(M[k], p[c], acc[A_MP + 3 * k + c]);
#pragma unroll
        for (int j = 0; j < 6; ++j)
            acc[A_MPP + 6 * k + j] = fmaf(M[k], pp[j], acc[A_MPP + 6 * k + j]);
    }
}

// g (6) and H (6x6) from the reduced moments (FP64), lanes of one warp share the work.
__device__ void finalize_gH(const double* tot, const double* pose, bool small, double* g,
                            double* H, int lane) {
    double A[3][9], B[6][9];
    angular_mats(pose, small, A, B);
    const double* GP = tot + A_GP;
    const double* MT = tot + A_M;
    const double* MP = tot + A_MP;
    const double* MPP = tot + A_MPP;
    // lanes 0..5: gradient; lanes 0..20: one upper-triangle Hessian entry each
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
        double v = 0.0;
        if (j < 3) {
            v = MT[sym3(i, j)];
        } else if (i < 3) {
            const double* Ak = A[j - 3];
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c) v += Ak[b * 3 + c] * MP[3 * sym3(i, b) + c];
        } else {
            int k = i - 3, l = j - 3;
            const double* Ak = A[k];
            const double* Al = A[l];
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    int ab = sym3(a, b);
                    for (int c = 0; c < 3; ++c) {
                        double akac = Ak[a * 3 + c];
                        if (akac == 0.0) continue;
                        for (int d = 0; d < 3; ++d)
                            v += akac * Al[b * 3 + d] * MPP[6 * ab + sym3(c, d)];
                    }
                }
            // pair index of (k, l), k <= l: rr rp ry pp py yy
            int kl = (k == 0) ? l : (k == 1 ? 2 + l : 5);
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
__device__ int control_step(const AlignParams& P, AlignShared& sh, const AlignJob& job,
                            AlignOut& o, int it, double score, int ncorr) {
    double* pose = sh.pose;
    const double* g = sh.g;
    const double* H = sh.H;
    if (!CPU_SEM) {
        double x[6];
        if (!solve_graph(H, g, x))
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
    if (!solve_cpu(H, g, x)) {
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

template <int THREADS, bool CPU_SEM>
__global__ void __launch_bounds__(THREADS, (THREADS <= 256 ? 2 : 1))
    k_ndt_align(const AlignParams P) {
    constexpr int NW = THREADS / 32;
    __shared__ AlignShared sh;
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
        pose_to_Rt(sh.pose, sh.Rt);
    }
    __syncthreads();

    uint64_t point_iters = 0, corr_total = 0;
    for (int it = 0;; ++it) {
        float Rt[12];
#pragma unroll
        for (int i = 0; i < 12; ++i) Rt[i] = sh.Rt[i];
        float acc[NACC];
#pragma unroll
        for (int i = 0; i < NACC; ++i) acc[i] = 0.f;
        int nc = 0;
        for (uint32_t i = (uint32_t)rank * THREADS + tid; i < n; i += (uint32_t)K * THREADS) {
            float px = __ldg(pts + 3 * (size_t)i), py = __ldg(pts + 3 * (size_t)i + 1),
                  pz = __ldg(pts + 3 * (size_t)i + 2);
            if (!(isfinite(px) && isfinite(py) && isfinite(pz))) continue;
            point_terms<CPU_SEM>(m, px, py, pz, Rt, P.max_nb, P.d1f, P.d2f, acc, nc);
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
        cluster.sync();  // partials of every CTA of the cluster are ready
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
                if (lane == 0) {
                    int ncorr = (int)sh.tot[NACC];
                    point_iters += n;
                    corr_total += (uint64_t)ncorr;
                    AlignOut& o = P.out[jid];
                    int done = control_step<CPU_SEM>(P, sh, job, o, it, sh.tot[A_SC], ncorr);
                    if (done) {
                        o.point_iters = point_iters;
                        o.corr_total = corr_total;
                    }
                    pose_to_Rt(sh.pose, sh.Rt);
                    sh.done = done;
                }
                __syncwarp();
                if (lane > 0 && lane < K) {
                    AlignShared* rs = cluster.map_shared_rank(&sh, lane);
                    for (int i = 0; i < 6; ++i) rs->pose[i] = sh.pose[i];
                    for (int i = 0; i < 12; ++i) rs->Rt[i] = sh.Rt[i];
                    rs->done = sh.done;
                }
            }
        }
        cluster.sync();  // next pose (or done) visible in every CTA
        if (sh.done) break;
    }
}

template <int T>
static int launch_t(const AlignParams& p, int K, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.num_jobs * K, 1, 1);
    cfg.blockDim = dim3(T, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e;
    if (p.semantics == NDT_SEMANTICS_CPU) {
        if (K > 8)
            cudaFuncSetAttribute(k_ndt_align<T, true>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaLaunchKernelEx(&cfg, k_ndt_align<T, true>, p);
    } else {
        if (K > 8)
            cudaFuncSetAttribute(k_ndt_align<T, false>,
                                 cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        e = cudaLaunchKernelEx(&cfg, k_ndt_align<T, false>, p);
    }
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
    switch (shape.threads) {
        case 128: return launch_t<128>(q, K, s);
        case 256: return launch_t<256>(q, K, s);
        case 512: return launch_t<512>(q, K, s);
        default:
            set_error("threads per CTA must be 128, 256 or 512");
            return NDT_ERR_INVALID_ARGUMENT;
    }
}

}  // namespace ndtgb
