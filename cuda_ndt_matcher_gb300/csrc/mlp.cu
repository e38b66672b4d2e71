// mlp.cu — the learned initial-pose proposal network (training and inference on sm_103a).
//
// The reference has no learned stage; this is the proposal stage that replaces most random
// particles of the initial-pose search. Network: input 64x64x8 scan occupancy + 64x64 map
// height crop (36,864 features, bf16) -> 4 hidden layers of 512 (GELU) -> 16 proposals of
// (dx, dy, dyaw, logit). Every matrix product is the tcgen05 GEMM of tc_gemm.cu
// (D = A B^T, both operands K-major bf16, f32 accumulate):
//   forward   Z_l   = X_l  W_l^T          A = X_l  [B x in],  B = W_l    [out x in]
//   dW_l            = dZ_l^T X_l          A = dZ_l^T [out x B], B = X_l^T [in x B]
//   dX_l            = dZ_l W_l            A = dZ_l [B x out],  B = W_l^T  [in x out]
// so activations and output gradients are written in both layouts by the elementwise kernels,
// and each weight keeps a bf16 copy and a bf16 transposed copy next to its f32 master.
//
// Features (per sample, on the device):
//   scan grid : sensor points rotated by the coarse yaw (world-aligned, centred on the sensor),
//               cells of 1 m over x, y in [-32, 32) m and z in [-2, 6) m; 1 where a point falls;
//   map crop  : 64 x 64 cells of 1 m centred on the coarse x, y from the map's height image
//               (highest map point per 1 m column): 0 for an empty column, else
//               0.1 + clamp((h - z_coarse + 2) / 10, 0, 0.9).
// Targets: the correction from the coarse pose to the converged pose, dx, dy (world frame,
// metres) and dyaw (wrapped to [-pi, pi)). Outputs are in normalised units: dx = 4 o0,
// dy = 4 o1, dyaw = pi o2, logit = o3.
// Loss per sample (relaxed winner-take-all over proposals j, Rupprecht et al. 2017):
//   e_j = (o0 - tx/4)^2 + (o1 - ty/4)^2 + (w wrap(pi o2 - tyaw) / pi)^2,  j* = argmin e_j,
//   (w = yaw_weight, 8 by default: NDT's yaw basin is far narrower than pi next to 4 m),
//   L = e_j* + CE(softmax(logits), j*) + 0.05 mean_{j != j*} e_j,   averaged over the batch.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ndt_internal.h"

namespace ndtgb {

int gemm_bf16_tn(const void* A, const void* B, float* D, int M, int N, int K, int ldd,
                 uint32_t* d_err, cudaStream_t s, int splits, const GemmEpilogue* epi);
constexpr int PN_MAX_SPLITS = 16;

constexpr int PN_GRID = 64, PN_ZB = 8;
constexpr int PN_SCAN_FEATS = PN_GRID * PN_GRID * PN_ZB;  // 32768
constexpr int PN_MAP_FEATS = PN_GRID * PN_GRID;           // 4096
constexpr int PN_OUT_PER = 4;                             // dx, dy, dyaw, logit
constexpr float PN_XY_SCALE = 4.0f;
constexpr float PN_PI = 3.14159265358979f;
constexpr float PN_EPS_WTA = 0.05f;

__device__ __forceinline__ float gelu(float z) {  // tanh approximation
    const float k = 0.7978845608f;                 // sqrt(2 / pi)
    const float u = k * (z + 0.044715f * z * z * z);
    return 0.5f * z * (1.f + tanhf(u));
}
__device__ __forceinline__ float gelu_grad(float z) {
    const float k = 0.7978845608f;
    const float u = k * (z + 0.044715f * z * z * z);
    const float t = tanhf(u);
    return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * k * (1.f + 3.f * 0.044715f * z * z);
}
__device__ __forceinline__ float wrap_pi(float a) {
    return a - 2.f * PN_PI * floorf((a + PN_PI) / (2.f * PN_PI));
}

// ---- elementwise kernels ----------------------------------------------------------
// Z [B x N] f32 (+ bias) -> X [B x N] bf16 and XT [N x B] bf16 (GELU unless `linear`);
// with split-K partials Zp (splits x [B x N]) Z is their sum
__global__ void k_bias_act(float* __restrict__ Z, const float* __restrict__ Zp, int splits,
                           const float* __restrict__ bias, int B, int N, int linear,
                           __nv_bfloat16* __restrict__ X, __nv_bfloat16* __restrict__ XT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * N) return;
    const int b = i / N, n = i % N;
    float acc;
    if (Zp) {
        acc = 0.f;
        for (int s = 0; s < splits; ++s) acc += Zp[(size_t)s * B * N + i];
    } else {
        acc = Z[i];
    }
    const float z = acc + bias[n];
    Z[i] = z;
    if (X) {
        const __nv_bfloat16 h = __float2bfloat16(linear ? z : gelu(z));
        X[i] = h;
        if (XT) XT[(size_t)n * B + b] = h;
    }
}

// Bias gradients of every layer in one launch: column sums over the batch of each layer's
// output gradient (one thread per column of the concatenated layers, fixed summation order)
constexpr int PN_MAX_LAYERS = 16;
struct ColsumTable {
    const float* g[PN_MAX_LAYERS];
    float* out[PN_MAX_LAYERS];
    int n[PN_MAX_LAYERS];
    int start[PN_MAX_LAYERS + 1];
    int layers;
};
// One block of 32 x 32 threads per 32 columns: lane x takes column c0 + x, row group y the
// rows y, y + 32, ... (coalesced 128-byte rows), then the 32 row-group sums of a column are
// added in a fixed order (deterministic).
constexpr int PN_CS_ROWS = 32;
__global__ void __launch_bounds__(32 * PN_CS_ROWS) k_colsum_all(const ColsumTable t, int B) {
    __shared__ float part[PN_CS_ROWS][33];
    const int x = threadIdx.x & 31, y = threadIdx.x >> 5;
    const int c = blockIdx.x * 32 + x;
    float s = 0.f;
    int l = 0, n = 0;
    const bool ok = c < t.start[t.layers];
    if (ok) {
        while (c >= t.start[l + 1]) ++l;
        n = c - t.start[l];
        const int N = t.n[l];
        const float* G = t.g[l] + n;
#pragma unroll 4
        for (int b = y; b < B; b += PN_CS_ROWS) s += G[(size_t)b * N];
    }
    part[y][x] = s;
    __syncthreads();
    if (y == 0 && ok) {
        float tot = 0.f;
        for (int r = 0; r < PN_CS_ROWS; ++r) tot += part[r][x];
        t.out[l][n] = tot;
    }
}

// loss and output gradient, one thread per sample; O [B x P*4] (biased), T [B x 3]
__global__ void k_loss(const float* __restrict__ O, const float* __restrict__ T, int B, int P,
                       float yw, float* __restrict__ loss, float* __restrict__ dOf,
                       __nv_bfloat16* __restrict__ dO, __nv_bfloat16* __restrict__ dOT) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float* o = O + (size_t)b * P * PN_OUT_PER;
    const float tx = T[3 * b] / PN_XY_SCALE, ty = T[3 * b + 1] / PN_XY_SCALE, tyaw = T[3 * b + 2];
    float best = INFINITY, mx = -INFINITY, esum = 0.f;
    int jb = 0;
    for (int j = 0; j < P; ++j) {
        const float ex = o[4 * j] - tx, ey = o[4 * j + 1] - ty;
        const float ea = yw * wrap_pi(PN_PI * o[4 * j + 2] - tyaw) / PN_PI;
        const float e = ex * ex + ey * ey + ea * ea;
        esum += e;
        if (e < best) {
            best = e;
            jb = j;
        }
        mx = fmaxf(mx, o[4 * j + 3]);
    }
    float z = 0.f;
    for (int j = 0; j < P; ++j) z += expf(o[4 * j + 3] - mx);
    const float lse = mx + logf(z);
    const float w_other = P > 1 ? PN_EPS_WTA / (float)(P - 1) : 0.f;
    loss[b] = best + (lse - o[4 * jb + 3]) + w_other * (esum - best);
    const float inv_b = 1.f / (float)B;
    const int ld = P * PN_OUT_PER;
    for (int j = 0; j < P; ++j) {
        const float w = (j == jb ? 1.f : w_other) * inv_b;
        const float ex = o[4 * j] - tx, ey = o[4 * j + 1] - ty;
        const float ea = yw * wrap_pi(PN_PI * o[4 * j + 2] - tyaw) / PN_PI;
        float g[4];
        g[0] = 2.f * ex * w;
        g[1] = 2.f * ey * w;
        g[2] = 2.f * ea * yw * w;
        g[3] = (expf(o[4 * j + 3] - lse) - (j == jb ? 1.f : 0.f)) * inv_b;
        for (int q = 0; q < 4; ++q) {
            const int c = 4 * j + q;
            dOf[(size_t)b * ld + c] = g[q];
            const __nv_bfloat16 h = __float2bfloat16(g[q]);
            dO[(size_t)b * ld + c] = h;
            dOT[(size_t)c * B + b] = h;
        }
    }
}

// Adam on the f32 masters of every parameter tensor in one launch (weights and biases of all
// layers, concatenated), refreshing each weight's bf16 copy and bf16 transposed copy. The
// step count t comes from the device counter the step's sampling kernel advanced, so a
// captured training step replays without host updates.
struct AdamTable {
    float* w[2 * PN_MAX_LAYERS];
    const float* g[2 * PN_MAX_LAYERS];
    float* m[2 * PN_MAX_LAYERS];
    float* v[2 * PN_MAX_LAYERS];
    __nv_bfloat16* wb[2 * PN_MAX_LAYERS];
    __nv_bfloat16* wbt[2 * PN_MAX_LAYERS];
    int cols[2 * PN_MAX_LAYERS];   // C of a [R x C] weight (the transposed copy's index rule)
    int rows[2 * PN_MAX_LAYERS];
    uint64_t start[2 * PN_MAX_LAYERS + 1];
    int tensors;
};
// Four consecutive elements per thread (every tensor's size and start is a multiple of 4):
// 16-byte loads and stores of the f32 state, 8-byte stores of the bf16 copy. The bias
// corrections are formed once per block.
__global__ void k_adam_all(const AdamTable t, const uint64_t* __restrict__ step_ctr, float lr,
                           float b1, float b2, float eps) {
    __shared__ float s_c[2];
    if (threadIdx.x == 0) {
        const float step = (float)*step_ctr;
        s_c[0] = lr / (1.f - powf(b1, step));  // lr / (1 - b1^t)
        s_c[1] = 1.f / (1.f - powf(b2, step));  // 1 / (1 - b2^t)
    }
    __syncthreads();
    const uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4ull;
    if (i >= t.start[t.tensors]) return;
    int k = 0;
    while (i >= t.start[k + 1]) ++k;
    const size_t j = (size_t)(i - t.start[k]);
    const float lc1 = s_c[0], ic2 = s_c[1];
    const float4 g4 = *reinterpret_cast<const float4*>(t.g[k] + j);
    float4 m4 = *reinterpret_cast<const float4*>(t.m[k] + j);
    float4 v4 = *reinterpret_cast<const float4*>(t.v[k] + j);
    float4 w4 = *reinterpret_cast<const float4*>(t.w[k] + j);
    float* const gm[4] = {&m4.x, &m4.y, &m4.z, &m4.w};
    float* const gv[4] = {&v4.x, &v4.y, &v4.z, &v4.w};
    float* const gw[4] = {&w4.x, &w4.y, &w4.z, &w4.w};
    const float gg[4] = {g4.x, g4.y, g4.z, g4.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const float mi = b1 * *gm[q] + (1.f - b1) * gg[q];
        const float vi = b2 * *gv[q] + (1.f - b2) * gg[q] * gg[q];
        *gm[q] = mi;
        *gv[q] = vi;
        *gw[q] -= lc1 * mi / (sqrtf(vi * ic2) + eps);
    }
    *reinterpret_cast<float4*>(t.m[k] + j) = m4;
    *reinterpret_cast<float4*>(t.v[k] + j) = v4;
    *reinterpret_cast<float4*>(t.w[k] + j) = w4;
    if (t.wb[k]) {
        const __nv_bfloat162 h01 = __floats2bfloat162_rn(w4.x, w4.y);
        const __nv_bfloat162 h23 = __floats2bfloat162_rn(w4.z, w4.w);
        __nv_bfloat162* wb2 = reinterpret_cast<__nv_bfloat162*>(t.wb[k] + j);
        wb2[0] = h01;
        wb2[1] = h23;
        if (t.wbt[k]) {
            const int C = t.cols[k];
            const __nv_bfloat16 hs[4] = {h01.x, h01.y, h23.x, h23.y};
#pragma unroll
            for (int q = 0; q < 4; ++q)
                t.wbt[k][(size_t)((j + q) % C) * t.rows[k] + (j + q) / C] = hs[q];
        }
    }
}

__global__ void k_to_bf16(const float* __restrict__ w, size_t n, int C, int R,
                          __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wbt) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const __nv_bfloat16 h = __float2bfloat16(w[i]);
    wb[i] = h;
    if (wbt) wbt[(size_t)(i % C) * R + i / C] = h;
}

// ---- features ----------------------------------------------------------------------
// height image of a map: highest point per 1 m column (ordered-int atomicMax on f32)
__device__ __forceinline__ int f2ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

__global__ void k_height(const float* __restrict__ pts, size_t n, float ox, float oy, int W,
                         int H, int* __restrict__ img) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
    if (!(isfinite(x) && isfinite(y) && isfinite(z))) return;
    const int cx = (int)floorf(x - ox), cy = (int)floorf(y - oy);
    if (cx < 0 || cy < 0 || cx >= W || cy >= H) return;
    atomicMax(img + (size_t)cx * H + cy, f2ord(z));
}

struct PnMap {
    const int* img;  // ordered-int heights, INT_MIN-ish sentinel = empty
    float ox, oy;
    int W, H;
};
struct PnSample {       // one training / inference sample
    uint32_t scan;      // index into the scan table
    uint32_t map;
    float cx, cy, cz, cyaw;  // coarse pose (x, y, z, yaw)
};
struct PnScan {
    uint64_t offset;
    uint32_t n, map;
};

constexpr int EMPTY_ORD = (int)0x80808080;  // the memset byte 0x80: below every finite height

// scan grid + map crop of every sample into X [B x F] and XT [F x B] (both zeroed first)
__global__ void k_features(const float* __restrict__ scan_pts, const PnScan* __restrict__ scans,
                           const PnSample* __restrict__ smp, const PnMap* __restrict__ maps,
                           int B, int F, __nv_bfloat16* __restrict__ X,
                           __nv_bfloat16* __restrict__ XT) {
    const int b = blockIdx.y;
    if (b >= B) return;
    const PnSample s = smp[b];
    const PnScan sc = scans[s.scan];
    const __nv_bfloat16 one = __float2bfloat16(1.f);
    float sy, cy;
    sincosf(s.cyaw, &sy, &cy);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < sc.n; i += gridDim.x * blockDim.x) {
        const float* p = scan_pts + 3 * (sc.offset + i);
        const float px = p[0], py = p[1], pz = p[2];
        const float wx = cy * px - sy * py, wy = sy * px + cy * py;
        const int gx = (int)floorf(wx + 32.f), gy = (int)floorf(wy + 32.f), gz = (int)floorf(pz + 2.f);
        if (gx < 0 || gy < 0 || gz < 0 || gx >= PN_GRID || gy >= PN_GRID || gz >= PN_ZB) continue;
        const int f = (gx * PN_GRID + gy) * PN_ZB + gz;
        X[(size_t)b * F + f] = one;
        if (XT) XT[(size_t)f * B + b] = one;
    }
    const PnMap m = maps[s.map];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < PN_MAP_FEATS; c += gridDim.x * blockDim.x) {
        const int u = c / PN_GRID, v = c % PN_GRID;
        const float wx = s.cx - 32.f + (float)u + 0.5f, wy = s.cy - 32.f + (float)v + 0.5f;
        const int ix = (int)floorf(wx - m.ox), iy = (int)floorf(wy - m.oy);
        float val = 0.f;
        if (ix >= 0 && iy >= 0 && ix < m.W && iy < m.H) {
            const int hv = m.img[(size_t)ix * m.H + iy];
            if (hv != EMPTY_ORD) {
                const float h = ord2f(hv);
                val = 0.1f + fminf(fmaxf((h - s.cz + 2.f) / 10.f, 0.f), 0.9f);
            }
        }
        const __nv_bfloat16 h = __float2bfloat16(val);
        const int f = PN_SCAN_FEATS + c;
        X[(size_t)b * F + f] = h;
        if (XT) XT[(size_t)f * B + b] = h;
    }
}

// SplitMix64 on the device: training perturbations
__device__ __forceinline__ uint64_t sm64(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ float sm_unit(uint64_t& s) {
    return (float)(sm64(s) >> 40) * (1.f / 16777216.f);
}

__device__ __forceinline__ void sample_one(uint64_t seed, uint64_t step, int b,
                                           uint32_t n_scans, const PnScan* __restrict__ scans,
                                           const double* __restrict__ conv, float xy_range,
                                           PnSample* __restrict__ smp, float* __restrict__ T) {
    uint64_t s = seed ^ (0x9e3779b97f4a7c15ull * (step + 1)) ^ (0xd1b54a32d192ed03ull * (b + 1));
    sm64(s);
    const uint32_t k = (uint32_t)(sm64(s) % n_scans);
    const double* c = conv + 6 * (size_t)k;
    const float ex = (2.f * sm_unit(s) - 1.f) * xy_range, ey = (2.f * sm_unit(s) - 1.f) * xy_range;
    const float yaw = (2.f * sm_unit(s) - 1.f) * PN_PI;
    PnSample o;
    o.scan = k;
    o.map = scans[k].map;
    o.cx = (float)c[0] + ex;
    o.cy = (float)c[1] + ey;
    o.cz = (float)c[2];
    o.cyaw = yaw;
    smp[b] = o;
    T[3 * b] = -ex;
    T[3 * b + 1] = -ey;
    T[3 * b + 2] = wrap_pi((float)c[5] - yaw);
}


// training batch: random scan, coarse pose = converged pose + (U(+-r), U(+-r)), yaw uniform.
// One block: it reads the step counter, draws the batch of that step and advances the
// counter (the later kernels of the step read the new value as Adam's step count t).
__global__ void k_sample(uint64_t seed, uint64_t* __restrict__ step_ctr, int B,
                         uint32_t n_scans, const PnScan* __restrict__ scans,
                         const double* __restrict__ conv, float xy_range,
                         PnSample* __restrict__ smp, float* __restrict__ T) {
    __shared__ uint64_t s_step;
    if (threadIdx.x == 0) s_step = *step_ctr;
    __syncthreads();
    const uint64_t step = s_step;
    for (int b = threadIdx.x; b < B; b += blockDim.x)
        sample_one(seed, step, b, n_scans, scans, conv, xy_range, smp, T);
    __syncthreads();
    if (threadIdx.x == 0) *step_ctr = step + 1;
}
// proposals: pose = coarse + (4 o0, 4 o1, 0, 0, 0, pi o2), yaw wrapped; logits o3
__global__ void k_decode(const float* __restrict__ O, const PnSample* __restrict__ smp,
                         const double* __restrict__ coarse6, int B, int P,
                         double* __restrict__ poses, double* __restrict__ logits) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * P) return;
    const int b = i / P, j = i % P;
    const float* o = O + (size_t)b * P * PN_OUT_PER + 4 * j;
    const double* c = coarse6 + 6 * (size_t)b;
    double* p = poses + 6 * (size_t)i;
    p[0] = c[0] + PN_XY_SCALE * o[0];
    p[1] = c[1] + PN_XY_SCALE * o[1];
    p[2] = c[2];
    p[3] = c[3];
    p[4] = c[4];
    double yaw = c[5] + (double)(PN_PI * o[2]);
    yaw -= 6.283185307179586 * floor((yaw + 3.141592653589793) / 6.283185307179586);
    p[5] = yaw;
    logits[i] = o[3];
}

}  // namespace ndtgb

using namespace ndtgb;

// ------------------------------------------------------------------------------------
// Host object
// ------------------------------------------------------------------------------------
struct PnLayer {
    int in = 0, out = 0;
    DevBuf w, b, wb, wbt, mw, vw, mb, vb, gw, gb;
};

struct ndt_pnet {
    ndt_pnet_config cfg{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<PnLayer> L;
    // batch buffers (capacity cap_b samples)
    int cap_b = 0;
    std::vector<DevBuf> X, XT, Z, dZ, dZT, dZf;  // per layer
    DevBuf loss, T, smp, coarse, poses, logits, err;
    DevBuf Zp;              // split-K partial products
    DevBuf q_pts, q_scans;  // inference queries
    // data
    std::vector<PnMap> maps_h;
    std::vector<DevBuf> map_imgs;
    DevBuf maps_d;
    std::vector<float> scan_pts_h;
    std::vector<PnScan> scans_h;
    std::vector<double> conv_h;
    DevBuf scan_pts_d, scans_d, conv_d;
    bool data_dirty = true;
    uint64_t step = 0;
    PinBuf h_loss;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // CUDA-event timing on the network's stream
    ndt_pnet_stats stats{};
    DevBuf step_ctr;                    // Adam step count on the device (advanced by k_sample)
    cudaGraphExec_t train_exec = nullptr;  // one captured training step, replayed
};

static uint64_t host_sm64(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static int pn_check(ndt_pnet* p, const char* what) {
    uint32_t h = 0;
    cudaMemcpyAsync(&h, p->err.p, 4, cudaMemcpyDeviceToHost, p->stream);
    int rc = cuda_fail(cudaStreamSynchronize(p->stream), what);
    if (rc) return rc;
    if (h) {
        set_error(std::string(what) + ": a GEMM pipeline wait timed out (code " +
                  std::to_string(h) + ")");
        return NDT_ERR_DEVICE;
    }
    return 0;
}

static int pn_reserve_batch(ndt_pnet* p, int B) {
    if (B <= p->cap_b) return 0;
    const int nl = (int)p->L.size();
    p->X.resize(nl + 1);
    p->XT.resize(nl + 1);
    p->Z.resize(nl);
    p->dZ.resize(nl);
    p->dZT.resize(nl);
    p->dZf.resize(nl);
    int rc;
    for (int l = 0; l < nl; ++l) {
        const size_t in = p->L[l].in, out = p->L[l].out;
        if ((rc = dev_reserve(p->X[l], (size_t)B * in * 2)) ||
            (rc = dev_reserve(p->XT[l], (size_t)B * in * 2)) ||
            (rc = dev_reserve(p->Z[l], (size_t)B * out * 4)) ||
            (rc = dev_reserve(p->dZ[l], (size_t)B * out * 2)) ||
            (rc = dev_reserve(p->dZT[l], (size_t)B * out * 2)) ||
            (rc = dev_reserve(p->dZf[l], (size_t)B * out * 4)))
            return rc;
    }
    const size_t no = (size_t)p->cfg.proposals * PN_OUT_PER;
    size_t max_out = 0;
    for (auto& L : p->L) max_out = std::max(max_out, (size_t)L.out);
    if ((rc = dev_reserve(p->Zp, (size_t)PN_MAX_SPLITS * B * max_out * 4))) return rc;
    if ((rc = dev_reserve(p->loss, (size_t)B * 4)) || (rc = dev_reserve(p->T, (size_t)B * 12)) ||
        (rc = dev_reserve(p->smp, (size_t)B * sizeof(PnSample))) ||
        (rc = dev_reserve(p->coarse, (size_t)B * 48)) ||
        (rc = dev_reserve(p->poses, (size_t)B * no / PN_OUT_PER * 48)) ||
        (rc = dev_reserve(p->logits, (size_t)B * no / PN_OUT_PER * 8)) ||
        (rc = pin_reserve(p->h_loss, (size_t)B * 4)))
        return rc;
    p->cap_b = B;
    return 0;
}

static int pn_upload_data(ndt_pnet* p) {
    if (!p->data_dirty) return 0;
    // the captured training step holds the data buffers' addresses, which may move here
    if (p->train_exec) {
        cudaGraphExecDestroy(p->train_exec);
        p->train_exec = nullptr;
    }
    int rc;
    if ((rc = dev_reserve(p->maps_d, std::max<size_t>(1, p->maps_h.size()) * sizeof(PnMap))) ||
        (rc = dev_reserve(p->scan_pts_d, std::max<size_t>(1, p->scan_pts_h.size()) * 4)) ||
        (rc = dev_reserve(p->scans_d, std::max<size_t>(1, p->scans_h.size()) * sizeof(PnScan))) ||
        (rc = dev_reserve(p->conv_d, std::max<size_t>(1, p->conv_h.size()) * 8)))
        return rc;
    cudaStream_t s = p->stream;
    if (!p->maps_h.empty())
        cudaMemcpyAsync(p->maps_d.p, p->maps_h.data(), p->maps_h.size() * sizeof(PnMap),
                        cudaMemcpyHostToDevice, s);
    if (!p->scan_pts_h.empty())
        cudaMemcpyAsync(p->scan_pts_d.p, p->scan_pts_h.data(), p->scan_pts_h.size() * 4,
                        cudaMemcpyHostToDevice, s);
    if (!p->scans_h.empty())
        cudaMemcpyAsync(p->scans_d.p, p->scans_h.data(), p->scans_h.size() * sizeof(PnScan),
                        cudaMemcpyHostToDevice, s);
    if (!p->conv_h.empty())
        cudaMemcpyAsync(p->conv_d.p, p->conv_h.data(), p->conv_h.size() * 8,
                        cudaMemcpyHostToDevice, s);
    p->data_dirty = false;
    return cuda_fail(cudaStreamSynchronize(s), "proposal data upload");
}

static inline unsigned blocks(size_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

// forward over X[0] (already filled) for B samples; leaves the biased output in Z[last].
// Layers after the first add their bias and activation in the GEMM's epilogue, which also
// writes the next layer's bf16 input (and, for training, its transposed copy). The input
// layer's long K is split so every SM streams a share of the operands; its partial products
// are summed by k_bias_act.
static int pn_forward(ndt_pnet* p, int B, bool need_t) {
    const int nl = (int)p->L.size();
    cudaStream_t s = p->stream;
    int rc;
    for (int l = 0; l < nl; ++l) {
        PnLayer& L = p->L[l];
        const bool last = l == nl - 1;
        const int tiles = ((B + 127) / 128) * ((L.out + 127) / 128);
        int splits = 1;
        if (tiles < 64 && L.in >= 4096) splits = std::min(PN_MAX_SPLITS, L.in / 64 / 8);
        if (splits > 1) {
            if ((rc = gemm_bf16_tn(p->X[l].p, L.wb.p, (float*)p->Zp.p, B, L.out, L.in, L.out,
                                   (uint32_t*)p->err.p, s, splits, nullptr)))
                return rc;
            k_bias_act<<<blocks((size_t)B * L.out), 256, 0, s>>>(
                (float*)p->Z[l].p, (const float*)p->Zp.p, splits, (const float*)L.b.p, B, L.out,
                last ? 1 : 0, last ? nullptr : (__nv_bfloat16*)p->X[l + 1].p,
                last || !need_t ? nullptr : (__nv_bfloat16*)p->XT[l + 1].p);
            continue;
        }
        GemmEpilogue e{};
        e.mode = last ? GEMM_EPI_BIAS : GEMM_EPI_BIAS_GELU;
        e.bias = (const float*)L.b.p;
        e.x = last ? nullptr : (__nv_bfloat16*)p->X[l + 1].p;
        e.xt = last || !need_t ? nullptr : (__nv_bfloat16*)p->XT[l + 1].p;
        if ((rc = gemm_bf16_tn(p->X[l].p, L.wb.p, (float*)p->Z[l].p, B, L.out, L.in, L.out,
                               (uint32_t*)p->err.p, s, 1, &e)))
            return rc;
    }
    return cuda_fail(cudaGetLastError(), "proposal forward");
}

// backward from the loss gradient in dZ*[last]; fills every layer's gw, gb. The input
// gradient's GEMM applies GELU' of the layer below in its epilogue and writes that layer's
// output gradient in f32 and in both bf16 layouts; the bias gradients are one launch.
static int pn_backward(ndt_pnet* p, int B) {
    const int nl = (int)p->L.size();
    cudaStream_t s = p->stream;
    int rc;
    ColsumTable ct{};
    ct.layers = nl;
    ct.start[0] = 0;
    for (int l = nl - 1; l >= 0; --l) {
        PnLayer& L = p->L[l];
        // dW = dZ^T X  (A = dZ^T [out x B], B-operand = X^T [in x B])
        if ((rc = gemm_bf16_tn(p->dZT[l].p, p->XT[l].p, (float*)L.gw.p, L.out, L.in, B, L.in,
                               (uint32_t*)p->err.p, s, 1, nullptr)))
            return rc;
        if (l > 0) {
            // dX = dZ W  (A = dZ [B x out], B-operand = W^T [in x out]), then * GELU'(Z_{l-1})
            GemmEpilogue e{};
            e.mode = GEMM_EPI_GELU_BACK;
            e.zin = (const float*)p->Z[l - 1].p;
            e.x = (__nv_bfloat16*)p->dZ[l - 1].p;
            e.xt = (__nv_bfloat16*)p->dZT[l - 1].p;
            if ((rc = gemm_bf16_tn(p->dZ[l].p, L.wbt.p, (float*)p->dZf[l - 1].p, B, L.in, L.out,
                                   L.in, (uint32_t*)p->err.p, s, 1, &e)))
                return rc;
        }
    }
    for (int l = 0; l < nl; ++l) {
        ct.g[l] = (const float*)p->dZf[l].p;
        ct.out[l] = (float*)p->L[l].gb.p;
        ct.n[l] = p->L[l].out;
        ct.start[l + 1] = ct.start[l] + p->L[l].out;
    }
    k_colsum_all<<<(unsigned)((ct.start[nl] + 31) / 32), 32 * PN_CS_ROWS, 0, s>>>(ct, B);
    return cuda_fail(cudaGetLastError(), "proposal backward");
}

static int pn_loss(ndt_pnet* p, int B) {
    const int nl = (int)p->L.size();
    k_loss<<<blocks(B, 128), 128, 0, p->stream>>>(
        (const float*)p->Z[nl - 1].p, (const float*)p->T.p, B, p->cfg.proposals,
        p->cfg.yaw_weight, (float*)p->loss.p, (float*)p->dZf[nl - 1].p,
        (__nv_bfloat16*)p->dZ[nl - 1].p,
        (__nv_bfloat16*)p->dZT[nl - 1].p);
    return cuda_fail(cudaGetLastError(), "proposal loss");
}

// Adam over every parameter tensor in one launch; the step count is the device counter
static int pn_adam(ndt_pnet* p) {
    AdamTable t{};
    int k = 0;
    t.start[0] = 0;
    for (size_t l = 0; l < p->L.size(); ++l) {
        PnLayer& L = p->L[l];
        const size_t nw = (size_t)L.in * L.out;
        t.w[k] = (float*)L.w.p;
        t.g[k] = (const float*)L.gw.p;
        t.m[k] = (float*)L.mw.p;
        t.v[k] = (float*)L.vw.p;
        t.wb[k] = (__nv_bfloat16*)L.wb.p;
        t.wbt[k] = l > 0 ? (__nv_bfloat16*)L.wbt.p : nullptr;
        t.cols[k] = L.in;
        t.rows[k] = L.out;
        t.start[k + 1] = t.start[k] + nw;
        ++k;
        t.w[k] = (float*)L.b.p;
        t.g[k] = (const float*)L.gb.p;
        t.m[k] = (float*)L.mb.p;
        t.v[k] = (float*)L.vb.p;
        t.wb[k] = nullptr;
        t.wbt[k] = nullptr;
        t.cols[k] = L.out;
        t.rows[k] = 1;
        t.start[k + 1] = t.start[k] + (uint64_t)L.out;
        ++k;
    }
    t.tensors = k;
    k_adam_all<<<blocks((t.start[k] + 3) / 4), 256, 0, p->stream>>>(
        t, (const uint64_t*)p->step_ctr.p, p->cfg.learning_rate, 0.9f, 0.999f, 1e-8f);
    return cuda_fail(cudaGetLastError(), "proposal update");
}

// input features of B samples into X[0] (and, for training, the transposed copy XT[0])
static int pn_features(ndt_pnet* p, int B, const void* pts, const void* scans, bool need_t) {
    const size_t F = (size_t)p->L[0].in;
    cudaMemsetAsync(p->X[0].p, 0, (size_t)B * F * 2, p->stream);
    if (need_t) cudaMemsetAsync(p->XT[0].p, 0, (size_t)B * F * 2, p->stream);
    k_features<<<dim3(8, B), 256, 0, p->stream>>>(
        (const float*)pts, (const PnScan*)scans, (const PnSample*)p->smp.p,
        (const PnMap*)p->maps_d.p, B, (int)F, (__nv_bfloat16*)p->X[0].p,
        need_t ? (__nv_bfloat16*)p->XT[0].p : nullptr);
    return cuda_fail(cudaGetLastError(), "proposal features");
}

// One training step on the network's stream: sample a batch (advancing the device step
// counter), features, forward, loss, backward, Adam. Stream-ordered only, so it can be
// captured into a graph.
static int pn_train_step(ndt_pnet* p, int B) {
    cudaStream_t s = p->stream;
    k_sample<<<1, 256, 0, s>>>(p->cfg.seed, (uint64_t*)p->step_ctr.p, B,
                               (uint32_t)p->scans_h.size(), (const PnScan*)p->scans_d.p,
                               (const double*)p->conv_d.p, p->cfg.xy_range, (PnSample*)p->smp.p,
                               (float*)p->T.p);
    int rc;
    if ((rc = pn_features(p, B, p->scan_pts_d.p, p->scans_d.p, true)) ||
        (rc = pn_forward(p, B, true)) || (rc = pn_loss(p, B)) || (rc = pn_backward(p, B)) ||
        (rc = pn_adam(p)))
        return rc;
    return 0;
}

extern "C" {

int ndt_pnet_config_default(ndt_pnet_config* c) {
    if (!c) return NDT_ERR_INVALID_ARGUMENT;
    std::memset(c, 0, sizeof *c);
    c->input_dim = PN_SCAN_FEATS + PN_MAP_FEATS;
    c->hidden = 512;
    c->hidden_layers = 4;
    c->proposals = 16;
    c->batch = 256;
    c->train_batch = 1024;
    c->learning_rate = 3e-4f;
    c->xy_range = 5.0f;
    c->yaw_weight = 8.0f;
    c->seed = 1;
    return NDT_OK;
}

int ndt_pnet_create(const ndt_pnet_config* cfg, int32_t device, ndt_pnet** out) {
    if (!out) return NDT_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    ndt_pnet_config c;
    if (cfg)
        c = *cfg;
    else
        ndt_pnet_config_default(&c);
    const int no = c.proposals * PN_OUT_PER;
    if (c.input_dim <= 0 || c.input_dim % 64 || c.hidden <= 0 || c.hidden % 64 ||
        c.hidden_layers < 1 || c.hidden_layers + 1 > PN_MAX_LAYERS || c.proposals < 1 ||
        no % 64 || c.batch < 1 || c.batch % 64 || c.train_batch < 0 || c.train_batch % 64 ||
        !(c.learning_rate > 0.f)) {
        set_error("proposal network: input_dim, hidden, 4 * proposals, batch and train_batch "
                  "must be positive multiples of 64");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    if (c.train_batch == 0) c.train_batch = c.batch;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device) {
        set_error("no CUDA device available");
        return NDT_ERR_NO_DEVICE;
    }
    cudaSetDevice(device);
    ndt_pnet* p = new ndt_pnet();
    p->cfg = c;
    p->device = device;
    cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    cudaEventCreate(&p->ev0);
    cudaEventCreate(&p->ev1);
    int rc = dev_reserve(p->err, 16);
    if (!rc) cudaMemsetAsync(p->err.p, 0, 16, p->stream);
    if (!rc && !(rc = dev_reserve(p->step_ctr, 8))) cudaMemsetAsync(p->step_ctr.p, 0, 8, p->stream);
    // layers: input -> hidden x hidden_layers -> 4 * proposals; weights N(0, 2 / in)
    std::vector<int> dims = {c.input_dim};
    for (int i = 0; i < c.hidden_layers; ++i) dims.push_back(c.hidden);
    dims.push_back(no);
    p->L.resize(dims.size() - 1);
    uint64_t s = c.seed;
    for (size_t l = 0; l + 1 < dims.size() && !rc; ++l) {
        PnLayer& L = p->L[l];
        L.in = dims[l];
        L.out = dims[l + 1];
        const size_t nw = (size_t)L.in * L.out;
        if ((rc = dev_reserve(L.w, nw * 4)) || (rc = dev_reserve(L.b, L.out * 4)) ||
            (rc = dev_reserve(L.wb, nw * 2)) || (rc = dev_reserve(L.wbt, nw * 2)) ||
            (rc = dev_reserve(L.mw, nw * 4)) || (rc = dev_reserve(L.vw, nw * 4)) ||
            (rc = dev_reserve(L.mb, L.out * 4)) || (rc = dev_reserve(L.vb, L.out * 4)) ||
            (rc = dev_reserve(L.gw, nw * 4)) || (rc = dev_reserve(L.gb, L.out * 4)))
            break;
        std::vector<float> w(nw);
        const double sd = std::sqrt(2.0 / L.in) * (l + 2 == dims.size() ? 0.1 : 1.0);
        for (size_t i = 0; i < nw; i += 2) {  // Box-Muller pairs
            const double u1 = 1.0 - (double)(host_sm64(s) >> 11) * 0x1.0p-53;
            const double u2 = (double)(host_sm64(s) >> 11) * 0x1.0p-53;
            const double r = std::sqrt(-2.0 * std::log(u1)) * sd;
            w[i] = (float)(r * std::cos(6.283185307179586 * u2));
            if (i + 1 < nw) w[i + 1] = (float)(r * std::sin(6.283185307179586 * u2));
        }
        cudaMemcpyAsync(L.w.p, w.data(), nw * 4, cudaMemcpyHostToDevice, p->stream);
        cudaMemsetAsync(L.b.p, 0, L.out * 4, p->stream);
        cudaMemsetAsync(L.mw.p, 0, nw * 4, p->stream);
        cudaMemsetAsync(L.vw.p, 0, nw * 4, p->stream);
        cudaMemsetAsync(L.mb.p, 0, L.out * 4, p->stream);
        cudaMemsetAsync(L.vb.p, 0, L.out * 4, p->stream);
        k_to_bf16<<<blocks(nw), 256, 0, p->stream>>>((const float*)L.w.p, nw, L.in, L.out,
                                                     (__nv_bfloat16*)L.wb.p,
                                                     (__nv_bfloat16*)L.wbt.p);
        rc = cuda_fail(cudaStreamSynchronize(p->stream), "proposal network init");
    }
    if (!rc) rc = pn_reserve_batch(p, std::max(c.batch, c.train_batch));
    if (rc) {
        ndt_pnet_destroy(p);
        return rc;
    }
    *out = p;
    return NDT_OK;
}

int ndt_pnet_get_config(ndt_pnet* p, ndt_pnet_config* out) {
    if (!p || !out) return NDT_ERR_INVALID_ARGUMENT;
    *out = p->cfg;
    return NDT_OK;
}

int ndt_pnet_destroy(ndt_pnet* p) {
    if (!p) return NDT_OK;
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (auto& L : p->L)
        for (DevBuf* b : {&L.w, &L.b, &L.wb, &L.wbt, &L.mw, &L.vw, &L.mb, &L.vb, &L.gw, &L.gb})
            dev_free(*b);
    for (auto* v : {&p->X, &p->XT, &p->Z, &p->dZ, &p->dZT, &p->dZf})
        for (auto& b : *v) dev_free(b);
    for (auto& b : p->map_imgs) dev_free(b);
    for (DevBuf* b : {&p->loss, &p->T, &p->smp, &p->coarse, &p->poses, &p->logits, &p->err,
                      &p->q_pts, &p->q_scans, &p->Zp, &p->maps_d, &p->scan_pts_d, &p->scans_d,
                      &p->conv_d})
        dev_free(*b);
    pin_free(p->h_loss);
    if (p->train_exec) cudaGraphExecDestroy(p->train_exec);
    dev_free(p->step_ctr);
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
    return NDT_OK;
}

int ndt_pnet_add_map(ndt_pnet* p, const float* xyz, uint64_t n, int32_t* map_id) {
    if (!p || !map_id || (n && !xyz)) return NDT_ERR_INVALID_ARGUMENT;
    if (n == 0) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    float lo[2] = {INFINITY, INFINITY}, hi[2] = {-INFINITY, -INFINITY};
    for (uint64_t i = 0; i < n; ++i)
        for (int a = 0; a < 2; ++a) {
            const float v = xyz[3 * i + a];
            if (std::isfinite(v)) {
                lo[a] = std::min(lo[a], v);
                hi[a] = std::max(hi[a], v);
            }
        }
    if (!(lo[0] <= hi[0])) {
        set_error("Target point cloud is empty");
        return NDT_ERR_EMPTY_INPUT;
    }
    PnMap m;
    m.ox = std::floor(lo[0]);
    m.oy = std::floor(lo[1]);
    m.W = (int)std::floor(hi[0] - m.ox) + 1;
    m.H = (int)std::floor(hi[1] - m.oy) + 1;
    if ((uint64_t)m.W * (uint64_t)m.H > (1ull << 28)) {
        set_error("map footprint exceeds 2^28 one-metre columns");
        return NDT_ERR_CAPACITY;
    }
    cudaSetDevice(p->device);
    DevBuf img, pts;
    int rc;
    if ((rc = dev_reserve(img, (size_t)m.W * m.H * 4)) || (rc = dev_reserve(pts, n * 12)))
        return rc;
    cudaMemsetAsync(img.p, 0x80, (size_t)m.W * m.H * 4, p->stream);  // 0x80808080 < any f2ord
    cudaMemcpyAsync(pts.p, xyz, n * 12, cudaMemcpyHostToDevice, p->stream);
    k_height<<<blocks(n), 256, 0, p->stream>>>((const float*)pts.p, n, m.ox, m.oy, m.W, m.H,
                                                (int*)img.p);
    rc = cuda_fail(cudaStreamSynchronize(p->stream), "height image");
    dev_free(pts);
    if (rc) {
        dev_free(img);
        return rc;
    }
    m.img = (const int*)img.p;
    p->map_imgs.push_back(img);
    p->maps_h.push_back(m);
    p->data_dirty = true;
    *map_id = (int32_t)(p->maps_h.size() - 1);
    return NDT_OK;
}

int ndt_pnet_add_scan(ndt_pnet* p, int32_t map_id, const float* xyz, uint64_t n,
                      const double pose[6], int32_t* scan_id) {
    if (!p || !pose || (n && !xyz) || map_id < 0 || map_id >= (int32_t)p->maps_h.size())
        return NDT_ERR_INVALID_ARGUMENT;
    if (n == 0 || n > 0xFFFFFFF0ull) {
        set_error("scan must hold 1 .. 2^32 points");
        return NDT_ERR_EMPTY_INPUT;
    }
    PnScan sc;
    sc.offset = p->scan_pts_h.size() / 3;
    sc.n = (uint32_t)n;
    sc.map = (uint32_t)map_id;
    p->scan_pts_h.insert(p->scan_pts_h.end(), xyz, xyz + 3 * n);
    p->scans_h.push_back(sc);
    p->conv_h.insert(p->conv_h.end(), pose, pose + 6);
    p->data_dirty = true;
    if (scan_id) *scan_id = (int32_t)(p->scans_h.size() - 1);
    return NDT_OK;
}

int ndt_pnet_train(ndt_pnet* p, uint64_t steps, float* loss_out) {
    if (!p) return NDT_ERR_INVALID_ARGUMENT;
    if (p->scans_h.empty()) {
        set_error("proposal network: no training scans");
        return NDT_ERR_EMPTY_INPUT;
    }
    cudaSetDevice(p->device);
    int rc = pn_upload_data(p);
    if (rc) return rc;
    const int B = p->cfg.train_batch;
    cudaStream_t s = p->stream;
    cudaEventRecord(p->ev0, s);
    for (uint64_t it = 0; it < steps; ++it) {
        if (p->train_exec) {
            rc = cuda_fail(cudaGraphLaunch(p->train_exec, s), "proposal training step");
        } else {
            // the first step runs eagerly (kernel attributes, launch checks); the step is
            // then captured once and replayed: every step reads its step count from the
            // device counter, so the replays need no host updates
            if ((rc = pn_train_step(p, B)) || (rc = pn_check(p, "proposal training"))) return rc;
            cudaGraph_t g = nullptr;
            cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                const int rc_cap = pn_train_step(p, B);
                e = cudaStreamEndCapture(s, &g);
                if (rc_cap) {
                    if (g) cudaGraphDestroy(g);
                    return rc_cap;
                }
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&p->train_exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if ((rc = cuda_fail(e, "proposal training step capture"))) return rc;
        }
        if (rc) return rc;
        p->step++;
        if (loss_out) {
            cudaMemcpyAsync(p->h_loss.p, p->loss.p, (size_t)B * 4, cudaMemcpyDeviceToHost, s);
            if ((rc = pn_check(p, "proposal training"))) return rc;
            double acc = 0.0;
            for (int b = 0; b < B; ++b) acc += ((float*)p->h_loss.p)[b];
            loss_out[it] = (float)(acc / B);
        }
    }
    cudaEventRecord(p->ev1, s);
    if ((rc = pn_check(p, "proposal training"))) return rc;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p->ev0, p->ev1) == cudaSuccess) p->stats.train_ms += ms;
    p->stats.train_steps += steps;
    return NDT_OK;
}

int ndt_pnet_propose(ndt_pnet* p, int32_t map_id, const ndt_scan* q, uint64_t nq,
                     double* poses, double* logits) {
    if (!p || (nq && (!q || !poses)) || map_id < 0 || map_id >= (int32_t)p->maps_h.size())
        return NDT_ERR_INVALID_ARGUMENT;
    if (nq == 0) return NDT_OK;
    cudaSetDevice(p->device);
    const int P = p->cfg.proposals;
    cudaStream_t s = p->stream;
    std::vector<PnSample> smp(nq);
    std::vector<PnScan> sc(nq);
    std::vector<double> coarse(6 * nq);
    uint64_t total = 0;
    for (uint64_t i = 0; i < nq; ++i) {
        if (!q[i].xyz || q[i].num_points == 0 || q[i].num_points > 0xFFFFFFF0ull) {
            set_error("Source point cloud is empty");
            return NDT_ERR_EMPTY_INPUT;
        }
        sc[i].offset = total;
        sc[i].n = (uint32_t)q[i].num_points;
        sc[i].map = (uint32_t)map_id;
        total += q[i].num_points;
        smp[i].scan = (uint32_t)i;
        smp[i].map = (uint32_t)map_id;
        smp[i].cx = (float)q[i].initial_pose[0];
        smp[i].cy = (float)q[i].initial_pose[1];
        smp[i].cz = (float)q[i].initial_pose[2];
        smp[i].cyaw = (float)q[i].initial_pose[5];
        for (int k = 0; k < 6; ++k) coarse[6 * i + k] = q[i].initial_pose[k];
    }
    int rc;
    if ((rc = pn_upload_data(p)) || (rc = dev_reserve(p->q_pts, total * 12)) ||
        (rc = dev_reserve(p->q_scans, nq * sizeof(PnScan))))
        return rc;
    for (uint64_t i = 0; i < nq; ++i)
        cudaMemcpyAsync((char*)p->q_pts.p + sc[i].offset * 12, q[i].xyz, q[i].num_points * 12,
                        cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(p->q_scans.p, sc.data(), nq * sizeof(PnScan), cudaMemcpyHostToDevice, s);
    for (uint64_t b0 = 0; b0 < nq && !rc; b0 += (uint64_t)p->cfg.batch) {
        const int B = (int)std::min<uint64_t>(nq - b0, (uint64_t)p->cfg.batch);
        cudaMemcpyAsync(p->smp.p, smp.data() + b0, B * sizeof(PnSample), cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(p->coarse.p, coarse.data() + 6 * b0, B * 48, cudaMemcpyHostToDevice, s);
        cudaEventRecord(p->ev0, s);
        if ((rc = pn_features(p, B, p->q_pts.p, p->q_scans.p, false)) ||
            (rc = pn_forward(p, B, false)))
            break;
        k_decode<<<blocks((size_t)B * P), 256, 0, s>>>(
            (const float*)p->Z[p->L.size() - 1].p, (const PnSample*)p->smp.p,
            (const double*)p->coarse.p, B, P, (double*)p->poses.p, (double*)p->logits.p);
        cudaEventRecord(p->ev1, s);
        cudaMemcpyAsync(poses + 6 * P * b0, p->poses.p, (size_t)B * P * 48, cudaMemcpyDeviceToHost, s);
        if (logits)
            cudaMemcpyAsync(logits + P * b0, p->logits.p, (size_t)B * P * 8,
                            cudaMemcpyDeviceToHost, s);
        rc = pn_check(p, "proposal inference");
        float ms = 0.f;
        if (!rc && cudaEventElapsedTime(&ms, p->ev0, p->ev1) == cudaSuccess)
            p->stats.inference_kernel_ms += ms;
        p->stats.inference_batches++;
    }
    if (!rc) p->stats.queries += nq;
    return rc;
}

int ndt_pnet_stats_get(ndt_pnet* p, ndt_pnet_stats* out) {
    if (!p || !out) return NDT_ERR_INVALID_ARGUMENT;
    *out = p->stats;
    return NDT_OK;
}

// One forward + backward on caller-given inputs (no features, no update): the loss and every
// parameter's gradient, for checking the kernels against an FP64 restatement.
int ndt_pnet_debug_grad(ndt_pnet* p, const float* x, const float* targets, uint64_t b,
                        float* loss, float* grads) {
    if (!p || !x || !targets || !loss || !grads || b == 0 || b > (uint64_t)p->cfg.batch)
        return NDT_ERR_INVALID_ARGUMENT;
    cudaSetDevice(p->device);
    const int B = (int)b;
    const size_t F = (size_t)p->L[0].in;
    cudaStream_t s = p->stream;
    std::vector<uint16_t> xb(B * F), xt(B * F);
    for (int i = 0; i < B; ++i)
        for (size_t f = 0; f < F; ++f) {
            float v = x[(size_t)i * F + f];
            uint32_t u;
            std::memcpy(&u, &v, 4);
            u += 0x7FFFu + ((u >> 16) & 1u);  // round to nearest even
            const uint16_t h = (uint16_t)(u >> 16);
            xb[(size_t)i * F + f] = h;
            xt[f * B + i] = h;
        }
    cudaMemcpyAsync(p->X[0].p, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(p->XT[0].p, xt.data(), xt.size() * 2, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(p->T.p, targets, (size_t)B * 12, cudaMemcpyHostToDevice, s);
    int rc;
    if ((rc = pn_forward(p, B, true)) || (rc = pn_loss(p, B)) || (rc = pn_backward(p, B)))
        return rc;
    std::vector<float> lb(B);
    cudaMemcpyAsync(lb.data(), p->loss.p, (size_t)B * 4, cudaMemcpyDeviceToHost, s);
    size_t off = 0;
    for (auto& L : p->L) {
        const size_t nw = (size_t)L.in * L.out;
        cudaMemcpyAsync(grads + off, L.gw.p, nw * 4, cudaMemcpyDeviceToHost, s);
        off += nw;
        cudaMemcpyAsync(grads + off, L.gb.p, L.out * 4, cudaMemcpyDeviceToHost, s);
        off += L.out;
    }
    if ((rc = pn_check(p, "proposal gradient"))) return rc;
    double acc = 0.0;
    for (float v : lb) acc += v;
    *loss = (float)(acc / B);
    return NDT_OK;
}

// Parameters (f32 masters), layer by layer: W [out x in] row-major, then b [out].
int ndt_pnet_params(ndt_pnet* p, float* out, uint64_t* count, int32_t set) {
    if (!p || !count) return NDT_ERR_INVALID_ARGUMENT;
    uint64_t n = 0;
    for (auto& L : p->L) n += (uint64_t)L.in * L.out + L.out;
    if (!out) {
        *count = n;
        return NDT_OK;
    }
    if (*count < n) return NDT_ERR_INVALID_ARGUMENT;
    cudaSetDevice(p->device);
    size_t off = 0;
    for (size_t l = 0; l < p->L.size(); ++l) {
        PnLayer& L = p->L[l];
        const size_t nw = (size_t)L.in * L.out;
        if (set) {
            cudaMemcpyAsync(L.w.p, out + off, nw * 4, cudaMemcpyHostToDevice, p->stream);
            cudaMemcpyAsync(L.b.p, out + off + nw, L.out * 4, cudaMemcpyHostToDevice, p->stream);
            k_to_bf16<<<blocks(nw), 256, 0, p->stream>>>(
                (const float*)L.w.p, nw, L.in, L.out, (__nv_bfloat16*)L.wb.p,
                (__nv_bfloat16*)L.wbt.p);
        } else {
            cudaMemcpyAsync(out + off, L.w.p, nw * 4, cudaMemcpyDeviceToHost, p->stream);
            cudaMemcpyAsync(out + off + nw, L.b.p, L.out * 4, cudaMemcpyDeviceToHost, p->stream);
        }
        off += nw + L.out;
    }
    *count = n;
    return cuda_fail(cudaStreamSynchronize(p->stream), "proposal parameters");
}

}  // extern "C"
