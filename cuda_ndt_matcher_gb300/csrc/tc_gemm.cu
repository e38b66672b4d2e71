// tc_gemm.cu — BF16 GEMM on the 5th-generation tensor cores of sm_103a (tcgen05 + TMA).
//
//   D[M x N] (f32) = A[M x K] * B[N x K]^T      A, B bf16, row-major, K contiguous
//
// Both operands are K-major, so every product of the proposal network is this one form:
// the host keeps transposed copies where a product needs them (W^T for the input
// gradients, X^T and dY^T for the weight gradients).
//
// One CTA computes a 128 x 128 tile of D with 128 threads:
//   warp 0, lane 0  TMA producer: 128 x 64 bf16 boxes of A and B (128-byte swizzle) into a
//                   4-stage shared-memory ring, completion counted on a "full" mbarrier;
//   warp 1, lane 0  MMA issuer: per stage four tcgen05.mma.kind::f16 (M 128, N 128, K 16)
//                   into a 128-column f32 accumulator in tensor memory; tcgen05.commit
//                   arrives on the stage's "empty" mbarrier when those MMAs are done;
//   warps 0-3       epilogue: tcgen05.ld of their 32 accumulator rows, f32 stores, and
//                   optionally the network's elementwise step fused in (GemmEpilogue): bias
//                   + GELU (or identity) with the activation stored as bf16 in both layouts,
//                   or the GELU derivative of the backward pass.
// Every mbarrier wait is bounded (about one second of the global timer); on timeout the CTA
// records an error code in *err, stops issuing work and frees its tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include "ndt_internal.h"

namespace ndtgb {

__device__ __forceinline__ float gelu_tanh(float z) {  // tanh approximation of GELU
    const float k = 0.7978845608f;                      // sqrt(2 / pi)
    const float u = k * (z + 0.044715f * z * z * z);
    return 0.5f * z * (1.f + tanhf(u));
}
__device__ __forceinline__ float gelu_tanh_grad(float z) {
    const float k = 0.7978845608f;
    const float u = k * (z + 0.044715f * z * z * z);
    const float t = tanhf(u);
    return 0.5f * (1.f + t) + 0.5f * z * (1.f - t * t) * k * (1.f + 3.f * 0.044715f * z * z);
}


constexpr int GB_M = 128, GB_N = 128, GB_K = 64, GB_STAGES = 4;
constexpr int GB_TILE_BYTES = GB_M * GB_K * 2;          // 16 KB per operand box
constexpr int GB_STAGE_BYTES = 2 * GB_TILE_BYTES;
constexpr int GB_SMEM = GB_STAGES * GB_STAGE_BYTES + 1024;  // + alignment slack
constexpr uint64_t GB_WAIT_NS = 1000000000ull;          // bounded waits: 1 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t gb_now() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait for the given phase parity of an mbarrier; false (and *err |= code) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t* err,
                                          uint32_t code) {
    const uint32_t a = smem_u32(bar);
    const uint64_t t0 = gb_now();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (gb_now() - t0 > GB_WAIT_NS) {
            atomicOr(err, code);
            return false;
        }
    }
}

// K-major operand tile in shared memory, 128-byte swizzle (the layout a TMA box of 64 bf16
// columns with CU_TENSOR_MAP_SWIZZLE_128B writes): rows of 128 B in 8-row, 1024-byte atoms.
// Descriptor fields: start address >> 4 (bits 0-13), leading-dimension offset >> 4 (16-29;
// unused by swizzled K-major layouts), stride-dimension offset >> 4 (32-45: 1024 B between
// 8-row groups), descriptor version 1 (46-47), base offset 0 (49-51: atoms 1024-B aligned),
// layout type 2 = 128-byte swizzle (61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)1 << 16) |
           ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// Instruction descriptor of tcgen05.mma.kind::f16: D f32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 (bits 17-22),
// M >> 4 (bits 24-28).
__host__ __device__ constexpr uint32_t mma_idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

// Fused epilogue of 32 accumulator columns [c0, c0 + 32) of row `row` (one lane = one row):
// per column, the 32 lanes of a warp write 32 consecutive rows of xt (64 coalesced bytes);
// the row-major f32 and bf16 outputs (and the f32 input of the backward mode) move as 16-byte
// vectors when the columns are full and aligned.
__device__ __forceinline__ void epilogue_fused(const GemmEpilogue& epi, const uint32_t* r,
                                               float* D, int ldd, int M, int N, int row,
                                               int c0) {
    if (row >= M) return;
    const bool full = c0 + 32 <= N && (N & 7) == 0 && (ldd & 3) == 0;
    float out[32], v[32];
    if (full) {
        if (epi.mode == GEMM_EPI_GELU_BACK) {
            const float4* z4 = reinterpret_cast<const float4*>(epi.zin + (size_t)row * N + c0);
#pragma unroll
            for (int q = 0; q < 32; q += 4) {
                const float4 z = z4[q / 4];
                const float zz[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    out[q + u] = __uint_as_float(r[q + u]) * gelu_tanh_grad(zz[u]);
                    v[q + u] = out[q + u];
                }
            }
        } else {
            const float4* b4 = reinterpret_cast<const float4*>(epi.bias + c0);
#pragma unroll
            for (int q = 0; q < 32; q += 4) {
                const float4 b = b4[q / 4];
                const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    out[q + u] = __uint_as_float(r[q + u]) + bb[u];
                    v[q + u] = epi.mode == GEMM_EPI_BIAS_GELU ? gelu_tanh(out[q + u]) : out[q + u];
                }
            }
        }
        float4* d4 = reinterpret_cast<float4*>(D + (size_t)row * ldd + c0);
#pragma unroll
        for (int q = 0; q < 32; q += 4)
            d4[q / 4] = make_float4(out[q], out[q + 1], out[q + 2], out[q + 3]);
        if (epi.x) {
            uint4* x4 = reinterpret_cast<uint4*>(epi.x + (size_t)row * N + c0);
#pragma unroll
            for (int q = 0; q < 32; q += 8) {
                __nv_bfloat162 h[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) h[u] = __floats2bfloat162_rn(v[q + 2 * u], v[q + 2 * u + 1]);
                uint4 w;
                w.x = *reinterpret_cast<uint32_t*>(&h[0]);
                w.y = *reinterpret_cast<uint32_t*>(&h[1]);
                w.z = *reinterpret_cast<uint32_t*>(&h[2]);
                w.w = *reinterpret_cast<uint32_t*>(&h[3]);
                x4[q / 8] = w;
            }
        }
        if (epi.xt) {
#pragma unroll
            for (int q = 0; q < 32; ++q)
                epi.xt[(size_t)(c0 + q) * M + row] = __float2bfloat16(v[q]);
        }
        return;
    }
    for (int q = 0; q < 32 && c0 + q < N; ++q) {
        const int n = c0 + q;
        const float a = __uint_as_float(r[q]);
        float o, x;
        if (epi.mode == GEMM_EPI_GELU_BACK) {
            o = a * gelu_tanh_grad(epi.zin[(size_t)row * N + n]);
            x = o;
        } else {
            o = a + epi.bias[n];
            x = epi.mode == GEMM_EPI_BIAS_GELU ? gelu_tanh(o) : o;
        }
        D[(size_t)row * ldd + n] = o;
        if (epi.x) epi.x[(size_t)row * N + n] = __float2bfloat16(x);
        if (epi.xt) epi.xt[(size_t)n * M + row] = __float2bfloat16(x);
    }
}

__global__ void __launch_bounds__(128, 1)
    k_gemm_bf16_tn(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                   float* __restrict__ D, int M, int N, int K, int ldd, int splits,
                   size_t split_stride, uint32_t* err, const GemmEpilogue epi) {
    extern __shared__ __align__(1024) uint8_t gb_smem_raw[];
    __shared__ __align__(8) uint64_t full[GB_STAGES], empty[GB_STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    uint8_t* smem = (uint8_t*)(((uintptr_t)gb_smem_raw + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
    // split-K: blockIdx.z takes k-blocks [kb0, kb1) and writes its own f32 partial of D
    const int nk_all = K / GB_K, z = (int)blockIdx.z;
    const int kb0 = (int)((long long)nk_all * z / splits);
    const int nk = (int)((long long)nk_all * (z + 1) / splits) - kb0;
    D += (size_t)z * split_stride;

    if (tid == 0) {
        for (int s = 0; s < GB_STAGES; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[s])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty[s])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        abort_flag = 0;
    }
    if (warp == 1) {  // 128 f32 columns x 128 lanes of tensor memory for the accumulator
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base)),
                     "r"(GB_N));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {  // TMA producer
        const uint64_t pa = (uint64_t)&tmA, pb = (uint64_t)&tmB;
        for (int kb = 0; kb < nk; ++kb) {
            const int s = kb % GB_STAGES;
            if (kb >= GB_STAGES &&
                !mbar_wait(&empty[s], ((kb / GB_STAGES) - 1) & 1, err, 1u)) {
                abort_flag = 1;
                break;
            }
            if (*(volatile int*)&abort_flag) break;
            uint8_t* sa = smem + s * GB_STAGE_BYTES;
            uint8_t* sb = sa + GB_TILE_BYTES;
            const uint32_t fb = smem_u32(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(fb),
                         "r"(GB_STAGE_BYTES)
                         : "memory");
            const int kx = (kb0 + kb) * GB_K;  // innermost coordinate: a multiple of 64 bf16
                                               // = 128 B
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(sa)),
                "l"(pa), "r"(kx), "r"(m0), "r"(fb)
                : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(sb)),
                "l"(pb), "r"(kx), "r"(n0), "r"(fb)
                : "memory");
        }
    } else if (warp == 1 && lane == 0) {  // MMA issuer
        constexpr uint32_t idesc = mma_idesc_bf16(GB_M, GB_N);
        int kb = 0;
        for (; kb < nk; ++kb) {
            const int s = kb % GB_STAGES;
            if (!mbar_wait(&full[s], (kb / GB_STAGES) & 1, err, 2u)) {
                abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(smem + s * GB_STAGE_BYTES);
            const uint32_t sb = sa + GB_TILE_BYTES;
#pragma unroll
            for (int k = 0; k < GB_K / 16; ++k) {  // 16 bf16 = 32 B along K per MMA
                const uint64_t ad = sw128_desc(sa + 32 * k), bd = sw128_desc(sb + 32 * k);
                const uint32_t acc = (kb | k) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                    : "memory");
            }
            asm volatile(
                "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                    smem_u32(&empty[s]))
                : "memory");
        }
        // accumulator complete (or abandoned): the epilogue waits on `done`
        asm volatile(
            "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                smem_u32(&done))
            : "memory");
    }
    __syncwarp();
    // epilogue: warp w reads accumulator lanes 32w..32w+31 (rows of the tile)
    const bool ok = mbar_wait(&done, 0, err, 4u);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int row = m0 + warp * 32 + lane;
    if (ok && !*(volatile int*)&abort_flag) {
#pragma unroll 1
        for (int c = 0; c < GB_N; c += 32) {
            uint32_t r[32];
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, "
                "%9, %10, %11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, "
                "%25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                  "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                  "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
                  "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                  "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                  "=r"(r[30]), "=r"(r[31])
                : "r"(ta));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (epi.mode != GEMM_EPI_STORE) {
                epilogue_fused(epi, r, D, ldd, M, N, row, n0 + c);
                continue;
            }
            if (row < M) {
                float* dst = D + (size_t)row * ldd + n0 + c;
                if (n0 + c + 32 <= N) {
#pragma unroll
                    for (int q = 0; q < 32; q += 4)
                        *reinterpret_cast<float4*>(dst + q) =
                            make_float4(__uint_as_float(r[q]), __uint_as_float(r[q + 1]),
                                        __uint_as_float(r[q + 2]), __uint_as_float(r[q + 3]));
                } else {
                    for (int q = 0; q < 32 && n0 + c + q < N; ++q) dst[q] = __uint_as_float(r[q]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                     "r"(GB_N));
    }
}

// ------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------
static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// 2-D bf16 row-major [rows x cols] tensor map with 128 x 64 boxes and 128-byte swizzle.
static int make_map(CUtensorMap* m, const void* base, uint64_t rows, uint64_t cols) {
    auto enc = tensor_map_encoder();
    if (!enc) {
        set_error("cuTensorMapEncodeTiled unavailable");
        return NDT_ERR_DEVICE;
    }
    const cuuint64_t dims[2] = {cols, rows};
    const cuuint64_t strides[1] = {cols * 2};
    const cuuint32_t box[2] = {GB_K, GB_M};
    const cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    return 0;
}

// splits > 1: split-K, partial products of k-range z at D + z * M * ldd (the caller sums)
int gemm_bf16_tn(const void* A, const void* B, float* D, int M, int N, int K, int ldd,
                 uint32_t* d_err, cudaStream_t s, int splits, const GemmEpilogue* epi) {
    if (M <= 0 || N <= 0 || K <= 0 || K % GB_K || ldd < N || ((uintptr_t)A & 15) ||
        ((uintptr_t)B & 15) || ((uintptr_t)D & 15) || (ldd & 3) || splits < 1 ||
        splits > K / GB_K || splits > 65535) {
        set_error("gemm: K must be a multiple of 64, operands 16-byte aligned, ldd >= N, "
                  "1 <= splits <= K / 64");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    GemmEpilogue e{};
    if (epi) e = *epi;
    if (e.mode != GEMM_EPI_STORE &&
        (splits != 1 || ldd != N || ((uintptr_t)e.x & 15) ||
         (e.mode == GEMM_EPI_GELU_BACK ? !e.zin : !e.bias))) {
        set_error("gemm: a fused epilogue needs splits = 1, ldd = N, its bias (or input) and "
                  "16-byte aligned outputs");
        return NDT_ERR_INVALID_ARGUMENT;
    }
    CUtensorMap ta, tb;
    int rc;
    if ((rc = make_map(&ta, A, (uint64_t)M, (uint64_t)K)) ||
        (rc = make_map(&tb, B, (uint64_t)N, (uint64_t)K)))
        return rc;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_gemm_bf16_tn, cudaFuncAttributeMaxDynamicSharedMemorySize, GB_SMEM);
        attr = true;
    }
    dim3 grid((unsigned)((N + GB_N - 1) / GB_N), (unsigned)((M + GB_M - 1) / GB_M),
              (unsigned)splits);
    k_gemm_bf16_tn<<<grid, 128, GB_SMEM, s>>>(ta, tb, D, M, N, K, ldd, splits,
                                              (size_t)M * ldd, d_err, e);
    return cuda_fail(cudaGetLastError(), "gemm launch");
}

// error word of the standalone entry point (device global, no allocation)
static __device__ uint32_t g_gemm_err;

}  // namespace ndtgb

extern "C" int ndt_gemm_bf16(const void* d_a, const void* d_b, float* d_d, int32_t m, int32_t n,
                             int32_t k, int32_t splits, void* stream) {
    using namespace ndtgb;
    uint32_t* err = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void**)&err, g_gemm_err);
    if (e != cudaSuccess) return cuda_fail(e, "gemm error word");
    cudaStream_t s = (cudaStream_t)stream;
    cudaMemsetAsync(err, 0, 4, s);
    int rc = gemm_bf16_tn(d_a, d_b, d_d, m, n, k, n, err, s, splits, nullptr);
    if (rc) return rc;
    uint32_t h = 0;
    cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, s);
    if ((rc = cuda_fail(cudaStreamSynchronize(s), "gemm"))) return rc;
    if (h) {
        set_error("gemm: a pipeline wait timed out (code " + std::to_string(h) + ")");
        return NDT_ERR_DEVICE;
    }
    return NDT_OK;
}
