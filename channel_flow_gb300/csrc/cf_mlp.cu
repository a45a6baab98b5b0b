// Learned initial guess of the pseudo-time iterations: a per-cell MLP
// (270 -> 128 -> 128 -> 5, SiLU) with BF16 weights and FP32 accumulation on
// the 5th-generation tensor cores, and the kernels that train it.
//
// GEMM (k_gemm_tn): C[M x N] = A[M x K] B[N x K]^T with A and B BF16,
// K-major.  One CTA computes a 128 x BN tile: warp 0 streams 128 x 64 and
// BN x 64 K-slabs with TMA (128-byte swizzle) through a 4-stage mbarrier
// ring, warp 1 issues tcgen05.mma (kind::f16, M = 128, K = 16 per
// instruction) into a TMEM accumulator and frees each stage with
// tcgen05.commit, and all four warps read the accumulator back with
// tcgen05.ld for the fused epilogue (bias, SiLU, BF16 or FP32 output).
// Every mbarrier wait is bounded; a wait that runs out sets an error word
// and the CTA still releases its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/channel_flow_gb300.h"

namespace cf_mlp {

constexpr int BM = 128, BK = 64, STAGES = 4;
constexpr unsigned long long WAIT_NS = 2000000000ull;   // a wait gives up after two seconds

enum { EPI_F32 = 0, EPI_BIAS_SILU_BF16 = 1, EPI_BIAS_F32 = 2 };

struct gemm_epi {
    int kind;
    const float *bias;       // [N] or null
    float *outf;             // fp32 output [M x ldo] (EPI_F32, EPI_BIAS_F32)
    __nv_bfloat16 *outb;     // bf16 output [M x ldo] (EPI_BIAS_SILU_BF16)
    float *zout;             // optional fp32 pre-activation [M x ldo] (EPI_BIAS_SILU_BF16)
    int ldo;
};

__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase)
{
    const unsigned long long t0 = gtimer();
    for (unsigned it = 0;; it++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(bar), "r"(phase) : "memory");
        if (done) return true;
        if ((it & 255u) == 255u && gtimer() - t0 > WAIT_NS) return false;
    }
}

// shared-memory matrix descriptor of a K-major tile stored with the
// 128-byte swizzle (rows of 128 bytes, 8-row atoms of 1024 bytes)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);       // start address
    d |= (uint64_t)1 << 16;                         // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;               // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                         // descriptor version
    d |= (uint64_t)2 << 61;                         // 128-byte swizzle
    return d;
}

// instruction descriptor: kind::f16, A = B = BF16, D = FP32, both K-major
__host__ __device__ constexpr uint32_t mma_idesc(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

template <int BN>
struct tmem_cols {
    static constexpr uint32_t v = BN <= 32 ? 32 : BN <= 64 ? 64 : BN <= 128 ? 128 : 256;
};

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }

template <int BN>
__global__ void __launch_bounds__(128, 1) k_gemm_tn(const __grid_constant__ CUtensorMap tA,
                                                    const __grid_constant__ CUtensorMap tB, int M, int N, int K,
                                                    gemm_epi e, int *err)
{
    extern __shared__ unsigned char dsm[];
    __shared__ __align__(8) uint64_t full[STAGES], empty[STAGES], accb;
    __shared__ uint32_t tmem_base;
    constexpr uint32_t A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2, STAGE = A_BYTES + B_BYTES;
    constexpr uint32_t NCOL = tmem_cols<BN>::v;
    constexpr uint32_t IDESC = mma_idesc(BM, BN);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int KT = K / BK;
    unsigned char *base = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(dsm) + 1023) &
                                                            ~static_cast<uintptr_t>(1023));
    const uint32_t sbase = saddr(base);
    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; s++) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&full[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&empty[s])) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(saddr(&accb)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(saddr(&tmem_base)), "r"(NCOL) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {
        // TMA producer
        for (int kt = 0; kt < KT; kt++) {
            const int s = kt % STAGES;
            const uint32_t ph = (uint32_t)(kt / STAGES) & 1u;
            if (kt >= STAGES && !mbar_wait(saddr(&empty[s]), ph ^ 1u)) {
                atomicOr(err, 1);
                break;
            }
            const uint32_t fb = saddr(&full[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(fb), "r"(STAGE) : "memory");
            const uint32_t da = sbase + s * STAGE, db = da + A_BYTES;
            asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2, %3}], [%4];"
                         :: "r"(da), "l"(reinterpret_cast<uint64_t>(&tA)), "r"(kt * BK), "r"(m0), "r"(fb)
                         : "memory");
            asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
                         " [%0], [%1, {%2, %3}], [%4];"
                         :: "r"(db), "l"(reinterpret_cast<uint64_t>(&tB)), "r"(kt * BK), "r"(n0), "r"(fb)
                         : "memory");
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        bool ok = true;
        for (int kt = 0; kt < KT; kt++) {
            const int s = kt % STAGES;
            const uint32_t ph = (uint32_t)(kt / STAGES) & 1u;
            if (!mbar_wait(saddr(&full[s]), ph)) {
                atomicOr(err, 2);
                ok = false;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t da = sbase + s * STAGE, db = da + A_BYTES;
#pragma unroll
            for (int kk = 0; kk < BK / 16; kk++) {
                const uint64_t ad = sw128_desc(da + kk * 32), bd = sw128_desc(db + kk * 32);
                const uint32_t acc = (kt | kk) != 0;
                asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                             " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                             :: "r"(tmem), "l"(ad), "l"(bd), "r"(IDESC), "r"(acc) : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(saddr(&empty[s])) : "memory");
        }
        if (ok)
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(saddr(&accb)) : "memory");
    }
    __syncwarp();
    // epilogue: warp w owns accumulator rows 32w..32w+31 (TMEM lanes)
    const bool have = mbar_wait(saddr(&accb), 0);
    if (!have && threadIdx.x == 0) atomicOr(err, 4);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (have) {
        const int row = m0 + warp * 32 + lane;
#pragma unroll 1
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t r[16];
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
                         "%11, %12, %13, %14, %15}, [%16];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
                           "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                         : "r"(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < M) {
                const int col = n0 + c0;
                float v[16];
#pragma unroll
                for (int t = 0; t < 16; t++) v[t] = __uint_as_float(r[t]);
                if (e.kind != EPI_F32 && e.bias)
#pragma unroll
                    for (int t = 0; t < 16; t++) v[t] += e.bias[col + t];
                if (e.kind == EPI_BIAS_SILU_BF16) {
                    if (e.zout) {
                        float4 *z = reinterpret_cast<float4 *>(e.zout + (size_t)row * e.ldo + col);
#pragma unroll
                        for (int t = 0; t < 4; t++) z[t] = make_float4(v[4 * t], v[4 * t + 1], v[4 * t + 2], v[4 * t + 3]);
                    }
                    __align__(16) __nv_bfloat16 h[16];
#pragma unroll
                    for (int t = 0; t < 16; t++) h[t] = __float2bfloat16(silu(v[t]));
                    uint4 *o = reinterpret_cast<uint4 *>(e.outb + (size_t)row * e.ldo + col);
                    o[0] = *reinterpret_cast<const uint4 *>(&h[0]);
                    o[1] = *reinterpret_cast<const uint4 *>(&h[8]);
                } else {
                    float4 *o = reinterpret_cast<float4 *>(e.outf + (size_t)row * e.ldo + col);
#pragma unroll
                    for (int t = 0; t < 4; t++) o[t] = make_float4(v[4 * t], v[4 * t + 1], v[4 * t + 2], v[4 * t + 3]);
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(NCOL) : "memory");
}

// ---------------------------------------------------------------------------
// host: tensor maps through the driver entry point (no libcuda link)

typedef CUresult (*encode_fn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static encode_fn get_encode()
{
    static encode_fn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<encode_fn>(p);
    });
    return fn;
}

// row-major [rows x cols] bf16 matrix, box of box_rows x 64 columns, 128-byte swizzle
static bool make_map(CUtensorMap *m, const void *ptr, int rows, int cols, int box_rows)
{
    encode_fn enc = get_encode();
    if (!enc) return false;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
static cudaError_t launch_gemm(const CUtensorMap &ta, const CUtensorMap &tb, int M, int N, int K, const gemm_epi &e,
                               int *err, cudaStream_t s)
{
    constexpr size_t smem = (size_t)STAGES * (BM * BK * 2 + BN * BK * 2) + 1024;
    cudaError_t r = cudaFuncSetAttribute(k_gemm_tn<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (r != cudaSuccess) return r;
    dim3 g((unsigned)(M / BM), (unsigned)(N / BN));
    k_gemm_tn<BN><<<g, 128, smem, s>>>(ta, tb, M, N, K, e, err);
    return cudaGetLastError();
}

}  // namespace cf_mlp

using namespace cf_mlp;

extern "C" {

// C = A B^T (see channel_flow_gb300.h)
int cf_gemm_bf16(void *stream, const void *A, const void *B, int M, int N, int K, int epilogue, const float *bias,
                 void *out, float *zout, int ldo, int *err_dev)
{
    if (!A || !B || !out || !err_dev) return CF_ERR_ARG;
    if (M <= 0 || N <= 0 || K <= 0 || M % BM || K % BK || N % 16 || ldo < N || ldo % 8) return CF_ERR_ARG;
    if (epilogue < EPI_F32 || epilogue > EPI_BIAS_F32) return CF_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15) return CF_ERR_ARG;
    int bn = 0;
    for (int c : {256, 128, 64, 32, 16})
        if (N % c == 0) { bn = c; break; }
    CUtensorMap ta, tb;
    if (!make_map(&ta, A, M, K, BM) || !make_map(&tb, B, N, K, bn)) return CF_ERR_CUDA;
    gemm_epi e{epilogue, bias, nullptr, nullptr, zout, ldo};
    if (epilogue == EPI_BIAS_SILU_BF16) e.outb = static_cast<__nv_bfloat16 *>(out);
    else e.outf = static_cast<float *>(out);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaError_t r;
    switch (bn) {
    case 256: r = launch_gemm<256>(ta, tb, M, N, K, e, err_dev, s); break;
    case 128: r = launch_gemm<128>(ta, tb, M, N, K, e, err_dev, s); break;
    case 64: r = launch_gemm<64>(ta, tb, M, N, K, e, err_dev, s); break;
    case 32: r = launch_gemm<32>(ta, tb, M, N, K, e, err_dev, s); break;
    default: r = launch_gemm<16>(ta, tb, M, N, K, e, err_dev, s); break;
    }
    return r == cudaSuccess ? CF_OK : CF_ERR_CUDA;
}

}  // extern "C"
